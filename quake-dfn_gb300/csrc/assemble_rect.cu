// Rectangular-patch stiffness kernel (Okada DC3D), one thread per
// (receiver, source) pair, FP64.  Follows StiffnessMatrix_ByParts_Calculation_Rec
// (scripts/Functions_BuildInputFile.jl:386-512).
#include <cuda_runtime.h>

#include "assemble_kernels.h"
#include "qdfn_internal.h"
#include "okada.cuh"

namespace qdfn {
namespace {

__global__ void __launch_bounds__(kAsmThreads)
k_assemble_rect(int64_t n_src, const double* __restrict__ src, int64_t n_recv,
                const double* __restrict__ recv, double G, double nu, double* __restrict__ Ks,
                double* __restrict__ Kn, int64_t ld, int layout) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_recv) return;
    const double lam = 2 * G * nu / (1 - 2 * nu);
    const double alpha = (lam + G) / (lam + 2 * G);
    const double* rr = recv + r * 8;
    const double rcx = rr[0], rcy = rr[1], rcz = rr[2], rstr = rr[5], rdip = rr[6], rrake = rr[7];
    const double cdp = cosd_d(-rdip), sdp = sind_d(-rdip);
    const double crk = cosd_d(rrake), srk = sind_d(rrake);
    for (int64_t s = blockIdx.y; s < n_src; s += gridDim.y) {
        const double* ss = src + s * 8;
        const double scx = ss[0], scy = ss[1], scz = ss[2], sls = ss[3], sld = ss[4],
                     sstr = ss[5], sdip = ss[6], srake = ss[7];
        const double DISL1 = cosd_d(srake), DISL2 = sind_d(srake), DISL3 = 0.0;
        const double AL = sls / 2, AW = sld / 2;
        const double cs = cosd_d(-sstr), sn = sind_d(-sstr);
        const double Xd = rcx - scx, Yd = rcy - scy;
        const double X = Xd * cs - Yd * sn;
        const double Y = Xd * sn + Yd * cs;
        const double Z = -rcz;
        const okada::C0 c0 = okada::dccon0(alpha, sdip);
        double U[9];
        okada::dc3d_gradients(c0, X, Y, Z, scz, AL, AL, AW, AW, DISL1, DISL2, DISL3, U);
        const double UXX = U[0], UYX = U[1], UZX = U[2], UXY = U[3], UYY = U[4], UZY = U[5],
                     UXZ = U[6], UYZ = U[7], UZZ = U[8];
        // Hooke's law in the source frame (:462-467)
        const double sxx = lam * (UXX + UYY + UZZ) + 2 * G * UXX;
        const double syy = lam * (UXX + UYY + UZZ) + 2 * G * UYY;
        const double szz = lam * (UXX + UYY + UZZ) + 2 * G * UZZ;
        const double sxy = (UXY + UYX) * G;
        const double sxz = (UXZ + UZX) * G;
        const double syz = (UYZ + UZY) * G;
        // R = R_dip * R_strike(-relative strike); sigma' = R sigma R^T (:480-492).
        // Only sigma'_13, sigma'_23, sigma'_33 are needed.
        const double rel = rstr - sstr;
        const double cr = cosd_d(-rel), sr = sind_d(-rel);
        // RS = [cr -sr 0; sr cr 0; 0 0 1], RD = [1 0 0; 0 cdp -sdp; 0 sdp cdp]
        const double R00 = 1 * cr + 0 * sr + 0 * 0, R01 = 1 * -sr + 0 * cr + 0 * 0, R02 = 1 * 0 + 0 * 0 + 0 * 1;
        const double R10 = 0 * cr + cdp * sr + -sdp * 0, R11 = 0 * -sr + cdp * cr + -sdp * 0,
                     R12 = 0 * 0 + cdp * 0 + -sdp * 1;
        const double R20 = 0 * cr + sdp * sr + cdp * 0, R21 = 0 * -sr + sdp * cr + cdp * 0,
                     R22 = 0 * 0 + sdp * 0 + cdp * 1;
        // M = R * S
        const double M00 = R00 * sxx + R01 * sxy + R02 * sxz, M01 = R00 * sxy + R01 * syy + R02 * syz,
                     M02 = R00 * sxz + R01 * syz + R02 * szz;
        const double M10 = R10 * sxx + R11 * sxy + R12 * sxz, M11 = R10 * sxy + R11 * syy + R12 * syz,
                     M12 = R10 * sxz + R11 * syz + R12 * szz;
        const double M20 = R20 * sxx + R21 * sxy + R22 * sxz, M21 = R20 * sxy + R21 * syy + R22 * syz,
                     M22 = R20 * sxz + R21 * syz + R22 * szz;
        // (M R^T)[i][2] = M[i][0]*R[2][0] + M[i][1]*R[2][1] + M[i][2]*R[2][2]
        const double S02 = M00 * R20 + M01 * R21 + M02 * R22;
        const double S12 = M10 * R20 + M11 * R21 + M12 * R22;
        const double S22 = M20 * R20 + M21 * R21 + M22 * R22;
        const double kn = -S22;
        const double ks = crk * S02 + srk * S12;
        const int64_t idx = layout == QDFN_LAYOUT_COL ? s * ld + r : r * ld + s;
        Kn[idx] = kn;
        Ks[idx] = ks;
    }
}

}  // namespace

void launch_assemble_rect(dim3 grid, cudaStream_t st, int64_t n_src, const double* src,
                          int64_t n_recv, const double* recv, double G, double nu, double* Ks,
                          double* Kn, int64_t ld, int layout) {
    k_assemble_rect<<<grid, kAsmThreads, 0, st>>>(n_src, src, n_recv, recv, G, nu, Ks, Kn, ld,
                                                 layout);
}

}  // namespace qdfn
