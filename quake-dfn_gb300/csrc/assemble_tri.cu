// Triangular-patch stiffness kernel (TDstressHS), one thread per
// (receiver, source) pair, FP64.  Follows StiffnessMatrix_ByParts_Calculation_Tri
// (scripts/Functions_BuildInputFile.jl:551-594).
#include <cuda_runtime.h>

#include "assemble_kernels.h"
#include "qdfn_internal.h"
#include "tdhs.cuh"

namespace qdfn {
namespace {

__global__ void __launch_bounds__(kAsmThreads)
k_assemble_tri(int64_t n_src, const double* __restrict__ P1, const double* __restrict__ P2,
               const double* __restrict__ P3, const double* __restrict__ rake, int64_t n_recv,
               const double* __restrict__ centre, const double* __restrict__ nhat,
               const double* __restrict__ shat, double G, double nu, double* __restrict__ Ks,
               double* __restrict__ Kn, int64_t ld, int layout) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_recv) return;
    const double lam = 2 * G * nu / (1 - 2 * nu);
    const double X = centre[r * 3], Y = centre[r * 3 + 1], Z = centre[r * 3 + 2];
    const double n0 = nhat[r * 3], n1 = nhat[r * 3 + 1], n2 = nhat[r * 3 + 2];
    const double v0 = shat[r * 3], v1 = shat[r * 3 + 1], v2 = shat[r * 3 + 2];
    for (int64_t s = blockIdx.y; s < n_src; s += gridDim.y) {
        const double Ss = -cosd_d(rake[s]), Ds = sind_d(rake[s]), Ts = 0.0;
        double st[6];
        tdhs::tdstress_hs(X, Y, Z, P1 + s * 3, P2 + s * 3, P3 + s * 3, Ss, Ds, Ts, G, lam, st);
        const double t0 = st[0] * n0 + st[3] * n1 + st[4] * n2;
        const double t1 = st[3] * n0 + st[1] * n1 + st[5] * n2;
        const double t2 = st[4] * n0 + st[5] * n1 + st[2] * n2;
        const int64_t idx = layout == QDFN_LAYOUT_COL ? s * ld + r : r * ld + s;
        Kn[idx] = t0 * n0 + t1 * n1 + t2 * n2;
        Ks[idx] = t0 * v0 + t1 * v1 + t2 * v2;
    }
}

// One thread per (receiver, source) pair of an index list: the entries that
// adaptive cross approximation asks for (rows and columns of admissible
// blocks) or any gathered set.  Same arithmetic as k_assemble_tri.
__global__ void __launch_bounds__(kAsmThreads)
k_assemble_tri_pairs(int64_t npairs, const int64_t* __restrict__ ridx, const int64_t* __restrict__ sidx,
                     const double* __restrict__ P1, const double* __restrict__ P2, const double* __restrict__ P3,
                     const double* __restrict__ rake, const double* __restrict__ centre,
                     const double* __restrict__ nhat, const double* __restrict__ shat, double G, double nu,
                     double* __restrict__ Ks, double* __restrict__ Kn) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npairs) return;
    const int64_t r = ridx[k], s = sidx[k];
    const double lam = 2 * G * nu / (1 - 2 * nu);
    const double n0 = nhat[r * 3], n1 = nhat[r * 3 + 1], n2 = nhat[r * 3 + 2];
    const double v0 = shat[r * 3], v1 = shat[r * 3 + 1], v2 = shat[r * 3 + 2];
    const double Ss = -cosd_d(rake[s]), Ds = sind_d(rake[s]), Ts = 0.0;
    double st[6];
    tdhs::tdstress_hs(centre[r * 3], centre[r * 3 + 1], centre[r * 3 + 2], P1 + s * 3, P2 + s * 3, P3 + s * 3, Ss,
                      Ds, Ts, G, lam, st);
    const double t0 = st[0] * n0 + st[3] * n1 + st[4] * n2;
    const double t1 = st[3] * n0 + st[1] * n1 + st[5] * n2;
    const double t2 = st[4] * n0 + st[5] * n1 + st[2] * n2;
    Kn[k] = t0 * n0 + t1 * n1 + t2 * n2;
    Ks[k] = t0 * v0 + t1 * v1 + t2 * v2;
}

}  // namespace

void launch_assemble_tri_pairs(cudaStream_t st, int64_t npairs, const int64_t* ridx, const int64_t* sidx,
                               const double* P1, const double* P2, const double* P3, const double* rake,
                               const double* centre, const double* nhat, const double* shat, double G, double nu,
                               double* Ks, double* Kn) {
    const int64_t nb = (npairs + kAsmThreads - 1) / kAsmThreads;
    k_assemble_tri_pairs<<<(unsigned)nb, kAsmThreads, 0, st>>>(npairs, ridx, sidx, P1, P2, P3, rake, centre, nhat,
                                                             shat, G, nu, Ks, Kn);
}

void launch_assemble_tri(dim3 grid, cudaStream_t st, int64_t n_src, const double* P1,
                         const double* P2, const double* P3, const double* rake, int64_t n_recv,
                         const double* centre, const double* nhat, const double* shat, double G,
                         double nu, double* Ks, double* Kn, int64_t ld, int layout) {
    k_assemble_tri<<<grid, kAsmThreads, 0, st>>>(n_src, P1, P2, P3, rake, n_recv, centre, nhat,
                                                shat, G, nu, Ks, Kn, ld, layout);
}

}  // namespace qdfn
