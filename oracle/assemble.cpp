// Oracle: stiffness-matrix assembly drivers, restated from
//   scripts/Functions_BuildInputFile.jl
//     StiffnessMatrix_ByParts_Calculation_Rec   :386-512  (Okada rectangles)
//     StiffnessMatrix_ByParts_Calculation_Tri   :551-594  (TD triangles)
// K[receiver, source]: normal = -sigma'_33 and shear = cos(rake_r) sigma'_13 +
// sin(rake_r) sigma'_23 in the receiver frame (rectangles, :496-497); traction
// t = sigma n on the receiver normal and slip vectors (triangles, :575-581).
// The reference splits the matrix into ~2000x2000 parts (:516-548, :599-638)
// only to bound memory; every entry depends on its own (receiver, source)
// pair alone, so the part split does not change any value.
//
// TEST INFRASTRUCTURE ONLY (CPU oracle); not part of the shipped library.
#include <cmath>
#include "jlmath.h"
#include "oracle.h"

using oracle::cosd;
using oracle::sind;

namespace {
// C = A * B for 3x3 row-major, each entry summed left to right
void mm3(const double A[9], const double B[9], double C[9]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            C[i * 3 + j] = A[i * 3 + 0] * B[0 * 3 + j] + A[i * 3 + 1] * B[1 * 3 + j] +
                           A[i * 3 + 2] * B[2 * 3 + j];
}
}  // namespace

extern "C" void oracle_assemble_rect(int64_t n_src, const double* s_cx, const double* s_cy,
                                     const double* s_cz, const double* s_ls,
                                     const double* s_ld, const double* s_str,
                                     const double* s_dip, const double* s_rake, int64_t n_recv,
                                     const double* r_cx, const double* r_cy, const double* r_cz,
                                     const double* r_str, const double* r_dip,
                                     const double* r_rake, double G, double nu, double* Ks,
                                     double* Kn, int nthreads) {
    const double lam = 2 * G * nu / (1 - 2 * nu);
    const double alpha = (lam + G) / (lam + 2 * G);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t s = 0; s < n_src; ++s) {
        const double DISL1 = cosd(s_rake[s]);
        const double DISL2 = sind(s_rake[s]);
        const double DISL3 = 0;
        const double DEPTH = s_cz[s];
        const double AL = s_ls[s] / 2, AW = s_ld[s] / 2;
        const double cs = cosd(-s_str[s]), ss = sind(-s_str[s]);
        for (int64_t r = 0; r < n_recv; ++r) {
            double Xd = r_cx[r] - s_cx[s];
            double Yd = r_cy[r] - s_cy[s];
            double X = Xd * cs - Yd * ss;
            double Y = Xd * ss + Yd * cs;
            double Z = -r_cz[r];
            double U[12];
            oracle_okada_dc3d(alpha, X, Y, Z, DEPTH, s_dip[s], AL, AL, AW, AW, DISL1, DISL2,
                              DISL3, U, nullptr);
            const double UXX = U[3], UYX = U[4], UZX = U[5], UXY = U[6], UYY = U[7],
                         UZY = U[8], UXZ = U[9], UYZ = U[10], UZZ = U[11];
            double sxx = lam * (UXX + UYY + UZZ) + 2 * G * UXX;
            double syy = lam * (UXX + UYY + UZZ) + 2 * G * UYY;
            double szz = lam * (UXX + UYY + UZZ) + 2 * G * UZZ;
            double sxy = (UXY + UYX) * G;
            double sxz = (UXZ + UZX) * G;
            double syz = (UYZ + UZY) * G;
            double S[9] = {sxx, sxy, sxz, sxy, syy, syz, sxz, syz, szz};
            double rel = r_str[r] - s_str[s];
            double cr = cosd(-rel), sr = sind(-rel);
            double RS[9] = {cr, -sr, 0, sr, cr, 0, 0, 0, 1};
            double cdp = cosd(-r_dip[r]), sdp = sind(-r_dip[r]);
            double RD[9] = {1, 0, 0, 0, cdp, -sdp, 0, sdp, cdp};
            double R[9], RSm[9], Rt[9], SR[9];
            mm3(RD, RS, R);
            mm3(R, S, RSm);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) Rt[i * 3 + j] = R[j * 3 + i];
            mm3(RSm, Rt, SR);
            Kn[r * n_src + s] = -SR[2 * 3 + 2];
            Ks[r * n_src + s] = cosd(r_rake[r]) * SR[0 * 3 + 2] + sind(r_rake[r]) * SR[1 * 3 + 2];
        }
    }
}

extern "C" int oracle_assemble_tri(int64_t n_src, const double* P1, const double* P2,
                                   const double* P3, const double* rake, int64_t n_recv,
                                   const double* centre, const double* nhat,
                                   const double* shat, double G, double nu, double* Ks,
                                   double* Kn, int nthreads) {
    const double lam = 2 * G * nu / (1 - 2 * nu);
    for (int64_t r = 0; r < n_recv; ++r)
        if (centre[r * 3 + 2] > 0) return -1;  // TDstressHS :99-101
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads > 0 ? nthreads : 1) reduction(| : bad)
    for (int64_t s = 0; s < n_src; ++s) {
        const double Ss = -cosd(rake[s]);
        const double Ds = sind(rake[s]);
        const double Ts = 0.0;
        for (int64_t r = 0; r < n_recv; ++r) {
            double st[6], sn[6];
            int rc = oracle_tdstress_hs(centre[r * 3], centre[r * 3 + 1], centre[r * 3 + 2],
                                        P1 + s * 3, P2 + s * 3, P3 + s * 3, Ss, Ds, Ts, G,
                                        lam, st, sn);
            if (rc) { bad = 1; continue; }
            // [Sxx Sxy Sxz; Sxy Syy Syz; Sxz Syz Szz] * n
            const double* n = nhat + r * 3;
            const double* sv = shat + r * 3;
            double t0 = st[0] * n[0] + st[3] * n[1] + st[4] * n[2];
            double t1 = st[3] * n[0] + st[1] * n[1] + st[5] * n[2];
            double t2 = st[4] * n[0] + st[5] * n[1] + st[2] * n[2];
            Kn[r * n_src + s] = t0 * n[0] + t1 * n[1] + t2 * n[2];
            Ks[r * n_src + s] = t0 * sv[0] + t1 * sv[1] + t2 * sv[2];
        }
    }
    return bad ? -1 : 0;
}
