// Device Okada (1992) DC3D: displacement GRADIENTS of a finite rectangular
// dislocation in a half-space, one receiver per thread.
//
// Follows scripts/Functions_OKADA3D.jl (DCCON0_V :12, DCCON2_V :51, UA_V :199,
// UB_V :266, UC_V :378, Okada_DC3D_Vector :464) with its exact semantics:
// DCCON2 zeroes |XI|,|ET|,|Q| < 1e-6 on its own copies only (UA/UB/UC get the
// caller's values), masks are applied by IEEE multiplication (a masked branch
// that is Inf/NaN still yields NaN), UB's atan NaN -> 0 and CD==0 -> 1e-12
// substitution, and DCCON2 supplies the Y and D that UA/UB/UC see.
//
// Only the nine gradient components (UXX..UZZ) are formed: the stiffness needs
// stresses only, and each of the twelve output components is accumulated
// independently in the reference, so dropping UX/UY/UZ changes no value.
#pragma once
#include "qdfn_internal.h"

namespace qdfn {
namespace okada {

struct C0 { double ALP1, ALP2, ALP3, ALP4, ALP5, SD, CD, SDSD, CDCD, SDCD; };

__device__ __forceinline__ C0 dccon0(double ALPHA, double DIP) {
    C0 c;
    c.ALP1 = (1.0 - ALPHA) / 2.0;
    c.ALP2 = ALPHA / 2.0;
    c.ALP3 = (1.0 - ALPHA) / ALPHA;
    c.ALP4 = 1.0 - ALPHA;
    c.ALP5 = ALPHA;
    const double P18 = 6.283185307179586 / 360.0;
    double SD = sin(DIP * P18), CD = cos(DIP * P18);
    double c1 = fabs(CD) < 1.0e-6, c2 = fabs(CD) >= 1.0e-6;
    double s1 = SD > 0.0, s2 = SD == 0.0, s3 = SD < 0.0;
    CD = 0.0 * c1 + CD * c2;
    SD = c1 * (1.0 * s1 + SD * s2 + (-1.0) * 1.0 * s3) + c2 * SD;
    c.SD = SD; c.CD = CD; c.SDSD = SD * SD; c.CDCD = CD * CD; c.SDCD = SD * CD;
    return c;
}

struct C2 {
    double XI2, ET2, Q2, R2, R, R3, R5, Y, D, X11, X32, Y11, Y32, EY, EZ, FY, FZ, GY, GZ, HY,
        HZ;
};

__device__ __forceinline__ void dccon2(double XI, double ET, double Q, double SD, double CD,
                                       C2& o) {
    const double EPS = 0.000001;
    XI = 0.0 * (fabs(XI) < EPS) + XI * (fabs(XI) >= EPS);
    ET = 0.0 * (fabs(ET) < EPS) + ET * (fabs(ET) >= EPS);
    Q = 0.0 * (fabs(Q) < EPS) + Q * (fabs(Q) >= EPS);
    o.XI2 = XI * XI; o.ET2 = ET * ET; o.Q2 = Q * Q;
    o.R2 = o.XI2 + o.ET2 + o.Q2;
    const double R = sqrt(o.R2);
    o.R = R; o.R3 = R * o.R2; o.R5 = o.R3 * o.R2;
    o.Y = ET * CD + Q * SD;
    o.D = ET * SD - Q * CD;
    // TT, ALX and ALE (atan/log terms) feed only the displacement rows and are
    // not formed.
    if ((XI < 0.0) && (Q == 0.0) && (ET == 0.0)) {
        o.X11 = 0.0; o.X32 = 0.0;
    } else {
        double RXI = R + XI;
        o.X11 = (1.0 / (R * RXI)) * 1.0;
        o.X32 = ((R + RXI) * o.X11 * o.X11 / R) * 1.0;
    }
    if ((ET < 0.0) && (Q == 0.0) && (XI == 0.0)) {
        o.Y11 = 0.0; o.Y32 = 0.0;
    } else {
        double RET = R + ET;
        o.Y11 = (1.0 / (R * RET)) * 1.0;
        o.Y32 = ((R + RET) * o.Y11 * o.Y11 / R) * 1.0;
    }
    o.EY = SD / R - o.Y * Q / o.R3;
    o.EZ = CD / R + o.D * Q / o.R3;
    o.FY = o.D / o.R3 + o.XI2 * o.Y32 * SD;
    o.FZ = o.Y / o.R3 + o.XI2 * o.Y32 * CD;
    o.GY = 2.0 * o.X11 * SD - o.Y * Q * o.X32;
    o.GZ = 2.0 * o.X11 * CD + o.D * Q * o.X32;
    o.HY = o.D * Q * o.X32 + XI * Q * o.Y32 * SD;
    o.HZ = o.Y * Q * o.X32 + XI * Q * o.Y32 * CD;
}

// U[k] += (DISL/2pi) * du[k] * (DISL != 0), for the 9 gradient components
__device__ __forceinline__ void acc9(double U[9], const double du[9], double DISL) {
    const double s = DISL / 6.283185307179586;
    const double c = (DISL != 0.0) ? 1.0 : 0.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) U[k] = U[k] + s * du[k] * c;
}

// UA_V gradient rows (components 4..12 of the reference, here 0..8)
__device__ void ua(double XI, double ET, double Q, double DISL1, double DISL2, double DISL3,
                   const C0& c0, const C2& g, double U[9]) {
    const double ALP1 = c0.ALP1, ALP2 = c0.ALP2, SD = c0.SD, CD = c0.CD;
    const double XY = XI * g.Y11, QY = Q * g.Y11;
#pragma unroll
    for (int k = 0; k < 9; ++k) U[k] = 0.0;
    double du[9];
    du[0] = -ALP1 * QY - ALP2 * g.XI2 * Q * g.Y32;
    du[1] = -ALP2 * XI * Q / g.R3;
    du[2] = ALP1 * XY + ALP2 * XI * g.Q2 * g.Y32;
    du[3] = ALP1 * XY * SD + ALP2 * XI * g.FY + g.D / 2.0 * g.X11;
    du[4] = ALP2 * g.EY;
    du[5] = ALP1 * (CD / g.R + QY * SD) - ALP2 * Q * g.FY;
    du[6] = ALP1 * XY * CD + ALP2 * XI * g.FZ + g.Y / 2.0 * g.X11;
    du[7] = ALP2 * g.EZ;
    du[8] = -ALP1 * (SD / g.R - QY * CD) - ALP2 * Q * g.FZ;
    acc9(U, du, DISL1);
    du[0] = -ALP2 * XI * Q / g.R3;
    du[1] = -QY / 2.0 - ALP2 * ET * Q / g.R3;
    du[2] = ALP1 / g.R + ALP2 * g.Q2 / g.R3;
    du[3] = ALP2 * g.EY;
    du[4] = ALP1 * g.D * g.X11 + XY / 2.0 * SD + ALP2 * ET * g.GY;
    du[5] = ALP1 * g.Y * g.X11 - ALP2 * Q * g.GY;
    du[6] = ALP2 * g.EZ;
    du[7] = ALP1 * g.Y * g.X11 + XY / 2.0 * CD + ALP2 * ET * g.GZ;
    du[8] = -ALP1 * g.D * g.X11 - ALP2 * Q * g.GZ;
    acc9(U, du, DISL2);
    du[0] = -ALP1 * XY + ALP2 * XI * g.Q2 * g.Y32;
    du[1] = -ALP1 / g.R + ALP2 * g.Q2 / g.R3;
    du[2] = -ALP1 * QY - ALP2 * Q * g.Q2 * g.Y32;
    du[3] = -ALP1 * (CD / g.R + QY * SD) - ALP2 * Q * g.FY;
    du[4] = -ALP1 * g.Y * g.X11 - ALP2 * Q * g.GY;
    du[5] = ALP1 * (g.D * g.X11 + XY * SD) + ALP2 * Q * g.HY;
    du[6] = ALP1 * (SD / g.R - QY * CD) - ALP2 * Q * g.FZ;
    du[7] = ALP1 * g.D * g.X11 - ALP2 * Q * g.GZ;
    du[8] = ALP1 * (g.Y * g.X11 + XY * CD) + ALP2 * Q * g.HZ;
    acc9(U, du, DISL3);
}

__device__ void ub(double XI, double ET, double Q, double DISL1, double DISL2, double DISL3,
                   const C0& c0, const C2& g, double U[9]) {
    const double ALP3 = c0.ALP3, SD = c0.SD, SDSD = c0.SDSD, SDCD = c0.SDCD;
    const double R = g.R, Y = g.Y, D = g.D;
    (void)ET;
    const double RD = R + D;
    const double D11 = 1.0 / (R * RD);
    const double AJ2 = XI * Y / RD * D11;
    const double AJ5 = -(D + Y * Y / RD) * D11;
    const double c1 = c0.CD != 0.0, c2 = c0.CD == 0.0;
    double CD = c1 * c0.CD + c2 * 1.0e-12;
    const double RD2 = RD * RD;
    // AI1..AI4 (with UB's atan and log(RD)) feed only the displacement rows and
    // are not formed.
    const double AK1 = c1 * (XI * (D11 - g.Y11 * SD) / CD) + c2 * (XI * Q / RD * D11);
    const double AK3 = c1 * ((Q * g.Y11 - Y * D11) / CD) + c2 * (SD / RD * (g.XI2 * D11 - 1.0));
    const double AJ3 = c1 * ((AK1 - AJ2 * SD) / CD) + c2 * (-XI / RD2 * (g.Q2 * D11 - 1.0 / 2.0));
    const double AJ6 = c1 * ((AK3 - AJ5 * SD) / CD) + c2 * (-Y / RD2 * (g.XI2 * D11 - 1.0 / 2.0));
    CD = c0.CD;
    const double XY = XI * g.Y11;
    const double AK2 = 1.0 / R + AK3 * SD;
    const double AK4 = XY * CD - AK1 * SD;
    const double AJ1 = AJ5 * CD - AJ6 * SD;
    const double AJ4 = -XY - AJ2 * CD + AJ3 * SD;
    const double QY = Q * g.Y11;
#pragma unroll
    for (int k = 0; k < 9; ++k) U[k] = 0.0;
    double du[9];
    du[0] = g.XI2 * Q * g.Y32 - ALP3 * AJ1 * SD;
    du[1] = XI * Q / g.R3 - ALP3 * AJ2 * SD;
    du[2] = -XI * g.Q2 * g.Y32 - ALP3 * AJ3 * SD;
    du[3] = -XI * g.FY - D * g.X11 + ALP3 * (XY + AJ4) * SD;
    du[4] = -g.EY + ALP3 * (1.0 / R + AJ5) * SD;
    du[5] = Q * g.FY - ALP3 * (QY - AJ6) * SD;
    du[6] = -XI * g.FZ - Y * g.X11 + ALP3 * AK1 * SD;
    du[7] = -g.EZ + ALP3 * Y * D11 * SD;
    du[8] = Q * g.FZ + ALP3 * AK2 * SD;
    acc9(U, du, DISL1);
    du[0] = XI * Q / g.R3 + ALP3 * AJ4 * SDCD;
    du[1] = ET * Q / g.R3 + QY + ALP3 * AJ5 * SDCD;
    du[2] = -g.Q2 / g.R3 + ALP3 * AJ6 * SDCD;
    du[3] = -g.EY + ALP3 * AJ1 * SDCD;
    du[4] = -ET * g.GY - XY * SD + ALP3 * AJ2 * SDCD;
    du[5] = Q * g.GY + ALP3 * AJ3 * SDCD;
    du[6] = -g.EZ - ALP3 * AK3 * SDCD;
    du[7] = -ET * g.GZ - XY * CD - ALP3 * XI * D11 * SDCD;
    du[8] = Q * g.GZ - ALP3 * AK4 * SDCD;
    acc9(U, du, DISL2);
    du[0] = -XI * g.Q2 * g.Y32 - ALP3 * AJ4 * SDSD;
    du[1] = -g.Q2 / g.R3 - ALP3 * AJ5 * SDSD;
    du[2] = Q * g.Q2 * g.Y32 - ALP3 * AJ6 * SDSD;
    du[3] = Q * g.FY - ALP3 * AJ1 * SDSD;
    du[4] = Q * g.GY - ALP3 * AJ2 * SDSD;
    du[5] = -Q * g.HY - ALP3 * AJ3 * SDSD;
    du[6] = Q * g.FZ + ALP3 * AK3 * SDSD;
    du[7] = Q * g.GZ + ALP3 * XI * D11 * SDSD;
    du[8] = -Q * g.HZ + ALP3 * AK4 * SDSD;
    acc9(U, du, DISL3);
}

// UC_V: all twelve rows are needed because the image combination adds
// DUC rows 1..3 into the z-gradient rows.
__device__ void uc(double XI, double ET, double Q, double DISL1, double DISL2, double DISL3,
                   double Z, const C0& c0, const C2& g, double U[12]) {
    const double ALP4 = c0.ALP4, ALP5 = c0.ALP5, SD = c0.SD, CD = c0.CD, SDSD = c0.SDSD,
                 CDCD = c0.CDCD, SDCD = c0.SDCD;
    const double R = g.R, R2 = g.R2, R3 = g.R3, R5 = g.R5, Y = g.Y, D = g.D, X11 = g.X11,
                 X32 = g.X32, Y11 = g.Y11, Y32 = g.Y32, XI2 = g.XI2, Q2 = g.Q2;
    const double C = D + Z;
    const double X53 = (8.0 * R2 + 9.0 * R * XI + 3.0 * XI2) * X11 * X11 * X11 / R2;
    const double Y53 = (8.0 * R2 + 9.0 * R * ET + 3.0 * g.ET2) * Y11 * Y11 * Y11 / R2;
    const double H = Q * CD - Z;
    const double Z32 = SD / R3 - H * Y32;
    const double Z53 = 3.0 * SD / R5 - H * Y53;
    const double Y0 = Y11 - XI2 * Y32;
    const double Z0 = Z32 - XI2 * Z53;
    const double PPY = CD / R3 + Q * Y32 * SD;
    const double PPZ = SD / R3 - Q * Y32 * CD;
    const double QQ = Z * Y32 + Z32 + Z0;
    const double QQY = 3.0 * C * D / R5 - QQ * SD;
    const double QQZ = 3.0 * C * Y / R5 - QQ * CD + Q * Y32;
    const double XY = XI * Y11, QY = Q * Y11, QR = 3.0 * Q / R5, CDR = (C + D) / R3;
    const double YY0 = Y / R3 - Y0 * CD;
    const double F1 = 1.0, F2 = 2.0, F3 = 3.0;
#pragma unroll
    for (int k = 0; k < 12; ++k) U[k] = 0.0;
    double du[12];
    const double PI2 = 6.283185307179586;
    auto acc12 = [&](double DISL) {
        const double s = DISL / PI2, c = (DISL != 0.0) ? 1.0 : 0.0;
#pragma unroll
        for (int k = 0; k < 12; ++k) U[k] = U[k] + s * du[k] * c;
    };
    du[0] = ALP4 * XY * CD - ALP5 * XI * Q * Z32;
    du[1] = ALP4 * (CD / R + F2 * QY * SD) - ALP5 * C * Q / R3;
    du[2] = ALP4 * QY * CD - ALP5 * (C * ET / R3 - Z * Y11 + XI2 * Z32);
    du[3] = ALP4 * Y0 * CD - ALP5 * Q * Z0;
    du[4] = -ALP4 * XI * (CD / R3 + F2 * Q * Y32 * SD) + ALP5 * C * XI * QR;
    du[5] = -ALP4 * XI * Q * Y32 * CD + ALP5 * XI * (F3 * C * ET / R5 - QQ);
    du[6] = -ALP4 * XI * PPY * CD - ALP5 * XI * QQY;
    du[7] = ALP4 * F2 * (D / R3 - Y0 * SD) * SD - Y / R3 * CD - ALP5 * (CDR * SD - ET / R3 - C * Y * QR);
    du[8] = -ALP4 * Q / R3 + YY0 * SD + ALP5 * (CDR * CD + C * D * QR - (Y0 * CD + Q * Z0) * SD);
    du[9] = ALP4 * XI * PPZ * CD - ALP5 * XI * QQZ;
    du[10] = ALP4 * F2 * (Y / R3 - Y0 * CD) * SD + D / R3 * CD - ALP5 * (CDR * CD + C * D * QR);
    du[11] = YY0 * CD - ALP5 * (CDR * SD - C * Y * QR - Y0 * SDSD + Q * Z0 * CD);
    acc12(DISL1);
    du[0] = ALP4 * CD / R - QY * SD - ALP5 * C * Q / R3;
    du[1] = ALP4 * Y * X11 - ALP5 * C * ET * Q * X32;
    du[2] = -D * X11 - XY * SD - ALP5 * C * (X11 - Q2 * X32);
    du[3] = -ALP4 * XI / R3 * CD + ALP5 * C * XI * QR + XI * Q * Y32 * SD;
    du[4] = -ALP4 * Y / R3 + ALP5 * C * ET * QR;
    du[5] = D / R3 - Y0 * SD + ALP5 * C / R3 * (F1 - F3 * Q2 / R2);
    du[6] = -ALP4 * ET / R3 + Y0 * SDSD - ALP5 * (CDR * SD - C * Y * QR);
    du[7] = ALP4 * (X11 - Y * Y * X32) - ALP5 * C * ((D + F2 * Q * CD) * X32 - Y * ET * Q * X53);
    du[8] = XI * PPY * SD + Y * D * X32 + ALP5 * C * ((Y + F2 * Q * SD) * X32 - Y * Q2 * X53);
    du[9] = -Q / R3 + Y0 * SDCD - ALP5 * (CDR * CD + C * D * QR);
    du[10] = ALP4 * Y * D * X32 - ALP5 * C * ((Y - F2 * Q * SD) * X32 + D * ET * Q * X53);
    du[11] = -XI * PPZ * SD + X11 - D * D * X32 - ALP5 * C * ((D - F2 * Q * CD) * X32 - D * Q2 * X53);
    acc12(DISL2);
    du[0] = -ALP4 * (SD / R + QY * CD) - ALP5 * (Z * Y11 - Q2 * Z32);
    du[1] = ALP4 * F2 * XY * SD + D * X11 - ALP5 * C * (X11 - Q2 * X32);
    du[2] = ALP4 * (Y * X11 + XY * CD) + ALP5 * Q * (C * ET * X32 + XI * Z32);
    du[3] = ALP4 * XI / R3 * SD + XI * Q * Y32 * CD + ALP5 * XI * (F3 * C * ET / R5 - F2 * Z32 - Z0);
    du[4] = ALP4 * F2 * Y0 * SD - D / R3 + ALP5 * C / R3 * (F1 - F3 * Q2 / R2);
    du[5] = -ALP4 * YY0 - ALP5 * (C * ET * QR - Q * Z0);
    du[6] = ALP4 * (Q / R3 + Y0 * SDCD) + ALP5 * (Z / R3 * CD + C * D * QR - Q * Z0 * SD);
    du[7] = -ALP4 * F2 * XI * PPY * SD - Y * D * X32 + ALP5 * C * ((Y + F2 * Q * SD) * X32 - Y * Q2 * X53);
    du[8] = -ALP4 * (XI * PPY * CD - X11 + Y * Y * X32) + ALP5 * (C * ((D + F2 * Q * CD) * X32 - Y * ET * Q * X53) + XI * QQY);
    du[9] = -ET / R3 + Y0 * CDCD - ALP5 * (Z / R3 * SD - C * Y * QR - Y0 * SDSD + Q * Z0 * CD);
    du[10] = ALP4 * F2 * XI * PPZ * SD - X11 + D * D * X32 - ALP5 * C * ((D - F2 * Q * CD) * X32 - D * Q2 * X53);
    du[11] = ALP4 * (XI * PPZ * CD + Y * D * X32) + ALP5 * (C * ((Y - F2 * Q * SD) * X32 + D * ET * Q * X53) + XI * QQZ);
    acc12(DISL3);
}

// Gradients g[0..8] = UXX,UYX,UZX,UXY,UYY,UZY,UXZ,UYZ,UZZ of Okada_DC3D_Vector.
__device__ void dc3d_gradients(const C0& c0, double X, double Y, double Z, double DEPTH,
                               double AL1, double AL2, double AW1, double AW2, double DISL1,
                               double DISL2, double DISL3, double Ug[9]) {
    const double SD = c0.SD, CD = c0.CD;
#pragma unroll
    for (int k = 0; k < 9; ++k) Ug[k] = 0.0;
    // real source (:495-567)
    {
        const double D = DEPTH + Z;
        const double P = Y * CD + D * SD;
        const double Q = Y * SD - D * CD;
#pragma unroll 1
        for (int K = 1; K <= 2; ++K) {
            const double ET = (K == 1) ? P + AW1 : P - AW2;
#pragma unroll 1
            for (int J = 1; J <= 2; ++J) {
                const double XI = (J == 1) ? X + AL1 : X - AL2;
                C2 g;
                dccon2(XI, ET, Q, SD, CD, g);
                double A[9];
                ua(XI, ET, Q, DISL1, DISL2, DISL3, c0, g, A);
                double DU[9];
                // rows I = 4,7 (here 0,3) and I = 10 (here 6, sign-flipped)
#pragma unroll
                for (int I = 0; I < 9; I += 3) {
                    DU[I] = -A[I];
                    DU[I + 1] = -A[I + 1] * CD + A[I + 2] * SD;
                    DU[I + 2] = -A[I + 1] * SD - A[I + 2] * CD;
                }
                DU[6] = -DU[6]; DU[7] = -DU[7]; DU[8] = -DU[8];
                const double sgn = (J + K != 3) ? 1.0 : -1.0;
#pragma unroll
                for (int k = 0; k < 9; ++k) Ug[k] = (sgn > 0) ? Ug[k] + DU[k] : Ug[k] - DU[k];
            }
        }
    }
    // image source (:574-634)
    {
        const double D = DEPTH - Z;
        const double P = Y * CD + D * SD;
        const double Q = Y * SD - D * CD;
#pragma unroll 1
        for (int K = 1; K <= 2; ++K) {
            const double ET = (K == 1) ? P + AW1 : P - AW2;
#pragma unroll 1
            for (int J = 1; J <= 2; ++J) {
                const double XI = (J == 1) ? X + AL1 : X - AL2;
                C2 g;
                dccon2(XI, ET, Q, SD, CD, g);
                double A[9], B[9], Cc[12];
                ua(XI, ET, Q, DISL1, DISL2, DISL3, c0, g, A);
                ub(XI, ET, Q, DISL1, DISL2, DISL3, c0, g, B);
                uc(XI, ET, Q, DISL1, DISL2, DISL3, Z, c0, g, Cc);
                double DU[9];
#pragma unroll
                for (int I = 0; I < 9; I += 3) {
                    const double* Ci = Cc + 3 + I;
                    DU[I] = A[I] + B[I] + Z * Ci[0];
                    DU[I + 1] = (A[I + 1] + B[I + 1] + Z * Ci[1]) * CD - (A[I + 2] + B[I + 2] + Z * Ci[2]) * SD;
                    DU[I + 2] = (A[I + 1] + B[I + 1] - Z * Ci[1]) * SD + (A[I + 2] + B[I + 2] - Z * Ci[2]) * CD;
                }
                DU[6] = DU[6] + Cc[0];
                DU[7] = DU[7] + Cc[1] * CD - Cc[2] * SD;
                DU[8] = DU[8] - Cc[1] * SD - Cc[2] * CD;
                const double sgn = (J + K != 3) ? 1.0 : -1.0;
#pragma unroll
                for (int k = 0; k < 9; ++k) Ug[k] = (sgn > 0) ? Ug[k] + DU[k] : Ug[k] - DU[k];
            }
        }
    }
}

}  // namespace okada
}  // namespace qdfn
