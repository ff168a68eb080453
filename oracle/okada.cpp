// Oracle: Okada (1992) DC3D displacement gradients of a finite rectangular
// dislocation in an elastic half-space, restated point by point from the
// reference's vectorised Julia version:
//   scripts/Functions_OKADA3D.jl
//     DCCON0_V            :12-48
//     DCCON2_V            :51-195
//     UA_V                :199-262
//     UB_V                :266-375
//     UC_V                :378-460
//     Okada_DC3D_Vector   :464-654
// The reference evaluates every receiver independently (all broadcasts are
// elementwise), so a scalar restatement per receiver is exact.  Reference
// semantics kept on purpose:
//   * the EPS zeroing of XI/ET/Q happens on DCCON2's local copies only; UA/UB/UC
//     receive the caller's un-zeroed XI, ET, Q (Julia rebinds, never mutates);
//   * masks are applied by IEEE multiplication (`c*expr`), so a masked-out
//     branch that is Inf/NaN still turns the sum into NaN, as in the reference;
//   * UB's `ATAN[isnan] = 0` and the CD==0 -> 1e-12 substitution (:288-311);
//   * DCCON2 overwrites the caller's Y and D (tuple assignment at :530/:599),
//     so UA/UB/UC see DCCON2's Y and D.
//
// TEST INFRASTRUCTURE ONLY (CPU oracle); not part of the shipped library.
#include <cmath>
#include "oracle.h"

namespace {

struct C0 { double ALP1, ALP2, ALP3, ALP4, ALP5, SD, CD, SDSD, CDCD, SDCD; };

C0 dccon0(double ALPHA, double DIP) {
    const double F0 = 0, F1 = 1, F2 = 2, PI2 = 6.283185307179586, EPS = 1.0e-6;
    C0 c;
    c.ALP1 = (F1 - ALPHA) / F2;
    c.ALP2 = ALPHA / F2;
    c.ALP3 = (F1 - ALPHA) / ALPHA;
    c.ALP4 = F1 - ALPHA;
    c.ALP5 = ALPHA;
    double P18 = PI2 / 360.0;
    double SD = std::sin(DIP * P18);
    double CD = std::cos(DIP * P18);
    double c1 = std::fabs(CD) < EPS, c2 = std::fabs(CD) >= EPS;
    double s1 = SD > F0, s2 = SD == F0, s3 = SD < F0;
    CD = F0 * c1 + CD * c2;
    SD = c1 * (F1 * s1 + SD * s2 + (-1.0) * F1 * s3) + c2 * SD;
    c.SD = SD; c.CD = CD;
    c.SDSD = SD * SD; c.CDCD = CD * CD; c.SDCD = SD * CD;
    return c;
}

struct C2 {
    double XI2, ET2, Q2, R2, R, R3, R5, Y, D, TT, ALX, X11, X32, ALE, Y11, Y32,
        EY, EZ, FY, FZ, GY, GZ, HY, HZ;
};

C2 dccon2(double XI, double ET, double Q, double SD, double CD) {
    const double F0 = 0, F1 = 1, F2 = 2.0, EPS = 0.000001;
    C2 o;
    {
        double c1 = std::fabs(XI) < EPS, c2 = std::fabs(XI) >= EPS;
        XI = F0 * c1 + XI * c2;
        c1 = std::fabs(ET) < EPS; c2 = std::fabs(ET) >= EPS;
        ET = F0 * c1 + ET * c2;
        c1 = std::fabs(Q) < EPS; c2 = std::fabs(Q) >= EPS;
        Q = F0 * c1 + Q * c2;
    }
    o.XI2 = XI * XI; o.ET2 = ET * ET; o.Q2 = Q * Q;
    o.R2 = o.XI2 + o.ET2 + o.Q2;
    o.R = std::sqrt(o.R2);
    double R = o.R;
    o.R3 = R * o.R2;
    o.R5 = o.R3 * o.R2;
    o.Y = ET * CD + Q * SD;
    o.D = ET * SD - Q * CD;
    // :90-101
    if (!(Q != F0)) o.TT = 0;
    else o.TT = 0.0 * F0 + 1.0 * std::atan(XI * ET / (Q * R));
    // :107-143
    {
        int c4 = (XI < F0) && (Q == F0) && (ET == F0);
        int c5 = 1 - c4;
        double RXI = R + XI;
        if (c5 == 0) {
            o.ALX = (-std::log(R - XI)) * c4;
            o.X11 = F0 * c4;
            o.X32 = F0 * c4;
        } else {
            o.ALX = std::log(RXI) * c5;
            o.X11 = (F1 / (R * RXI)) * c5;
            o.X32 = ((R + RXI) * o.X11 * o.X11 / R) * c5;
        }
    }
    // :145-182
    {
        int c4 = (ET < F0) && (Q == F0) && (XI == F0);
        double c5 = 1.0 - c4;
        double RET = R + ET;
        if (c5 == 0) {
            o.ALE = (-std::log(R - ET)) * c4;
            o.Y11 = F0 * c4;
            o.Y32 = F0 * c4;
        } else {
            o.ALE = std::log(RET) * c5;
            o.Y11 = (F1 / (R * RET)) * c5;
            o.Y32 = ((R + RET) * o.Y11 * o.Y11 / R) * c5;
        }
    }
    o.EY = SD / R - o.Y * Q / o.R3;
    o.EZ = CD / R + o.D * Q / o.R3;
    o.FY = o.D / o.R3 + o.XI2 * o.Y32 * SD;
    o.FZ = o.Y / o.R3 + o.XI2 * o.Y32 * CD;
    o.GY = F2 * o.X11 * SD - o.Y * Q * o.X32;
    o.GZ = F2 * o.X11 * CD + o.D * Q * o.X32;
    o.HY = o.D * Q * o.X32 + XI * Q * o.Y32 * SD;
    o.HZ = o.Y * Q * o.X32 + XI * Q * o.Y32 * CD;
    return o;
}

// U += (DISL/PI2) * du * c    (mask c = DISL != 0, applied by multiplication)
inline void accum(double U[12], const double du[12], double DISL) {
    const double PI2 = 6.283185307179586;
    double c = (DISL != 0.0) ? 1.0 : 0.0;
    double s = DISL / PI2;
    for (int k = 0; k < 12; ++k) U[k] = U[k] + s * du[k] * c;
}

void ua(double XI, double ET, double Q, double DISL1, double DISL2, double DISL3,
        const C0& c0, const C2& g, double U[12]) {
    const double F2 = 2.0;
    const double ALP1 = c0.ALP1, ALP2 = c0.ALP2, SD = c0.SD, CD = c0.CD;
    const double XI2 = g.XI2, Q2 = g.Q2, R = g.R, R3 = g.R3, Y = g.Y, D = g.D,
                 TT = g.TT, ALX = g.ALX, X11 = g.X11, ALE = g.ALE, Y11 = g.Y11,
                 Y32 = g.Y32, EY = g.EY, EZ = g.EZ, FY = g.FY, FZ = g.FZ, GY = g.GY,
                 GZ = g.GZ, HY = g.HY, HZ = g.HZ;
    for (int k = 0; k < 12; ++k) U[k] = 0.0;
    double XY = XI * Y11, QX = Q * X11, QY = Q * Y11;
    double du[12];
    du[0] = TT / F2 + ALP2 * XI * QY;
    du[1] = ALP2 * Q / R;
    du[2] = ALP1 * ALE - ALP2 * Q * QY;
    du[3] = -ALP1 * QY - ALP2 * XI2 * Q * Y32;
    du[4] = -ALP2 * XI * Q / R3;
    du[5] = ALP1 * XY + ALP2 * XI * Q2 * Y32;
    du[6] = ALP1 * XY * SD + ALP2 * XI * FY + D / F2 * X11;
    du[7] = ALP2 * EY;
    du[8] = ALP1 * (CD / R + QY * SD) - ALP2 * Q * FY;
    du[9] = ALP1 * XY * CD + ALP2 * XI * FZ + Y / F2 * X11;
    du[10] = ALP2 * EZ;
    du[11] = -ALP1 * (SD / R - QY * CD) - ALP2 * Q * FZ;
    accum(U, du, DISL1);
    du[0] = ALP2 * Q / R;
    du[1] = TT / F2 + ALP2 * ET * QX;
    du[2] = ALP1 * ALX - ALP2 * Q * QX;
    du[3] = -ALP2 * XI * Q / R3;
    du[4] = -QY / F2 - ALP2 * ET * Q / R3;
    du[5] = ALP1 / R + ALP2 * Q2 / R3;
    du[6] = ALP2 * EY;
    du[7] = ALP1 * D * X11 + XY / F2 * SD + ALP2 * ET * GY;
    du[8] = ALP1 * Y * X11 - ALP2 * Q * GY;
    du[9] = ALP2 * EZ;
    du[10] = ALP1 * Y * X11 + XY / F2 * CD + ALP2 * ET * GZ;
    du[11] = -ALP1 * D * X11 - ALP2 * Q * GZ;
    accum(U, du, DISL2);
    du[0] = -ALP1 * ALE - ALP2 * Q * QY;
    du[1] = -ALP1 * ALX - ALP2 * Q * QX;
    du[2] = TT / F2 - ALP2 * (ET * QX + XI * QY);
    du[3] = -ALP1 * XY + ALP2 * XI * Q2 * Y32;
    du[4] = -ALP1 / R + ALP2 * Q2 / R3;
    du[5] = -ALP1 * QY - ALP2 * Q * Q2 * Y32;
    du[6] = -ALP1 * (CD / R + QY * SD) - ALP2 * Q * FY;
    du[7] = -ALP1 * Y * X11 - ALP2 * Q * GY;
    du[8] = ALP1 * (D * X11 + XY * SD) + ALP2 * Q * HY;
    du[9] = ALP1 * (SD / R - QY * CD) - ALP2 * Q * FZ;
    du[10] = ALP1 * D * X11 - ALP2 * Q * GZ;
    du[11] = ALP1 * (Y * X11 + XY * CD) + ALP2 * Q * HZ;
    accum(U, du, DISL3);
}

void ub(double XI, double ET, double Q, double DISL1, double DISL2, double DISL3,
        const C0& c0, const C2& g, double U[12]) {
    const double F0 = 0.0, F1 = 1.0, F2 = 2.0;
    const double ALP3 = c0.ALP3, SD = c0.SD, SDSD = c0.SDSD, SDCD = c0.SDCD;
    double CD = c0.CD, CDCD = c0.CDCD;
    const double XI2 = g.XI2, Q2 = g.Q2, R = g.R, R3 = g.R3, Y = g.Y, D = g.D,
                 TT = g.TT, X11 = g.X11, ALE = g.ALE, Y11 = g.Y11, Y32 = g.Y32,
                 EY = g.EY, EZ = g.EZ, FY = g.FY, FZ = g.FZ, GY = g.GY, GZ = g.GZ,
                 HY = g.HY, HZ = g.HZ;
    double RD = R + D;
    double D11 = F1 / (R * RD);
    double AJ2 = XI * Y / RD * D11;
    double AJ5 = -(D + Y * Y / RD) * D11;
    double c1 = CD != F0, c2 = CD == F0;
    double s1 = XI == F0, s2 = XI != F0;
    const double tempCD = CD, tempCDCD = CDCD;
    CD = c1 * CD + c2 * 1.0e-12;
    CDCD = c1 * CDCD + c2 * 1.0e-12;
    double X = std::sqrt(XI2 + Q2);
    double ATAN = std::atan((ET * (X + Q * CD) + X * (R + X) * SD) / (XI * (R + X) * CD));
    if (std::isnan(ATAN)) ATAN = 0.0;
    double RD2 = RD * RD;
    double AI4 = c1 * (s1 * F0 + s2 * (F1 / CDCD * (XI / RD * SDCD + F2 * ATAN))) +
                 c2 * (XI * Y / RD2 / F2);
    double AI3 = c1 * ((Y * CD / RD - ALE + SD * std::log(RD)) / CDCD) +
                 c2 * ((ET / RD + Y * Q / RD2 - ALE) / F2);
    double AK1 = c1 * (XI * (D11 - Y11 * SD) / CD) + c2 * (XI * Q / RD * D11);
    double AK3 = c1 * ((Q * Y11 - Y * D11) / CD) + c2 * (SD / RD * (XI2 * D11 - F1));
    double AJ3 = c1 * ((AK1 - AJ2 * SD) / CD) + c2 * (-XI / RD2 * (Q2 * D11 - F1 / F2));
    double AJ6 = c1 * ((AK3 - AJ5 * SD) / CD) + c2 * (-Y / RD2 * (XI2 * D11 - F1 / F2));
    CD = tempCD;
    CDCD = tempCDCD;
    double XY = XI * Y11;
    double AI1 = -XI / RD * CD - AI4 * SD;
    double AI2 = std::log(RD) + AI3 * SD;
    double AK2 = F1 / R + AK3 * SD;
    double AK4 = XY * CD - AK1 * SD;
    double AJ1 = AJ5 * CD - AJ6 * SD;
    double AJ4 = -XY - AJ2 * CD + AJ3 * SD;
    for (int k = 0; k < 12; ++k) U[k] = 0.0;
    double QX = Q * X11, QY = Q * Y11;
    double du[12];
    du[0] = -XI * QY - TT - ALP3 * AI1 * SD;
    du[1] = -Q / R + ALP3 * Y / RD * SD;
    du[2] = Q * QY - ALP3 * AI2 * SD;
    du[3] = XI2 * Q * Y32 - ALP3 * AJ1 * SD;
    du[4] = XI * Q / R3 - ALP3 * AJ2 * SD;
    du[5] = -XI * Q2 * Y32 - ALP3 * AJ3 * SD;
    du[6] = -XI * FY - D * X11 + ALP3 * (XY + AJ4) * SD;
    du[7] = -EY + ALP3 * (F1 / R + AJ5) * SD;
    du[8] = Q * FY - ALP3 * (QY - AJ6) * SD;
    du[9] = -XI * FZ - Y * X11 + ALP3 * AK1 * SD;
    du[10] = -EZ + ALP3 * Y * D11 * SD;
    du[11] = Q * FZ + ALP3 * AK2 * SD;
    accum(U, du, DISL1);
    du[0] = -Q / R + ALP3 * AI3 * SDCD;
    du[1] = -ET * QX - TT - ALP3 * XI / RD * SDCD;
    du[2] = Q * QX + ALP3 * AI4 * SDCD;
    du[3] = XI * Q / R3 + ALP3 * AJ4 * SDCD;
    du[4] = ET * Q / R3 + QY + ALP3 * AJ5 * SDCD;
    du[5] = -Q2 / R3 + ALP3 * AJ6 * SDCD;
    du[6] = -EY + ALP3 * AJ1 * SDCD;
    du[7] = -ET * GY - XY * SD + ALP3 * AJ2 * SDCD;
    du[8] = Q * GY + ALP3 * AJ3 * SDCD;
    du[9] = -EZ - ALP3 * AK3 * SDCD;
    du[10] = -ET * GZ - XY * CD - ALP3 * XI * D11 * SDCD;
    du[11] = Q * GZ - ALP3 * AK4 * SDCD;
    accum(U, du, DISL2);
    du[0] = Q * QY - ALP3 * AI3 * SDSD;
    du[1] = Q * QX + ALP3 * XI / RD * SDSD;
    du[2] = ET * QX + XI * QY - TT - ALP3 * AI4 * SDSD;
    du[3] = -XI * Q2 * Y32 - ALP3 * AJ4 * SDSD;
    du[4] = -Q2 / R3 - ALP3 * AJ5 * SDSD;
    du[5] = Q * Q2 * Y32 - ALP3 * AJ6 * SDSD;
    du[6] = Q * FY - ALP3 * AJ1 * SDSD;
    du[7] = Q * GY - ALP3 * AJ2 * SDSD;
    du[8] = -Q * HY - ALP3 * AJ3 * SDSD;
    du[9] = Q * FZ + ALP3 * AK3 * SDSD;
    du[10] = Q * GZ + ALP3 * XI * D11 * SDSD;
    du[11] = -Q * HZ + ALP3 * AK4 * SDSD;
    accum(U, du, DISL3);
}

void uc(double XI, double ET, double Q, double DISL1, double DISL2, double DISL3,
        double Z, const C0& c0, const C2& g, double U[12]) {
    const double F1 = 1.0, F2 = 2.0, F3 = 3.0;
    const double ALP4 = c0.ALP4, ALP5 = c0.ALP5, SD = c0.SD, CD = c0.CD,
                 SDSD = c0.SDSD, CDCD = c0.CDCD, SDCD = c0.SDCD;
    const double XI2 = g.XI2, ET2 = g.ET2, Q2 = g.Q2, R2 = g.R2, R = g.R, R3 = g.R3,
                 R5 = g.R5, Y = g.Y, D = g.D, X11 = g.X11, X32 = g.X32, Y11 = g.Y11,
                 Y32 = g.Y32;
    double C = D + Z;
    double X53 = (8.0 * R2 + 9.0 * R * XI + F3 * XI2) * X11 * X11 * X11 / R2;
    double Y53 = (8.0 * R2 + 9.0 * R * ET + F3 * ET2) * Y11 * Y11 * Y11 / R2;
    double H = Q * CD - Z;
    double Z32 = SD / R3 - H * Y32;
    double Z53 = F3 * SD / R5 - H * Y53;
    double Y0 = Y11 - XI2 * Y32;
    double Z0 = Z32 - XI2 * Z53;
    double PPY = CD / R3 + Q * Y32 * SD;
    double PPZ = SD / R3 - Q * Y32 * CD;
    double QQ = Z * Y32 + Z32 + Z0;
    double QQY = F3 * C * D / R5 - QQ * SD;
    double QQZ = F3 * C * Y / R5 - QQ * CD + Q * Y32;
    double XY = XI * Y11;
    double QY = Q * Y11;
    double QR = F3 * Q / R5;
    double CDR = (C + D) / R3;
    double YY0 = Y / R3 - Y0 * CD;
    for (int k = 0; k < 12; ++k) U[k] = 0.0;
    double du[12];
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
    accum(U, du, DISL1);
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
    accum(U, du, DISL2);
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
    accum(U, du, DISL3);
}

}  // namespace

extern "C" void oracle_okada_dc3d(double ALPHA, double X, double Y, double Z, double DEPTH,
                                  double DIP, double AL1, double AL2, double AW1, double AW2,
                                  double DISL1, double DISL2, double DISL3, double out[12],
                                  int* iret) {
    double U[12];
    for (int k = 0; k < 12; ++k) U[k] = 0.0;
    C0 c0 = dccon0(ALPHA, DIP);
    const double SD = c0.SD, CD = c0.CD;
    int IRET = 0;
    // ---- real-source contribution (:495-567)
    {
        double D = DEPTH + Z;
        double P = Y * CD + D * SD;
        double Q = Y * SD - D * CD;
        int JXI = ((X + AL1) * (X - AL2) <= 0.0);
        int JET = ((P + AW1) * (P - AW2) <= 0.0);
        for (int K = 1; K <= 2; ++K) {
            double ET = (K == 1) ? P + AW1 : P - AW2;
            for (int J = 1; J <= 2; ++J) {
                double XI = (J == 1) ? X + AL1 : X - AL2;
                C2 g = dccon2(XI, ET, Q, SD, CD);
                int cq1 = std::fabs(Q) <= 1.0e-12, cet1 = std::fabs(ET) <= 1.0e-12,
                    cxi1 = std::fabs(XI) <= 1.0e-12;
                int cc1 = (JXI == 1) * cq1 * cet1, cc3 = (JET == 1) * cq1 * cxi1;
                IRET += ((cc1 + cc3) >= 1);
                double DUA[12], DU[12];
                ua(XI, ET, Q, DISL1, DISL2, DISL3, c0, g, DUA);
                for (int I = 0; I <= 9; I += 3) {
                    DU[I] = -DUA[I];
                    DU[I + 1] = -DUA[I + 1] * CD + DUA[I + 2] * SD;
                    DU[I + 2] = -DUA[I + 1] * SD - DUA[I + 2] * CD;
                    if (I < 9) continue;
                    DU[I] = -DU[I];
                    DU[I + 1] = -DU[I + 1];
                    DU[I + 2] = -DU[I + 2];
                }
                if (J + K != 3) for (int k = 0; k < 12; ++k) U[k] = U[k] + DU[k];
                else for (int k = 0; k < 12; ++k) U[k] = U[k] - DU[k];
            }
        }
    }
    // ---- image-source contribution (:574-634)
    {
        double D = DEPTH - Z;
        double P = Y * CD + D * SD;
        double Q = Y * SD - D * CD;
        for (int K = 1; K <= 2; ++K) {
            double ET = (K == 1) ? P + AW1 : P - AW2;
            for (int J = 1; J <= 2; ++J) {
                double XI = (J == 1) ? X + AL1 : X - AL2;
                C2 g = dccon2(XI, ET, Q, SD, CD);
                double DUA[12], DUB[12], DUC[12], DU[12];
                ua(XI, ET, Q, DISL1, DISL2, DISL3, c0, g, DUA);
                ub(XI, ET, Q, DISL1, DISL2, DISL3, c0, g, DUB);
                uc(XI, ET, Q, DISL1, DISL2, DISL3, Z, c0, g, DUC);
                for (int I = 0; I <= 9; I += 3) {
                    DU[I] = DUA[I] + DUB[I] + Z * DUC[I];
                    DU[I + 1] = (DUA[I + 1] + DUB[I + 1] + Z * DUC[I + 1]) * CD -
                                (DUA[I + 2] + DUB[I + 2] + Z * DUC[I + 2]) * SD;
                    DU[I + 2] = (DUA[I + 1] + DUB[I + 1] - Z * DUC[I + 1]) * SD +
                                (DUA[I + 2] + DUB[I + 2] - Z * DUC[I + 2]) * CD;
                    if (I < 9) continue;
                    DU[9] = DU[9] + DUC[0];
                    DU[10] = DU[10] + DUC[1] * CD - DUC[2] * SD;
                    DU[11] = DU[11] - DUC[1] * SD - DUC[2] * CD;
                }
                if (J + K != 3) for (int k = 0; k < 12; ++k) U[k] = U[k] + DU[k];
                else for (int k = 0; k < 12; ++k) U[k] = U[k] - DU[k];
            }
        }
    }
    for (int k = 0; k < 12; ++k) out[k] = U[k];
    if (iret) *iret = IRET >= 1;
}
