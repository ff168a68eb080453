// Device stresses of a triangular dislocation in an elastic half-space
// (Nikkhoo & Walter 2015, GJI; MIT-licensed original by M. Nikkhoo), one
// (receiver, source) pair per thread.  Follows scripts/Functions_TDstressHS.jl
// (TDstressHS :2-130, TDstressFS :133-286, TDstress_HarFunc :289-335,
// TensTrans :338, CoordTrans :365, trimodefinder :393, TDSetupS :433,
// AngSetupFSC_S :467, AngDisStrain :577, AngDisStrainFSC :654-1034).
// Points on a TD edge give NaN, as in the reference (:262-267).
#pragma once
#include <math_constants.h>
#include "qdfn_internal.h"

namespace qdfn {
namespace tdhs {


__device__ __forceinline__ double sq(double x) { return x * x; }
__device__ __forceinline__ double cube(double x) { return x * x * x; }
__device__ __forceinline__ double p5(double x) { double x2 = x * x; return x2 * x2 * x; }

// TensTrans with A given column-major (A[0..8] = A[1..9] of the reference).
__device__ void tens_trans(const double t[6], const double* A, double o[6]) {
    const double A1 = A[0], A2 = A[1], A3 = A[2], A4 = A[3], A5 = A[4], A6 = A[5],
                 A7 = A[6], A8 = A[7], A9 = A[8];
    const double Txx1 = t[0], Tyy1 = t[1], Tzz1 = t[2], Txy1 = t[3], Txz1 = t[4], Tyz1 = t[5];
    o[0] = sq(A1) * Txx1 + 2 * A1 * A4 * Txy1 + 2 * A1 * A7 * Txz1 + 2 * A4 * A7 * Tyz1 +
           sq(A4) * Tyy1 + sq(A7) * Tzz1;
    o[1] = sq(A2) * Txx1 + 2 * A2 * A5 * Txy1 + 2 * A2 * A8 * Txz1 + 2 * A5 * A8 * Tyz1 +
           sq(A5) * Tyy1 + sq(A8) * Tzz1;
    o[2] = sq(A3) * Txx1 + 2 * A3 * A6 * Txy1 + 2 * A3 * A9 * Txz1 + 2 * A6 * A9 * Tyz1 +
           sq(A6) * Tyy1 + sq(A9) * Tzz1;
    o[3] = A1 * A2 * Txx1 + (A1 * A5 + A2 * A4) * Txy1 + (A1 * A8 + A2 * A7) * Txz1 +
           (A8 * A4 + A7 * A5) * Tyz1 + A5 * A4 * Tyy1 + A7 * A8 * Tzz1;
    o[4] = A1 * A3 * Txx1 + (A1 * A6 + A3 * A4) * Txy1 + (A1 * A9 + A3 * A7) * Txz1 +
           (A9 * A4 + A7 * A6) * Tyz1 + A6 * A4 * Tyy1 + A7 * A9 * Tzz1;
    o[5] = A2 * A3 * Txx1 + (A3 * A5 + A2 * A6) * Txy1 + (A3 * A8 + A2 * A9) * Txz1 +
           (A8 * A6 + A9 * A5) * Tyz1 + A5 * A6 * Tyy1 + A8 * A9 * Tzz1;
}

// r = A * (x1,x2,x3) with A a 3x3 given column-major.
__device__ void coord_trans(double x1, double x2, double x3, const double* A, double r[3]) {
    r[0] = A[0] * x1 + A[3] * x2 + A[6] * x3;
    r[1] = A[1] * x1 + A[4] * x2 + A[7] * x3;
    r[2] = A[2] * x1 + A[5] * x2 + A[8] * x3;
}

__device__ void cross3(const double a[3], const double b[3], double c[3]) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ double norm3(const double a[3]) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

// AngDisStrain (:577-651): strains of an angular dislocation, full space.
__device__ void ang_dis_strain(double x, double y, double z, double alpha, double bx, double by,
                    double bz, double nu, double e[6]) {
    const double pi = CUDART_PI;
    double sinA = sin(alpha), cosA = cos(alpha);
    double eta = y * cosA - z * sinA;
    double zeta = y * sinA + z * cosA;
    double x2 = sq(x), y2 = sq(y), z2 = sq(z);
    double r2 = x2 + y2 + z2;
    double r = sqrt(r2);
    double r3 = r * r2;
    double rz = r * (r - z);
    double r2z2 = r2 * sq(r - z);
    double r3z = r3 * (r - z);
    double W = zeta - r;
    double W2 = sq(W);
    double Wr = W * r;
    double W2r = W2 * r;
    double Wr3 = W * r3;
    double W2r2 = W2 * r2;
    double C = (r * cosA - z) / Wr;
    double S = (r * sinA - y) / Wr;
    double rFi_rx = (eta / r / (r - zeta) - y / r / (r - z)) / 4 / pi;
    double rFi_ry = (x / r / (r - z) - cosA * x / r / (r - zeta)) / 4 / pi;
    double rFi_rz = (sinA * x / r / (r - zeta)) / 4 / pi;

    e[0] = bx * (rFi_rx) +
           bx / 8 / pi / (1 - nu) * (eta / Wr + eta * x2 / W2r2 - eta * x2 / Wr3 + y / rz -
                                      x2 * y / r2z2 - x2 * y / r3z) -
           by * x / 8 / pi / (1 - nu) *
               (((2 * nu + 1) / Wr + x2 / W2r2 - x2 / Wr3) * cosA + (2 * nu + 1) / rz -
                x2 / r2z2 - x2 / r3z) +
           bz * x * sinA / 8 / pi / (1 - nu) * ((2 * nu + 1) / Wr + x2 / W2r2 - x2 / Wr3);
    e[1] = by * (rFi_ry) +
           bx / 8 / pi / (1 - nu) *
               ((1 / Wr + sq(S) - y2 / Wr3) * eta + (2 * nu + 1) * y / rz - cube(y) / r2z2 -
                cube(y) / r3z - 2 * nu * cosA * S) -
           by * x / 8 / pi / (1 - nu) *
               (1 / rz - y2 / r2z2 - y2 / r3z + (1 / Wr + sq(S) - y2 / Wr3) * cosA) +
           bz * x * sinA / 8 / pi / (1 - nu) * (1 / Wr + sq(S) - y2 / Wr3);
    e[2] = bz * (rFi_rz) +
           bx / 8 / pi / (1 - nu) *
               (eta / W / r + eta * sq(C) - eta * z2 / Wr3 + y * z / r3 + 2 * nu * sinA * C) -
           by * x / 8 / pi / (1 - nu) * ((1 / Wr + sq(C) - z2 / Wr3) * cosA + z / r3) +
           bz * x * sinA / 8 / pi / (1 - nu) * (1 / Wr + sq(C) - z2 / Wr3);
    e[3] = bx * (rFi_ry) / 2 + by * (rFi_rx) / 2 -
           bx / 8 / pi / (1 - nu) *
               (x * y2 / r2z2 - nu * x / rz + x * y2 / r3z - nu * x * cosA / Wr +
                eta * x * S / Wr + eta * x * y / Wr3) +
           by / 8 / pi / (1 - nu) *
               (x2 * y / r2z2 - nu * y / rz + x2 * y / r3z + nu * cosA * S +
                x2 * y * cosA / Wr3 + x2 * cosA * S / Wr) -
           bz * sinA / 8 / pi / (1 - nu) * (nu * S + x2 * S / Wr + x2 * y / Wr3);
    e[4] = bx * (rFi_rz) / 2 + bz * (rFi_rx) / 2 -
           bx / 8 / pi / (1 - nu) *
               (-x * y / r3 + nu * x * sinA / Wr + eta * x * C / Wr + eta * x * z / Wr3) +
           by / 8 / pi / (1 - nu) *
               (-x2 / r3 + nu / r + nu * cosA * C + x2 * z * cosA / Wr3 + x2 * cosA * C / Wr) -
           bz * sinA / 8 / pi / (1 - nu) * (nu * C + x2 * C / Wr + x2 * z / Wr3);
    e[5] = by * (rFi_rz) / 2 + bz * (rFi_ry) / 2 +
           bx / 8 / pi / (1 - nu) *
               (y2 / r3 - nu / r - nu * cosA * C + nu * sinA * S + eta * sinA * cosA / W2 -
                eta * (y * cosA + z * sinA) / W2r + eta * y * z / W2r2 - eta * y * z / Wr3) -
           by * x / 8 / pi / (1 - nu) *
               (y / r3 + sinA * sq(cosA) / W2 - cosA * (y * cosA + z * sinA) / W2r +
                y * z * cosA / W2r2 - y * z * cosA / Wr3) -
           bz * x * sinA / 8 / pi / (1 - nu) *
               (y * z / Wr3 - sinA * cosA / W2 + (y * cosA + z * sinA) / W2r - y * z / W2r2);
}

// AngDisStrainFSC (:654-1034): harmonic (free-surface correction) strains of an
// angular dislocation in a half-space.  The six closed-form expressions are the
// published Nikkhoo & Walter (2015) formulas, written out term by term.
__device__ void ang_dis_strain_fsc(double y1, double y2, double y3, double beta, double b1, double b2,
                        double b3, double nu, double a, double v[6]) {
    const double pi = CUDART_PI;
    double sinB = sin(beta), cosB = cos(beta), cotB = 1.0 / tan(beta);
    double y3b = y3 + 2 * a;
    double z1b = y1 * cosB + y3b * sinB;
    double z3b = -y1 * sinB + y3b * cosB;
    double rb2 = sq(y1) + sq(y2) + sq(y3b);
    double rb = sqrt(rb2);
    double W1 = rb * cosB + y3b;
    double W2 = cosB + a / rb;
    double W3 = cosB + y3b / rb;
    double W4 = nu + a / rb;
    double W5 = 2 * nu + a / rb;
    double W6 = rb + y3b;
    double W7 = rb + z3b;
    double W8 = y3 + a;
    double W9 = 1 + a / rb / cosB;
    double N1 = 1 - 2 * nu;
    double rb3 = cube(rb), rb5 = p5(rb), rb4 = sq(rb2);
    double cot2 = sq(cotB);

    double rFib_ry2 = z1b / rb / (rb + z3b) - y1 / rb / (rb + y3b);
    double rFib_ry1 = y2 / rb / (rb + y3b) - cosB * y2 / rb / (rb + z3b);
    double rFib_ry3 = -sinB * y2 / rb / (rb + z3b);

    const double K = 1.0 / 4;  // the 1/4 factor of every bracket
    // ---------------------------------------------------------------- v11
    v[0] =
        b1 * (K * ((-2 + 2 * nu) * N1 * rFib_ry1 * cot2 -
                   N1 * y2 / sq(W6) * ((1 - W5) * cotB - y1 / W6 * W4) / rb * y1 +
                   N1 * y2 / W6 * (a / rb3 * y1 * cotB - 1 / W6 * W4 + sq(y1) / sq(W6) * W4 / rb + sq(y1) / W6 * a / rb3) -
                   N1 * y2 * cosB * cotB / sq(W7) * W2 * (y1 / rb - sinB) -
                   N1 * y2 * cosB * cotB / W7 * a / rb3 * y1 - 3 * a * y2 * W8 * cotB / rb5 * y1 -
                   y2 * W8 / rb3 / W6 * (-N1 * cotB + y1 / W6 * W5 + a * y1 / rb2) * y1 -
                   y2 * W8 / rb2 / sq(W6) * (-N1 * cotB + y1 / W6 * W5 + a * y1 / rb2) * y1 +
                   y2 * W8 / rb / W6 * (1 / W6 * W5 - sq(y1) / sq(W6) * W5 / rb - sq(y1) / W6 * a / rb3 + a / rb2 - 2 * a * sq(y1) / rb4) -
                   y2 * W8 / rb3 / W7 * (cosB / W7 * (W1 * (N1 * cosB - a / rb) * cotB + (2 - 2 * nu) * (rb * sinB - y1) * cosB) - a * y3b * cosB * cotB / rb2) * y1 -
                   y2 * W8 / rb / sq(W7) * (cosB / W7 * (W1 * (N1 * cosB - a / rb) * cotB + (2 - 2 * nu) * (rb * sinB - y1) * cosB) - a * y3b * cosB * cotB / rb2) * (y1 / rb - sinB) +
                   y2 * W8 / rb / W7 * (-cosB / sq(W7) * (W1 * (N1 * cosB - a / rb) * cotB + (2 - 2 * nu) * (rb * sinB - y1) * cosB) * (y1 / rb - sinB) +
                                        cosB / W7 * (1 / rb * cosB * y1 * (N1 * cosB - a / rb) * cotB + W1 * a / rb3 * y1 * cotB + (2 - 2 * nu) * (1 / rb * sinB * y1 - 1) * cosB) +
                                        2 * a * y3b * cosB * cotB / rb4 * y1)) / pi / (1 - nu)) +
        b2 * (K * (N1 * (((2 - 2 * nu) * cot2 + nu) / rb * y1 / W6 - ((2 - 2 * nu) * cot2 + 1) * cosB * (y1 / rb - sinB) / W7) -
                   N1 / sq(W6) * (-N1 * y1 * cotB + nu * y3b - a + a * y1 * cotB / rb + sq(y1) / W6 * W4) / rb * y1 +
                   N1 / W6 * (-N1 * cotB + a * cotB / rb - a * sq(y1) * cotB / rb3 + 2 * y1 / W6 * W4 - cube(y1) / sq(W6) * W4 / rb - cube(y1) / W6 * a / rb3) +
                   N1 * cotB / sq(W7) * (z1b * cosB - a * (rb * sinB - y1) / rb / cosB) * (y1 / rb - sinB) -
                   N1 * cotB / W7 * (sq(cosB) - a * (1 / rb * sinB * y1 - 1) / rb / cosB + a * (rb * sinB - y1) / rb3 / cosB * y1) -
                   a * W8 * cotB / rb3 + 3 * a * sq(y1) * W8 * cotB / rb5 -
                   W8 / sq(W6) * (2 * nu + 1 / rb * (N1 * y1 * cotB + a) - sq(y1) / rb / W6 * W5 - a * sq(y1) / rb3) / rb * y1 +
                   W8 / W6 * (-1 / rb3 * (N1 * y1 * cotB + a) * y1 + 1 / rb * N1 * cotB - 2 * y1 / rb / W6 * W5 + cube(y1) / rb3 / W6 * W5 + cube(y1) / rb2 / sq(W6) * W5 + cube(y1) / rb4 / W6 * a - 2 * a / rb3 * y1 + 3 * a * cube(y1) / rb5) -
                   W8 * cotB / sq(W7) * (-cosB * sinB + a * y1 * y3b / rb3 / cosB + (rb * sinB - y1) / rb * ((2 - 2 * nu) * cosB - W1 / W7 * W9)) * (y1 / rb - sinB) +
                   W8 * cotB / W7 * (a * y3b / rb3 / cosB - 3 * a * sq(y1) * y3b / rb5 / cosB + (1 / rb * sinB * y1 - 1) / rb * ((2 - 2 * nu) * cosB - W1 / W7 * W9) -
                                     (rb * sinB - y1) / rb3 * ((2 - 2 * nu) * cosB - W1 / W7 * W9) * y1 +
                                     (rb * sinB - y1) / rb * (-1 / rb * cosB * y1 / W7 * W9 + W1 / sq(W7) * W9 * (y1 / rb - sinB) + W1 / W7 * a / rb3 / cosB * y1))) / pi / (1 - nu)) +
        b3 * (K * (N1 * (-y2 / sq(W6) * (1 + a / rb) / rb * y1 - y2 / W6 * a / rb3 * y1 + y2 * cosB / sq(W7) * W2 * (y1 / rb - sinB) + y2 * cosB / W7 * a / rb3 * y1) +
                   y2 * W8 / rb3 * (a / rb2 + 1 / W6) * y1 - y2 * W8 / rb * (-2 * a / rb4 * y1 - 1 / sq(W6) / rb * y1) -
                   y2 * W8 * cosB / rb3 / W7 * (W1 / W7 * W2 + a * y3b / rb2) * y1 -
                   y2 * W8 * cosB / rb / sq(W7) * (W1 / W7 * W2 + a * y3b / rb2) * (y1 / rb - sinB) +
                   y2 * W8 * cosB / rb / W7 * (1 / rb * cosB * y1 / W7 * W2 - W1 / sq(W7) * W2 * (y1 / rb - sinB) - W1 / W7 * a / rb3 * y1 - 2 * a * y3b / rb4 * y1)) / pi / (1 - nu));

    // ---------------------------------------------------------------- v22
    v[1] =
        b1 * (K * (N1 * (((2 - 2 * nu) * cot2 - nu) / rb * y2 / W6 - ((2 - 2 * nu) * cot2 + 1 - 2 * nu) * cosB / rb * y2 / W7) +
                   N1 / sq(W6) * (y1 * cotB * (1 - W5) + nu * y3b - a + sq(y2) / W6 * W4) / rb * y2 -
                   N1 / W6 * (a * y1 * cotB / rb3 * y2 + 2 * y2 / W6 * W4 - cube(y2) / sq(W6) * W4 / rb - cube(y2) / W6 * a / rb3) +
                   N1 * z1b * cotB / sq(W7) * W2 / rb * y2 + N1 * z1b * cotB / W7 * a / rb3 * y2 + 3 * a * y2 * W8 * cotB / rb5 * y1 -
                   W8 / sq(W6) * (-2 * nu + 1 / rb * (N1 * y1 * cotB - a) + sq(y2) / rb / W6 * W5 + a * sq(y2) / rb3) / rb * y2 +
                   W8 / W6 * (-1 / rb3 * (N1 * y1 * cotB - a) * y2 + 2 * y2 / rb / W6 * W5 - cube(y2) / rb3 / W6 * W5 - cube(y2) / rb2 / sq(W6) * W5 - cube(y2) / rb4 / W6 * a + 2 * a / rb3 * y2 - 3 * a * cube(y2) / rb5) -
                   W8 / sq(W7) * (sq(cosB) - 1 / rb * (N1 * z1b * cotB + a * cosB) + a * y3b * z1b * cotB / rb3 - 1 / rb / W7 * (sq(y2) * sq(cosB) - a * z1b * cotB / rb * W1)) / rb * y2 +
                   W8 / W7 * (1 / rb3 * (N1 * z1b * cotB + a * cosB) * y2 - 3 * a * y3b * z1b * cotB / rb5 * y2 + 1 / rb3 / W7 * (sq(y2) * sq(cosB) - a * z1b * cotB / rb * W1) * y2 +
                              1 / rb2 / sq(W7) * (sq(y2) * sq(cosB) - a * z1b * cotB / rb * W1) * y2 -
                              1 / rb / W7 * (2 * y2 * sq(cosB) + a * z1b * cotB / rb3 * W1 * y2 - a * z1b * cotB / rb2 * cosB * y2))) / pi / (1 - nu)) +
        b2 * (K * ((2 - 2 * nu) * N1 * rFib_ry2 * cot2 + N1 / W6 * ((W5 - 1) * cotB + y1 / W6 * W4) -
                   N1 * sq(y2) / sq(W6) * ((W5 - 1) * cotB + y1 / W6 * W4) / rb +
                   N1 * y2 / W6 * (-a / rb3 * y2 * cotB - y1 / sq(W6) * W4 / rb * y2 - y2 / W6 * a / rb3 * y1) -
                   N1 * cotB / W7 * W9 + N1 * sq(y2) * cotB / sq(W7) * W9 / rb + N1 * sq(y2) * cotB / W7 * a / rb3 / cosB -
                   a * W8 * cotB / rb3 + 3 * a * sq(y2) * W8 * cotB / rb5 +
                   W8 / rb / W6 * (N1 * cotB - 2 * nu * y1 / W6 - a * y1 / rb * (1 / rb + 1 / W6)) -
                   sq(y2) * W8 / rb3 / W6 * (N1 * cotB - 2 * nu * y1 / W6 - a * y1 / rb * (1 / rb + 1 / W6)) -
                   sq(y2) * W8 / rb2 / sq(W6) * (N1 * cotB - 2 * nu * y1 / W6 - a * y1 / rb * (1 / rb + 1 / W6)) +
                   y2 * W8 / rb / W6 * (2 * nu * y1 / sq(W6) / rb * y2 + a * y1 / rb3 * (1 / rb + 1 / W6) * y2 - a * y1 / rb * (-1 / rb3 * y2 - 1 / sq(W6) / rb * y2)) +
                   W8 * cotB / rb / W7 * ((-2 + 2 * nu) * cosB + W1 / W7 * W9 + a * y3b / rb2 / cosB) -
                   sq(y2) * W8 * cotB / rb3 / W7 * ((-2 + 2 * nu) * cosB + W1 / W7 * W9 + a * y3b / rb2 / cosB) -
                   sq(y2) * W8 * cotB / rb2 / sq(W7) * ((-2 + 2 * nu) * cosB + W1 / W7 * W9 + a * y3b / rb2 / cosB) +
                   y2 * W8 * cotB / rb / W7 * (1 / rb * cosB * y2 / W7 * W9 - W1 / sq(W7) * W9 / rb * y2 - W1 / W7 * a / rb3 / cosB * y2 - 2 * a * y3b / rb4 / cosB * y2)) / pi / (1 - nu)) +
        b3 * (K * (N1 * (-sinB / rb * y2 / W7 + y2 / sq(W6) * (1 + a / rb) / rb * y1 + y2 / W6 * a / rb3 * y1 - z1b / sq(W7) * W2 / rb * y2 - z1b / W7 * a / rb3 * y2) -
                   y2 * W8 / rb3 * (a / rb2 + 1 / W6) * y1 + y1 * W8 / rb * (-2 * a / rb4 * y2 - 1 / sq(W6) / rb * y2) +
                   W8 / sq(W7) * (sinB * (cosB - a / rb) + z1b / rb * (1 + a * y3b / rb2) - 1 / rb / W7 * (sq(y2) * cosB * sinB - a * z1b / rb * W1)) / rb * y2 -
                   W8 / W7 * (sinB * a / rb3 * y2 - z1b / rb3 * (1 + a * y3b / rb2) * y2 - 2 * z1b / rb5 * a * y3b * y2 +
                              1 / rb3 / W7 * (sq(y2) * cosB * sinB - a * z1b / rb * W1) * y2 +
                              1 / rb2 / sq(W7) * (sq(y2) * cosB * sinB - a * z1b / rb * W1) * y2 -
                              1 / rb / W7 * (2 * y2 * cosB * sinB + a * z1b / rb3 * W1 * y2 - a * z1b / rb2 * cosB * y2))) / pi / (1 - nu));

    // ---------------------------------------------------------------- v33
    v[2] =
        b1 * (K * ((2 - 2 * nu) * (N1 * rFib_ry3 * cotB - y2 / sq(W6) * W5 * (y3b / rb + 1) - 0.5 * y2 / W6 * a / rb3 * 2 * y3b + y2 * cosB / sq(W7) * W2 * W3 + 0.5 * y2 * cosB / W7 * a / rb3 * 2 * y3b) +
                   y2 / rb * (2 * nu / W6 + a / rb2) - 0.5 * y2 * W8 / rb3 * (2 * nu / W6 + a / rb2) * 2 * y3b +
                   y2 * W8 / rb * (-2 * nu / sq(W6) * (y3b / rb + 1) - a / rb4 * 2 * y3b) +
                   y2 * cosB / rb / W7 * (1 - 2 * nu - W1 / W7 * W2 - a * y3b / rb2) -
                   0.5 * y2 * W8 * cosB / rb3 / W7 * (1 - 2 * nu - W1 / W7 * W2 - a * y3b / rb2) * 2 * y3b -
                   y2 * W8 * cosB / rb / sq(W7) * (1 - 2 * nu - W1 / W7 * W2 - a * y3b / rb2) * W3 +
                   y2 * W8 * cosB / rb / W7 * (-(cosB * y3b / rb + 1) / W7 * W2 + W1 / sq(W7) * W2 * W3 + 0.5 * W1 / W7 * a / rb3 * 2 * y3b - a / rb2 + a * y3b / rb4 * 2 * y3b)) / pi / (1 - nu)) +
        b2 * (K * ((-2 + 2 * nu) * N1 * cotB * ((y3b / rb + 1) / W6 - cosB * W3 / W7) + (2 - 2 * nu) * y1 / sq(W6) * W5 * (y3b / rb + 1) +
                   0.5 * (2 - 2 * nu) * y1 / W6 * a / rb3 * 2 * y3b + (2 - 2 * nu) * sinB / W7 * W2 - (2 - 2 * nu) * z1b / sq(W7) * W2 * W3 -
                   0.5 * (2 - 2 * nu) * z1b / W7 * a / rb3 * 2 * y3b + 1 / rb * (N1 * cotB - 2 * nu * y1 / W6 - a * y1 / rb2) -
                   0.5 * W8 / rb3 * (N1 * cotB - 2 * nu * y1 / W6 - a * y1 / rb2) * 2 * y3b +
                   W8 / rb * (2 * nu * y1 / sq(W6) * (y3b / rb + 1) + a * y1 / rb4 * 2 * y3b) -
                   1 / W7 * (cosB * sinB + W1 * cotB / rb * ((2 - 2 * nu) * cosB - W1 / W7) + a / rb * (sinB - y3b * z1b / rb2 - z1b * W1 / rb / W7)) +
                   W8 / sq(W7) * (cosB * sinB + W1 * cotB / rb * ((2 - 2 * nu) * cosB - W1 / W7) + a / rb * (sinB - y3b * z1b / rb2 - z1b * W1 / rb / W7)) * W3 -
                   W8 / W7 * ((cosB * y3b / rb + 1) * cotB / rb * ((2 - 2 * nu) * cosB - W1 / W7) - 0.5 * W1 * cotB / rb3 * ((2 - 2 * nu) * cosB - W1 / W7) * 2 * y3b +
                              W1 * cotB / rb * (-(cosB * y3b / rb + 1) / W7 + W1 / sq(W7) * W3) - 0.5 * a / rb3 * (sinB - y3b * z1b / rb2 - z1b * W1 / rb / W7) * 2 * y3b +
                              a / rb * (-z1b / rb2 - y3b * sinB / rb2 + y3b * z1b / rb4 * 2 * y3b - sinB * W1 / rb / W7 - z1b * (cosB * y3b / rb + 1) / rb / W7 +
                                        0.5 * z1b * W1 / rb3 / W7 * 2 * y3b + z1b * W1 / rb / sq(W7) * W3))) / pi / (1 - nu)) +
        b3 * (K * ((2 - 2 * nu) * rFib_ry3 - (2 - 2 * nu) * y2 * sinB / sq(W7) * W2 * W3 - 0.5 * (2 - 2 * nu) * y2 * sinB / W7 * a / rb3 * 2 * y3b +
                   y2 * sinB / rb / W7 * (1 + W1 / W7 * W2 + a * y3b / rb2) -
                   0.5 * y2 * W8 * sinB / rb3 / W7 * (1 + W1 / W7 * W2 + a * y3b / rb2) * 2 * y3b -
                   y2 * W8 * sinB / rb / sq(W7) * (1 + W1 / W7 * W2 + a * y3b / rb2) * W3 +
                   y2 * W8 * sinB / rb / W7 * ((cosB * y3b / rb + 1) / W7 * W2 - W1 / sq(W7) * W2 * W3 - 0.5 * W1 / W7 * a / rb3 * 2 * y3b + a / rb2 - a * y3b / rb4 * 2 * y3b)) / pi / (1 - nu));

    // ---------------------------------------------------------------- v12
    v[3] =
        b1 / 2 * (K * ((-2 + 2 * nu) * N1 * rFib_ry2 * cot2 + N1 / W6 * ((1 - W5) * cotB - y1 / W6 * W4) -
                       N1 * sq(y2) / sq(W6) * ((1 - W5) * cotB - y1 / W6 * W4) / rb +
                       N1 * y2 / W6 * (a / rb3 * y2 * cotB + y1 / sq(W6) * W4 / rb * y2 + y2 / W6 * a / rb3 * y1) +
                       N1 * cosB * cotB / W7 * W2 - N1 * sq(y2) * cosB * cotB / sq(W7) * W2 / rb - N1 * sq(y2) * cosB * cotB / W7 * a / rb3 +
                       a * W8 * cotB / rb3 - 3 * a * sq(y2) * W8 * cotB / rb5 +
                       W8 / rb / W6 * (-N1 * cotB + y1 / W6 * W5 + a * y1 / rb2) -
                       sq(y2) * W8 / rb3 / W6 * (-N1 * cotB + y1 / W6 * W5 + a * y1 / rb2) -
                       sq(y2) * W8 / rb2 / sq(W6) * (-N1 * cotB + y1 / W6 * W5 + a * y1 / rb2) +
                       y2 * W8 / rb / W6 * (-y1 / sq(W6) * W5 / rb * y2 - y2 / W6 * a / rb3 * y1 - 2 * a * y1 / rb4 * y2) +
                       W8 / rb / W7 * (cosB / W7 * (W1 * (N1 * cosB - a / rb) * cotB + (2 - 2 * nu) * (rb * sinB - y1) * cosB) - a * y3b * cosB * cotB / rb2) -
                       sq(y2) * W8 / rb3 / W7 * (cosB / W7 * (W1 * (N1 * cosB - a / rb) * cotB + (2 - 2 * nu) * (rb * sinB - y1) * cosB) - a * y3b * cosB * cotB / rb2) -
                       sq(y2) * W8 / rb2 / sq(W7) * (cosB / W7 * (W1 * (N1 * cosB - a / rb) * cotB + (2 - 2 * nu) * (rb * sinB - y1) * cosB) - a * y3b * cosB * cotB / rb2) +
                       y2 * W8 / rb / W7 * (-cosB / sq(W7) * (W1 * (N1 * cosB - a / rb) * cotB + (2 - 2 * nu) * (rb * sinB - y1) * cosB) / rb * y2 +
                                            cosB / W7 * (1 / rb * cosB * y2 * (N1 * cosB - a / rb) * cotB + W1 * a / rb3 * y2 * cotB + (2 - 2 * nu) / rb * sinB * y2 * cosB) +
                                            2 * a * y3b * cosB * cotB / rb4 * y2)) / pi / (1 - nu)) +
        b2 / 2 * (K * (N1 * (((2 - 2 * nu) * cot2 + nu) / rb * y2 / W6 - ((2 - 2 * nu) * cot2 + 1) * cosB / rb * y2 / W7) -
                       N1 / sq(W6) * (-N1 * y1 * cotB + nu * y3b - a + a * y1 * cotB / rb + sq(y1) / W6 * W4) / rb * y2 +
                       N1 / W6 * (-a * y1 * cotB / rb3 * y2 - sq(y1) / sq(W6) * W4 / rb * y2 - sq(y1) / W6 * a / rb3 * y2) +
                       N1 * cotB / sq(W7) * (z1b * cosB - a * (rb * sinB - y1) / rb / cosB) / rb * y2 -
                       N1 * cotB / W7 * (-a / rb2 * sinB * y2 / cosB + a * (rb * sinB - y1) / rb3 / cosB * y2) +
                       3 * a * y2 * W8 * cotB / rb5 * y1 -
                       W8 / sq(W6) * (2 * nu + 1 / rb * (N1 * y1 * cotB + a) - sq(y1) / rb / W6 * W5 - a * sq(y1) / rb3) / rb * y2 +
                       W8 / W6 * (-1 / rb3 * (N1 * y1 * cotB + a) * y2 + sq(y1) / rb3 / W6 * W5 * y2 + sq(y1) / rb2 / sq(W6) * W5 * y2 + sq(y1) / rb4 / W6 * a * y2 + 3 * a * sq(y1) / rb5 * y2) -
                       W8 * cotB / sq(W7) * (-cosB * sinB + a * y1 * y3b / rb3 / cosB + (rb * sinB - y1) / rb * ((2 - 2 * nu) * cosB - W1 / W7 * W9)) / rb * y2 +
                       W8 * cotB / W7 * (-3 * a * y1 * y3b / rb5 / cosB * y2 + 1 / rb2 * sinB * y2 * ((2 - 2 * nu) * cosB - W1 / W7 * W9) -
                                         (rb * sinB - y1) / rb3 * ((2 - 2 * nu) * cosB - W1 / W7 * W9) * y2 +
                                         (rb * sinB - y1) / rb * (-1 / rb * cosB * y2 / W7 * W9 + W1 / sq(W7) * W9 / rb * y2 + W1 / W7 * a / rb3 / cosB * y2))) / pi / (1 - nu)) +
        b3 / 2 * (K * (N1 * (1 / W6 * (1 + a / rb) - sq(y2) / sq(W6) * (1 + a / rb) / rb - sq(y2) / W6 * a / rb3 - cosB / W7 * W2 + sq(y2) * cosB / sq(W7) * W2 / rb + sq(y2) * cosB / W7 * a / rb3) -
                       W8 / rb * (a / rb2 + 1 / W6) + sq(y2) * W8 / rb3 * (a / rb2 + 1 / W6) -
                       y2 * W8 / rb * (-2 * a / rb4 * y2 - 1 / sq(W6) / rb * y2) +
                       W8 * cosB / rb / W7 * (W1 / W7 * W2 + a * y3b / rb2) -
                       sq(y2) * W8 * cosB / rb3 / W7 * (W1 / W7 * W2 + a * y3b / rb2) -
                       sq(y2) * W8 * cosB / rb2 / sq(W7) * (W1 / W7 * W2 + a * y3b / rb2) +
                       y2 * W8 * cosB / rb / W7 * (1 / rb * cosB * y2 / W7 * W2 - W1 / sq(W7) * W2 / rb * y2 - W1 / W7 * a / rb3 * y2 - 2 * a * y3b / rb4 * y2)) / pi / (1 - nu)) +
        b1 / 2 * (K * (N1 * (((2 - 2 * nu) * cot2 - nu) / rb * y1 / W6 - ((2 - 2 * nu) * cot2 + 1 - 2 * nu) * cosB * (y1 / rb - sinB) / W7) +
                       N1 / sq(W6) * (y1 * cotB * (1 - W5) + nu * y3b - a + sq(y2) / W6 * W4) / rb * y1 -
                       N1 / W6 * ((1 - W5) * cotB + a * sq(y1) * cotB / rb3 - sq(y2) / sq(W6) * W4 / rb * y1 - sq(y2) / W6 * a / rb3 * y1) -
                       N1 * cosB * cotB / W7 * W2 + N1 * z1b * cotB / sq(W7) * W2 * (y1 / rb - sinB) + N1 * z1b * cotB / W7 * a / rb3 * y1 -
                       a * W8 * cotB / rb3 + 3 * a * sq(y1) * W8 * cotB / rb5 -
                       W8 / sq(W6) * (-2 * nu + 1 / rb * (N1 * y1 * cotB - a) + sq(y2) / rb / W6 * W5 + a * sq(y2) / rb3) / rb * y1 +
                       W8 / W6 * (-1 / rb3 * (N1 * y1 * cotB - a) * y1 + 1 / rb * N1 * cotB - sq(y2) / rb3 / W6 * W5 * y1 - sq(y2) / rb2 / sq(W6) * W5 * y1 - sq(y2) / rb4 / W6 * a * y1 - 3 * a * sq(y2) / rb5 * y1) -
                       W8 / sq(W7) * (sq(cosB) - 1 / rb * (N1 * z1b * cotB + a * cosB) + a * y3b * z1b * cotB / rb3 - 1 / rb / W7 * (sq(y2) * sq(cosB) - a * z1b * cotB / rb * W1)) * (y1 / rb - sinB) +
                       W8 / W7 * (1 / rb3 * (N1 * z1b * cotB + a * cosB) * y1 - 1 / rb * N1 * cosB * cotB + a * y3b * cosB * cotB / rb3 - 3 * a * y3b * z1b * cotB / rb5 * y1 +
                                  1 / rb3 / W7 * (sq(y2) * sq(cosB) - a * z1b * cotB / rb * W1) * y1 +
                                  1 / rb / sq(W7) * (sq(y2) * sq(cosB) - a * z1b * cotB / rb * W1) * (y1 / rb - sinB) -
                                  1 / rb / W7 * (-a * cosB * cotB / rb * W1 + a * z1b * cotB / rb3 * W1 * y1 - a * z1b * cotB / rb2 * cosB * y1))) / pi / (1 - nu)) +
        b2 / 2 * (K * ((2 - 2 * nu) * N1 * rFib_ry1 * cot2 - N1 * y2 / sq(W6) * ((W5 - 1) * cotB + y1 / W6 * W4) / rb * y1 +
                       N1 * y2 / W6 * (-a / rb3 * y1 * cotB + 1 / W6 * W4 - sq(y1) / sq(W6) * W4 / rb - sq(y1) / W6 * a / rb3) +
                       N1 * y2 * cotB / sq(W7) * W9 * (y1 / rb - sinB) + N1 * y2 * cotB / W7 * a / rb3 / cosB * y1 +
                       3 * a * y2 * W8 * cotB / rb5 * y1 -
                       y2 * W8 / rb3 / W6 * (N1 * cotB - 2 * nu * y1 / W6 - a * y1 / rb * (1 / rb + 1 / W6)) * y1 -
                       y2 * W8 / rb2 / sq(W6) * (N1 * cotB - 2 * nu * y1 / W6 - a * y1 / rb * (1 / rb + 1 / W6)) * y1 +
                       y2 * W8 / rb / W6 * (-2 * nu / W6 + 2 * nu * sq(y1) / sq(W6) / rb - a / rb * (1 / rb + 1 / W6) + a * sq(y1) / rb3 * (1 / rb + 1 / W6) - a * y1 / rb * (-1 / rb3 * y1 - 1 / sq(W6) / rb * y1)) -
                       y2 * W8 * cotB / rb3 / W7 * ((-2 + 2 * nu) * cosB + W1 / W7 * W9 + a * y3b / rb2 / cosB) * y1 -
                       y2 * W8 * cotB / rb / sq(W7) * ((-2 + 2 * nu) * cosB + W1 / W7 * W9 + a * y3b / rb2 / cosB) * (y1 / rb - sinB) +
                       y2 * W8 * cotB / rb / W7 * (1 / rb * cosB * y1 / W7 * W9 - W1 / sq(W7) * W9 * (y1 / rb - sinB) - W1 / W7 * a / rb3 / cosB * y1 - 2 * a * y3b / rb4 / cosB * y1)) / pi / (1 - nu)) +
        b3 / 2 * (K * (N1 * (-sinB * (y1 / rb - sinB) / W7 - 1 / W6 * (1 + a / rb) + sq(y1) / sq(W6) * (1 + a / rb) / rb + sq(y1) / W6 * a / rb3 + cosB / W7 * W2 - z1b / sq(W7) * W2 * (y1 / rb - sinB) - z1b / W7 * a / rb3 * y1) +
                       W8 / rb * (a / rb2 + 1 / W6) - sq(y1) * W8 / rb3 * (a / rb2 + 1 / W6) + y1 * W8 / rb * (-2 * a / rb4 * y1 - 1 / sq(W6) / rb * y1) +
                       W8 / sq(W7) * (sinB * (cosB - a / rb) + z1b / rb * (1 + a * y3b / rb2) - 1 / rb / W7 * (sq(y2) * cosB * sinB - a * z1b / rb * W1)) * (y1 / rb - sinB) -
                       W8 / W7 * (sinB * a / rb3 * y1 + cosB / rb * (1 + a * y3b / rb2) - z1b / rb3 * (1 + a * y3b / rb2) * y1 - 2 * z1b / rb5 * a * y3b * y1 +
                                  1 / rb3 / W7 * (sq(y2) * cosB * sinB - a * z1b / rb * W1) * y1 +
                                  1 / rb / sq(W7) * (sq(y2) * cosB * sinB - a * z1b / rb * W1) * (y1 / rb - sinB) -
                                  1 / rb / W7 * (-a * cosB / rb * W1 + a * z1b / rb3 * W1 * y1 - a * z1b / rb2 * cosB * y1))) / pi / (1 - nu));

    // ---------------------------------------------------------------- v13
    v[4] =
        b1 / 2 * (K * ((-2 + 2 * nu) * N1 * rFib_ry3 * cot2 - N1 * y2 / sq(W6) * ((1 - W5) * cotB - y1 / W6 * W4) * (y3b / rb + 1) +
                       N1 * y2 / W6 * (0.5 * a / rb3 * 2 * y3b * cotB + y1 / sq(W6) * W4 * (y3b / rb + 1) + 0.5 * y1 / W6 * a / rb3 * 2 * y3b) -
                       N1 * y2 * cosB * cotB / sq(W7) * W2 * W3 - 0.5 * N1 * y2 * cosB * cotB / W7 * a / rb3 * 2 * y3b +
                       a / rb3 * y2 * cotB - 1.5 * a * y2 * W8 * cotB / rb5 * 2 * y3b +
                       y2 / rb / W6 * (-N1 * cotB + y1 / W6 * W5 + a * y1 / rb2) -
                       0.5 * y2 * W8 / rb3 / W6 * (-N1 * cotB + y1 / W6 * W5 + a * y1 / rb2) * 2 * y3b -
                       y2 * W8 / rb / sq(W6) * (-N1 * cotB + y1 / W6 * W5 + a * y1 / rb2) * (y3b / rb + 1) +
                       y2 * W8 / rb / W6 * (-y1 / sq(W6) * W5 * (y3b / rb + 1) - 0.5 * y1 / W6 * a / rb3 * 2 * y3b - a * y1 / rb4 * 2 * y3b) +
                       y2 / rb / W7 * (cosB / W7 * (W1 * (N1 * cosB - a / rb) * cotB + (2 - 2 * nu) * (rb * sinB - y1) * cosB) - a * y3b * cosB * cotB / rb2) -
                       0.5 * y2 * W8 / rb3 / W7 * (cosB / W7 * (W1 * (N1 * cosB - a / rb) * cotB + (2 - 2 * nu) * (rb * sinB - y1) * cosB) - a * y3b * cosB * cotB / rb2) * 2 * y3b -
                       y2 * W8 / rb / sq(W7) * (cosB / W7 * (W1 * (N1 * cosB - a / rb) * cotB + (2 - 2 * nu) * (rb * sinB - y1) * cosB) - a * y3b * cosB * cotB / rb2) * W3 +
                       y2 * W8 / rb / W7 * (-cosB / sq(W7) * (W1 * (N1 * cosB - a / rb) * cotB + (2 - 2 * nu) * (rb * sinB - y1) * cosB) * W3 +
                                            cosB / W7 * ((cosB * y3b / rb + 1) * (N1 * cosB - a / rb) * cotB + 0.5 * W1 * a / rb3 * 2 * y3b * cotB + 0.5 * (2 - 2 * nu) / rb * sinB * 2 * y3b * cosB) -
                                            a * cosB * cotB / rb2 + a * y3b * cosB * cotB / rb4 * 2 * y3b)) / pi / (1 - nu)) +
        b2 / 2 * (K * (N1 * (((2 - 2 * nu) * cot2 + nu) * (y3b / rb + 1) / W6 - ((2 - 2 * nu) * cot2 + 1) * cosB * W3 / W7) -
                       N1 / sq(W6) * (-N1 * y1 * cotB + nu * y3b - a + a * y1 * cotB / rb + sq(y1) / W6 * W4) * (y3b / rb + 1) +
                       N1 / W6 * (nu - 0.5 * a * y1 * cotB / rb3 * 2 * y3b - sq(y1) / sq(W6) * W4 * (y3b / rb + 1) - 0.5 * sq(y1) / W6 * a / rb3 * 2 * y3b) +
                       N1 * cotB / sq(W7) * (z1b * cosB - a * (rb * sinB - y1) / rb / cosB) * W3 -
                       N1 * cotB / W7 * (cosB * sinB - 0.5 * a / rb2 * sinB * 2 * y3b / cosB + 0.5 * a * (rb * sinB - y1) / rb3 / cosB * 2 * y3b) -
                       a / rb3 * y1 * cotB + 1.5 * a * y1 * W8 * cotB / rb5 * 2 * y3b +
                       1 / W6 * (2 * nu + 1 / rb * (N1 * y1 * cotB + a) - sq(y1) / rb / W6 * W5 - a * sq(y1) / rb3) -
                       W8 / sq(W6) * (2 * nu + 1 / rb * (N1 * y1 * cotB + a) - sq(y1) / rb / W6 * W5 - a * sq(y1) / rb3) * (y3b / rb + 1) +
                       W8 / W6 * (-0.5 / rb3 * (N1 * y1 * cotB + a) * 2 * y3b + 0.5 * sq(y1) / rb3 / W6 * W5 * 2 * y3b + sq(y1) / rb / sq(W6) * W5 * (y3b / rb + 1) +
                                  0.5 * sq(y1) / rb4 / W6 * a * 2 * y3b + 1.5 * a * sq(y1) / rb5 * 2 * y3b) +
                       cotB / W7 * (-cosB * sinB + a * y1 * y3b / rb3 / cosB + (rb * sinB - y1) / rb * ((2 - 2 * nu) * cosB - W1 / W7 * W9)) -
                       W8 * cotB / sq(W7) * (-cosB * sinB + a * y1 * y3b / rb3 / cosB + (rb * sinB - y1) / rb * ((2 - 2 * nu) * cosB - W1 / W7 * W9)) * W3 +
                       W8 * cotB / W7 * (a / rb3 / cosB * y1 - 1.5 * a * y1 * y3b / rb5 / cosB * 2 * y3b + 0.5 / rb2 * sinB * 2 * y3b * ((2 - 2 * nu) * cosB - W1 / W7 * W9) -
                                         0.5 * (rb * sinB - y1) / rb3 * ((2 - 2 * nu) * cosB - W1 / W7 * W9) * 2 * y3b +
                                         (rb * sinB - y1) / rb * (-(cosB * y3b / rb + 1) / W7 * W9 + W1 / sq(W7) * W9 * W3 + 0.5 * W1 / W7 * a / rb3 / cosB * 2 * y3b))) / pi / (1 - nu)) +
        b3 / 2 * (K * (N1 * (-y2 / sq(W6) * (1 + a / rb) * (y3b / rb + 1) - 0.5 * y2 / W6 * a / rb3 * 2 * y3b + y2 * cosB / sq(W7) * W2 * W3 + 0.5 * y2 * cosB / W7 * a / rb3 * 2 * y3b) -
                       y2 / rb * (a / rb2 + 1 / W6) + 0.5 * y2 * W8 / rb3 * (a / rb2 + 1 / W6) * 2 * y3b -
                       y2 * W8 / rb * (-a / rb4 * 2 * y3b - 1 / sq(W6) * (y3b / rb + 1)) +
                       y2 * cosB / rb / W7 * (W1 / W7 * W2 + a * y3b / rb2) -
                       0.5 * y2 * W8 * cosB / rb3 / W7 * (W1 / W7 * W2 + a * y3b / rb2) * 2 * y3b -
                       y2 * W8 * cosB / rb / sq(W7) * (W1 / W7 * W2 + a * y3b / rb2) * W3 +
                       y2 * W8 * cosB / rb / W7 * ((cosB * y3b / rb + 1) / W7 * W2 - W1 / sq(W7) * W2 * W3 - 0.5 * W1 / W7 * a / rb3 * 2 * y3b + a / rb2 - a * y3b / rb4 * 2 * y3b)) / pi / (1 - nu)) +
        b1 / 2 * (K * ((2 - 2 * nu) * (N1 * rFib_ry1 * cotB - y1 / sq(W6) * W5 / rb * y2 - y2 / W6 * a / rb3 * y1 + y2 * cosB / sq(W7) * W2 * (y1 / rb - sinB) + y2 * cosB / W7 * a / rb3 * y1) -
                       y2 * W8 / rb3 * (2 * nu / W6 + a / rb2) * y1 + y2 * W8 / rb * (-2 * nu / sq(W6) / rb * y1 - 2 * a / rb4 * y1) -
                       y2 * W8 * cosB / rb3 / W7 * (1 - 2 * nu - W1 / W7 * W2 - a * y3b / rb2) * y1 -
                       y2 * W8 * cosB / rb / sq(W7) * (1 - 2 * nu - W1 / W7 * W2 - a * y3b / rb2) * (y1 / rb - sinB) +
                       y2 * W8 * cosB / rb / W7 * (-1 / rb * cosB * y1 / W7 * W2 + W1 / sq(W7) * W2 * (y1 / rb - sinB) + W1 / W7 * a / rb3 * y1 + 2 * a * y3b / rb4 * y1)) / pi / (1 - nu)) +
        b2 / 2 * (K * ((-2 + 2 * nu) * N1 * cotB * (1 / rb * y1 / W6 - cosB * (y1 / rb - sinB) / W7) - (2 - 2 * nu) / W6 * W5 + (2 - 2 * nu) * sq(y1) / sq(W6) * W5 / rb +
                       (2 - 2 * nu) * sq(y1) / W6 * a / rb3 + (2 - 2 * nu) * cosB / W7 * W2 - (2 - 2 * nu) * z1b / sq(W7) * W2 * (y1 / rb - sinB) -
                       (2 - 2 * nu) * z1b / W7 * a / rb3 * y1 - W8 / rb3 * (N1 * cotB - 2 * nu * y1 / W6 - a * y1 / rb2) * y1 +
                       W8 / rb * (-2 * nu / W6 + 2 * nu * sq(y1) / sq(W6) / rb - a / rb2 + 2 * a * sq(y1) / rb4) +
                       W8 / sq(W7) * (cosB * sinB + W1 * cotB / rb * ((2 - 2 * nu) * cosB - W1 / W7) + a / rb * (sinB - y3b * z1b / rb2 - z1b * W1 / rb / W7)) * (y1 / rb - sinB) -
                       W8 / W7 * (1 / rb2 * cosB * y1 * cotB * ((2 - 2 * nu) * cosB - W1 / W7) - W1 * cotB / rb3 * ((2 - 2 * nu) * cosB - W1 / W7) * y1 +
                                  W1 * cotB / rb * (-1 / rb * cosB * y1 / W7 + W1 / sq(W7) * (y1 / rb - sinB)) - a / rb3 * (sinB - y3b * z1b / rb2 - z1b * W1 / rb / W7) * y1 +
                                  a / rb * (-y3b * cosB / rb2 + 2 * y3b * z1b / rb4 * y1 - cosB * W1 / rb / W7 - z1b / rb2 * cosB * y1 / W7 + z1b * W1 / rb3 / W7 * y1 +
                                            z1b * W1 / rb / sq(W7) * (y1 / rb - sinB)))) / pi / (1 - nu)) +
        b3 / 2 * (K * ((2 - 2 * nu) * rFib_ry1 - (2 - 2 * nu) * y2 * sinB / sq(W7) * W2 * (y1 / rb - sinB) - (2 - 2 * nu) * y2 * sinB / W7 * a / rb3 * y1 -
                       y2 * W8 * sinB / rb3 / W7 * (1 + W1 / W7 * W2 + a * y3b / rb2) * y1 -
                       y2 * W8 * sinB / rb / sq(W7) * (1 + W1 / W7 * W2 + a * y3b / rb2) * (y1 / rb - sinB) +
                       y2 * W8 * sinB / rb / W7 * (1 / rb * cosB * y1 / W7 * W2 - W1 / sq(W7) * W2 * (y1 / rb - sinB) - W1 / W7 * a / rb3 * y1 - 2 * a * y3b / rb4 * y1)) / pi / (1 - nu));

    // ---------------------------------------------------------------- v23
    v[5] =
        b1 / 2 * (K * (N1 * (((2 - 2 * nu) * cot2 - nu) * (y3b / rb + 1) / W6 - ((2 - 2 * nu) * cot2 + 1 - 2 * nu) * cosB * W3 / W7) +
                       N1 / sq(W6) * (y1 * cotB * (1 - W5) + nu * y3b - a + sq(y2) / W6 * W4) * (y3b / rb + 1) -
                       N1 / W6 * (0.5 * a * y1 * cotB / rb3 * 2 * y3b + nu - sq(y2) / sq(W6) * W4 * (y3b / rb + 1) - 0.5 * sq(y2) / W6 * a / rb3 * 2 * y3b) -
                       N1 * sinB * cotB / W7 * W2 + N1 * z1b * cotB / sq(W7) * W2 * W3 + 0.5 * N1 * z1b * cotB / W7 * a / rb3 * 2 * y3b -
                       a / rb3 * y1 * cotB + 1.5 * a * y1 * W8 * cotB / rb5 * 2 * y3b +
                       1 / W6 * (-2 * nu + 1 / rb * (N1 * y1 * cotB - a) + sq(y2) / rb / W6 * W5 + a * sq(y2) / rb3) -
                       W8 / sq(W6) * (-2 * nu + 1 / rb * (N1 * y1 * cotB - a) + sq(y2) / rb / W6 * W5 + a * sq(y2) / rb3) * (y3b / rb + 1) +
                       W8 / W6 * (-0.5 / rb3 * (N1 * y1 * cotB - a) * 2 * y3b - 0.5 * sq(y2) / rb3 / W6 * W5 * 2 * y3b - sq(y2) / rb / sq(W6) * W5 * (y3b / rb + 1) -
                                  0.5 * sq(y2) / rb4 / W6 * a * 2 * y3b - 1.5 * a * sq(y2) / rb5 * 2 * y3b) +
                       1 / W7 * (sq(cosB) - 1 / rb * (N1 * z1b * cotB + a * cosB) + a * y3b * z1b * cotB / rb3 - 1 / rb / W7 * (sq(y2) * sq(cosB) - a * z1b * cotB / rb * W1)) -
                       W8 / sq(W7) * (sq(cosB) - 1 / rb * (N1 * z1b * cotB + a * cosB) + a * y3b * z1b * cotB / rb3 - 1 / rb / W7 * (sq(y2) * sq(cosB) - a * z1b * cotB / rb * W1)) * W3 +
                       W8 / W7 * (0.5 / rb3 * (N1 * z1b * cotB + a * cosB) * 2 * y3b - 1 / rb * N1 * sinB * cotB + a * z1b * cotB / rb3 + a * y3b * sinB * cotB / rb3 -
                                  1.5 * a * y3b * z1b * cotB / rb5 * 2 * y3b + 0.5 / rb3 / W7 * (sq(y2) * sq(cosB) - a * z1b * cotB / rb * W1) * 2 * y3b +
                                  1 / rb / sq(W7) * (sq(y2) * sq(cosB) - a * z1b * cotB / rb * W1) * W3 -
                                  1 / rb / W7 * (-a * sinB * cotB / rb * W1 + 0.5 * a * z1b * cotB / rb3 * W1 * 2 * y3b - a * z1b * cotB / rb * (cosB * y3b / rb + 1)))) / pi / (1 - nu)) +
        b2 / 2 * (K * ((2 - 2 * nu) * N1 * rFib_ry3 * cot2 - N1 * y2 / sq(W6) * ((W5 - 1) * cotB + y1 / W6 * W4) * (y3b / rb + 1) +
                       N1 * y2 / W6 * (-0.5 * a / rb3 * 2 * y3b * cotB - y1 / sq(W6) * W4 * (y3b / rb + 1) - 0.5 * y1 / W6 * a / rb3 * 2 * y3b) +
                       N1 * y2 * cotB / sq(W7) * W9 * W3 + 0.5 * N1 * y2 * cotB / W7 * a / rb3 / cosB * 2 * y3b -
                       a / rb3 * y2 * cotB + 1.5 * a * y2 * W8 * cotB / rb5 * 2 * y3b +
                       y2 / rb / W6 * (N1 * cotB - 2 * nu * y1 / W6 - a * y1 / rb * (1 / rb + 1 / W6)) -
                       0.5 * y2 * W8 / rb3 / W6 * (N1 * cotB - 2 * nu * y1 / W6 - a * y1 / rb * (1 / rb + 1 / W6)) * 2 * y3b -
                       y2 * W8 / rb / sq(W6) * (N1 * cotB - 2 * nu * y1 / W6 - a * y1 / rb * (1 / rb + 1 / W6)) * (y3b / rb + 1) +
                       y2 * W8 / rb / W6 * (2 * nu * y1 / sq(W6) * (y3b / rb + 1) + 0.5 * a * y1 / rb3 * (1 / rb + 1 / W6) * 2 * y3b -
                                            a * y1 / rb * (-0.5 / rb3 * 2 * y3b - 1 / sq(W6) * (y3b / rb + 1))) +
                       y2 * cotB / rb / W7 * ((-2 + 2 * nu) * cosB + W1 / W7 * W9 + a * y3b / rb2 / cosB) -
                       0.5 * y2 * W8 * cotB / rb3 / W7 * ((-2 + 2 * nu) * cosB + W1 / W7 * W9 + a * y3b / rb2 / cosB) * 2 * y3b -
                       y2 * W8 * cotB / rb / sq(W7) * ((-2 + 2 * nu) * cosB + W1 / W7 * W9 + a * y3b / rb2 / cosB) * W3 +
                       y2 * W8 * cotB / rb / W7 * ((cosB * y3b / rb + 1) / W7 * W9 - W1 / sq(W7) * W9 * W3 - 0.5 * W1 / W7 * a / rb3 / cosB * 2 * y3b + a / rb2 / cosB -
                                                   a * y3b / rb4 / cosB * 2 * y3b)) / pi / (1 - nu)) +
        b3 / 2 * (K * (N1 * (-sinB * W3 / W7 + y1 / sq(W6) * (1 + a / rb) * (y3b / rb + 1) + 0.5 * y1 / W6 * a / rb3 * 2 * y3b + sinB / W7 * W2 - z1b / sq(W7) * W2 * W3 -
                             0.5 * z1b / W7 * a / rb3 * 2 * y3b) +
                       y1 / rb * (a / rb2 + 1 / W6) - 0.5 * y1 * W8 / rb3 * (a / rb2 + 1 / W6) * 2 * y3b +
                       y1 * W8 / rb * (-a / rb4 * 2 * y3b - 1 / sq(W6) * (y3b / rb + 1)) -
                       1 / W7 * (sinB * (cosB - a / rb) + z1b / rb * (1 + a * y3b / rb2) - 1 / rb / W7 * (sq(y2) * cosB * sinB - a * z1b / rb * W1)) +
                       W8 / sq(W7) * (sinB * (cosB - a / rb) + z1b / rb * (1 + a * y3b / rb2) - 1 / rb / W7 * (sq(y2) * cosB * sinB - a * z1b / rb * W1)) * W3 -
                       W8 / W7 * (0.5 * sinB * a / rb3 * 2 * y3b + sinB / rb * (1 + a * y3b / rb2) - 0.5 * z1b / rb3 * (1 + a * y3b / rb2) * 2 * y3b +
                                  z1b / rb * (a / rb2 - a * y3b / rb4 * 2 * y3b) + 0.5 / rb3 / W7 * (sq(y2) * cosB * sinB - a * z1b / rb * W1) * 2 * y3b +
                                  1 / rb / sq(W7) * (sq(y2) * cosB * sinB - a * z1b / rb * W1) * W3 -
                                  1 / rb / W7 * (-a * sinB / rb * W1 + 0.5 * a * z1b / rb3 * W1 * 2 * y3b - a * z1b / rb * (cosB * y3b / rb + 1)))) / pi / (1 - nu)) +
        b1 / 2 * (K * ((2 - 2 * nu) * (N1 * rFib_ry2 * cotB + 1 / W6 * W5 - sq(y2) / sq(W6) * W5 / rb - sq(y2) / W6 * a / rb3 - cosB / W7 * W2 + sq(y2) * cosB / sq(W7) * W2 / rb +
                                       sq(y2) * cosB / W7 * a / rb3) +
                       W8 / rb * (2 * nu / W6 + a / rb2) - sq(y2) * W8 / rb3 * (2 * nu / W6 + a / rb2) + y2 * W8 / rb * (-2 * nu / sq(W6) / rb * y2 - 2 * a / rb4 * y2) +
                       W8 * cosB / rb / W7 * (1 - 2 * nu - W1 / W7 * W2 - a * y3b / rb2) -
                       sq(y2) * W8 * cosB / rb3 / W7 * (1 - 2 * nu - W1 / W7 * W2 - a * y3b / rb2) -
                       sq(y2) * W8 * cosB / rb2 / sq(W7) * (1 - 2 * nu - W1 / W7 * W2 - a * y3b / rb2) +
                       y2 * W8 * cosB / rb / W7 * (-1 / rb * cosB * y2 / W7 * W2 + W1 / sq(W7) * W2 / rb * y2 + W1 / W7 * a / rb3 * y2 + 2 * a * y3b / rb4 * y2)) / pi / (1 - nu)) +
        b2 / 2 * (K * ((-2 + 2 * nu) * N1 * cotB * (1 / rb * y2 / W6 - cosB / rb * y2 / W7) + (2 - 2 * nu) * y1 / sq(W6) * W5 / rb * y2 + (2 - 2 * nu) * y1 / W6 * a / rb3 * y2 -
                       (2 - 2 * nu) * z1b / sq(W7) * W2 / rb * y2 - (2 - 2 * nu) * z1b / W7 * a / rb3 * y2 - W8 / rb3 * (N1 * cotB - 2 * nu * y1 / W6 - a * y1 / rb2) * y2 +
                       W8 / rb * (2 * nu * y1 / sq(W6) / rb * y2 + 2 * a * y1 / rb4 * y2) +
                       W8 / sq(W7) * (cosB * sinB + W1 * cotB / rb * ((2 - 2 * nu) * cosB - W1 / W7) + a / rb * (sinB - y3b * z1b / rb2 - z1b * W1 / rb / W7)) / rb * y2 -
                       W8 / W7 * (1 / rb2 * cosB * y2 * cotB * ((2 - 2 * nu) * cosB - W1 / W7) - W1 * cotB / rb3 * ((2 - 2 * nu) * cosB - W1 / W7) * y2 +
                                  W1 * cotB / rb * (-cosB / rb * y2 / W7 + W1 / sq(W7) / rb * y2) - a / rb3 * (sinB - y3b * z1b / rb2 - z1b * W1 / rb / W7) * y2 +
                                  a / rb * (2 * y3b * z1b / rb4 * y2 - z1b / rb2 * cosB * y2 / W7 + z1b * W1 / rb3 / W7 * y2 + z1b * W1 / rb2 / sq(W7) * y2))) / pi / (1 - nu)) +
        b3 / 2 * (K * ((2 - 2 * nu) * rFib_ry2 + (2 - 2 * nu) * sinB / W7 * W2 - (2 - 2 * nu) * sq(y2) * sinB / sq(W7) * W2 / rb - (2 - 2 * nu) * sq(y2) * sinB / W7 * a / rb3 +
                       W8 * sinB / rb / W7 * (1 + W1 / W7 * W2 + a * y3b / rb2) -
                       sq(y2) * W8 * sinB / rb3 / W7 * (1 + W1 / W7 * W2 + a * y3b / rb2) -
                       sq(y2) * W8 * sinB / rb2 / sq(W7) * (1 + W1 / W7 * W2 + a * y3b / rb2) +
                       y2 * W8 * sinB / rb / W7 * (1 / rb * cosB * y2 / W7 * W2 - W1 / sq(W7) * W2 / rb * y2 - W1 / W7 * a / rb3 * y2 - 2 * a * y3b / rb4 * y2)) / pi / (1 - nu));
}

// TDSetupS (:433-464)
__device__ void td_setup_s(double x, double y, double z, double alpha, double bx, double by, double bz,
                double nu, const double TV[3], const double SV[3], double e[6]) {
    // A = [SV3 -SV2; SV2 SV3]
    double y1 = SV[2] * (y - TV[1]) - SV[1] * (z - TV[2]);
    double z1 = SV[1] * (y - TV[1]) + SV[2] * (z - TV[2]);
    double by1 = SV[2] * by - SV[1] * bz;
    double bz1 = SV[1] * by + SV[2] * bz;
    double ea[6];
    ang_dis_strain(x, y1, z1, -CUDART_PI + alpha, bx, by1, bz1, nu, ea);
    // B = [1 0 0; 0 SV3 SV2; 0 -SV2 SV3], column-major
    double B[9] = {1, 0, 0, 0, SV[2], -SV[1], 0, SV[1], SV[2]};
    tens_trans(ea, B, e);
}

// trimodefinder (:393-430) for one point; x,y = TDCS y,z and z = TDCS x.
__device__ int trimode(double x, double y, double z, const double p1[2], const double p2[2],
            const double p3[2]) {
    double den = (p2[1] - p3[1]) * (p1[0] - p3[0]) + (p3[0] - p2[0]) * (p1[1] - p3[1]);
    double a = ((p2[1] - p3[1]) * (x - p3[0]) + (p3[0] - p2[0]) * (y - p3[1])) / den;
    double b = ((p3[1] - p1[1]) * (x - p3[0]) + (p1[0] - p3[0]) * (y - p3[1])) / den;
    double c = 1 - a - b;
    int t = 1;
    if (a <= 0 && b > c && c > a) t = -1;
    if (b <= 0 && c > a && a > b) t = -1;
    if (c <= 0 && a > b && b > c) t = -1;
    if (a == 0 && b >= 0 && c >= 0) t = 0;
    if (a >= 0 && b == 0 && c >= 0) t = 0;
    if (a >= 0 && b >= 0 && c == 0) t = 0;
    if (t == 0 && z != 0) t = 1;
    return t;
}

// TDstressFS (:133-286): strains (EFCS) of a TD in a full space.
__device__ void td_strain_fs(double X, double Y, double Z, const double P1[3], const double P2[3],
                  const double P3[3], double Ss, double Ds, double Ts, double mu, double lambda,
                  double E[6]) {
    double nu = 1 / (1 + lambda / mu) / 2;
    double bx = Ts, by = Ss, bz = Ds;
    double d21[3] = {P2[0] - P1[0], P2[1] - P1[1], P2[2] - P1[2]};
    double d31[3] = {P3[0] - P1[0], P3[1] - P1[1], P3[2] - P1[2]};
    double Vnorm[3];
    cross3(d21, d31, Vnorm);
    double nn = norm3(Vnorm);
    for (int k = 0; k < 3; ++k) Vnorm[k] = Vnorm[k] / nn;
    double eY[3] = {0, 1, 0}, eZ[3] = {0, 0, 1};
    double Vstrike[3];
    cross3(eZ, Vnorm, Vstrike);
    if (norm3(Vstrike) == 0) {
        for (int k = 0; k < 3; ++k) Vstrike[k] = eY[k] * Vnorm[2];
        if (P1[2] > 0)
            for (int k = 0; k < 3; ++k) Vstrike[k] = -Vstrike[k];
    }
    double ns = norm3(Vstrike);
    for (int k = 0; k < 3; ++k) Vstrike[k] = Vstrike[k] / ns;
    double Vdip[3];
    cross3(Vnorm, Vstrike, Vdip);
    // A = [Vnorm Vstrike Vdip]' : rows are Vnorm, Vstrike, Vdip; column-major storage
    double At[9] = {Vnorm[0], Vstrike[0], Vdip[0], Vnorm[1], Vstrike[1], Vdip[1],
                    Vnorm[2], Vstrike[2], Vdip[2]};
    double xyz[3], p1[3], p2[3] = {0, 0, 0}, p3[3];
    coord_trans(X - P2[0], Y - P2[1], Z - P2[2], At, xyz);
    coord_trans(P1[0] - P2[0], P1[1] - P2[1], P1[2] - P2[2], At, p1);
    coord_trans(P3[0] - P2[0], P3[1] - P2[1], P3[2] - P2[2], At, p3);
    double x = xyz[0], y = xyz[1], z = xyz[2];
    double e12[3], e13[3], e23[3];
    {
        double d[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
        double n = norm3(d);
        for (int k = 0; k < 3; ++k) e12[k] = d[k] / n;
        double d2[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
        n = norm3(d2);
        for (int k = 0; k < 3; ++k) e13[k] = d2[k] / n;
        double d3[3] = {p3[0] - p2[0], p3[1] - p2[1], p3[2] - p2[2]};
        n = norm3(d3);
        for (int k = 0; k < 3; ++k) e23[k] = d3[k] / n;
    }
    double A = acos(e12[0] * e13[0] + e12[1] * e13[1] + e12[2] * e13[2]);
    double B = acos(-e12[0] * e23[0] + -e12[1] * e23[1] + -e12[2] * e23[2]);
    double C = acos(e23[0] * e13[0] + e23[1] * e13[1] + e23[2] * e13[2]);
    double q1[2] = {p1[1], p1[2]}, q2[2] = {p2[1], p2[2]}, q3[2] = {p3[1], p3[2]};
    int tm = trimode(y, z, x, q1, q2, q3);
    double e[6];
    if (tm == 1) {
        double s1[6], s2[6], s3[6];
        double m13[3] = {-e13[0], -e13[1], -e13[2]};
        td_setup_s(x, y, z, A, bx, by, bz, nu, p1, m13, s1);
        td_setup_s(x, y, z, B, bx, by, bz, nu, p2, e12, s2);
        td_setup_s(x, y, z, C, bx, by, bz, nu, p3, e23, s3);
        for (int k = 0; k < 6; ++k) e[k] = s1[k] + s2[k] + s3[k];
    } else if (tm == -1) {
        double s1[6], s2[6], s3[6];
        double m12[3] = {-e12[0], -e12[1], -e12[2]}, m23[3] = {-e23[0], -e23[1], -e23[2]};
        td_setup_s(x, y, z, A, bx, by, bz, nu, p1, e13, s1);
        td_setup_s(x, y, z, B, bx, by, bz, nu, p2, m12, s2);
        td_setup_s(x, y, z, C, bx, by, bz, nu, p3, m23, s3);
        for (int k = 0; k < 6; ++k) e[k] = s1[k] + s2[k] + s3[k];
    } else {
        for (int k = 0; k < 6; ++k) e[k] = CUDART_NAN;
    }
    // back to EFCS with [Vnorm Vstrike Vdip] (columns), column-major
    double Am[9] = {Vnorm[0], Vnorm[1], Vnorm[2], Vstrike[0], Vstrike[1], Vstrike[2],
                    Vdip[0], Vdip[1], Vdip[2]};
    tens_trans(e, Am, E);
}

// AngSetupFSC_S (:467-574): free-surface correction of one TD side (strains).
__device__ void ang_setup_fsc(double X, double Y, double Z, double bX, double bY, double bZ,
                   const double PA[3], const double PB[3], double mu, double lambda,
                   double E[6]) {
    double nu = 1 / (1 + lambda / mu) / 2;
    double SV[3] = {PB[0] - PA[0], PB[1] - PA[1], PB[2] - PA[2]};
    double beta = acos(-SV[2] / norm3(SV));
    if (fabs(beta) < 1e-16 || fabs(CUDART_PI - beta) < 1e-16) {
        for (int k = 0; k < 6; ++k) E[k] = 0;
        return;
    }
    double ey1[3] = {SV[0], SV[1], 0};
    double n1 = norm3(ey1);
    for (int k = 0; k < 3; ++k) ey1[k] = ey1[k] / n1;
    double ey3[3] = {0, 0, -1};
    double ey2[3];
    cross3(ey3, ey1, ey2);
    // A = [ey1 ey2 ey3] (columns), column-major
    double A[9] = {ey1[0], ey1[1], ey1[2], ey2[0], ey2[1], ey2[2], ey3[0], ey3[1], ey3[2]};
    double yA[3], yAB[3], b[3];
    coord_trans(X - PA[0], Y - PA[1], Z - PA[2], A, yA);
    coord_trans(SV[0], SV[1], SV[2], A, yAB);
    double yB[3] = {yA[0] - yAB[0], yA[1] - yAB[1], yA[2] - yAB[2]};
    coord_trans(bX, bY, bZ, A, b);
    double vA[6], vB[6];
    if (beta * yA[0] >= 0) {
        ang_dis_strain_fsc(-yA[0], -yA[1], yA[2], CUDART_PI - beta, -b[0], -b[1], b[2], nu, -PA[2], vA);
        vA[4] = -vA[4];
        vA[5] = -vA[5];
        ang_dis_strain_fsc(-yB[0], -yB[1], yB[2], CUDART_PI - beta, -b[0], -b[1], b[2], nu, -PB[2], vB);
        vB[4] = -vB[4];
        vB[5] = -vB[5];
    } else {
        ang_dis_strain_fsc(yA[0], yA[1], yA[2], beta, b[0], b[1], b[2], nu, -PA[2], vA);
        ang_dis_strain_fsc(yB[0], yB[1], yB[2], beta, b[0], b[1], b[2], nu, -PB[2], vB);
    }
    double v[6];
    for (int k = 0; k < 6; ++k) v[k] = vB[k] - vA[k];
    // A' (transpose), column-major
    double At[9] = {A[0], A[3], A[6], A[1], A[4], A[7], A[2], A[5], A[8]};
    tens_trans(v, At, E);
}

__device__ void stress_from_strain(const double E[6], double mu, double lambda, double S[6]) {
    double tr = E[0] + E[1] + E[2];
    S[0] = 2 * mu * E[0] + lambda * tr;
    S[1] = 2 * mu * E[1] + lambda * tr;
    S[2] = 2 * mu * E[2] + lambda * tr;
    S[3] = 2 * mu * E[3];
    S[4] = 2 * mu * E[4];
    S[5] = 2 * mu * E[5];
}


// TDstressHS for one point: stress (xx,yy,zz,xy,xz,yz) in EFCS.
__device__ void tdstress_hs(double X, double Y, double Z, const double P1in[3],
                            const double P2in[3], const double P3in[3], double Ss, double Ds,
                            double Ts, double mu, double lambda, double stress[6]) {
    double P1[3] = {P1in[0], P1in[1], P1in[2]}, P2[3] = {P2in[0], P2in[1], P2in[2]},
           P3[3] = {P3in[0], P3in[1], P3in[2]};
    double E[6], S[6];
    td_strain_fs(X, Y, Z, P1, P2, P3, Ss, Ds, Ts, mu, lambda, E);
    stress_from_strain(E, mu, lambda, S);
    {
        double d21[3] = {P2[0] - P1[0], P2[1] - P1[1], P2[2] - P1[2]};
        double d31[3] = {P3[0] - P1[0], P3[1] - P1[1], P3[2] - P1[2]};
        double Vnorm[3];
        cross3(d21, d31, Vnorm);
        double nn = norm3(Vnorm);
        for (int k = 0; k < 3; ++k) Vnorm[k] = Vnorm[k] / nn;
        double Vstrike[3] = {-Vnorm[1], Vnorm[0], 0.0};  // eZ x Vnorm
        if (norm3(Vstrike) == 0) {
            Vstrike[0] = 0; Vstrike[1] = Vnorm[2]; Vstrike[2] = 0;
        }
        double ns = norm3(Vstrike);
        for (int k = 0; k < 3; ++k) Vstrike[k] = Vstrike[k] / ns;
        double Vdip[3];
        cross3(Vnorm, Vstrike, Vdip);
        double A[9] = {Vnorm[0], Vnorm[1], Vnorm[2], Vstrike[0], Vstrike[1], Vstrike[2],
                       Vdip[0], Vdip[1], Vdip[2]};
        double b[3];
        coord_trans(Ts, Ss, Ds, A, b);
        double Ef[6], e1[6], Sf[6];
        ang_setup_fsc(X, Y, Z, b[0], b[1], b[2], P1, P2, mu, lambda, e1);
        for (int k = 0; k < 6; ++k) Ef[k] = e1[k];
        ang_setup_fsc(X, Y, Z, b[0], b[1], b[2], P2, P3, mu, lambda, e1);
        for (int k = 0; k < 6; ++k) Ef[k] += e1[k];
        ang_setup_fsc(X, Y, Z, b[0], b[1], b[2], P3, P1, mu, lambda, e1);
        for (int k = 0; k < 6; ++k) Ef[k] += e1[k];
        stress_from_strain(Ef, mu, lambda, Sf);
        for (int k = 0; k < 6; ++k) S[k] += Sf[k];
    }
    P1[2] = -P1[2]; P2[2] = -P2[2]; P3[2] = -P3[2];
    double Ei[6], Si[6];
    td_strain_fs(X, Y, Z, P1, P2, P3, Ss, Ds, Ts, mu, lambda, Ei);
    stress_from_strain(Ei, mu, lambda, Si);
    if (P1[2] == 0 && P2[2] == 0 && P3[2] == 0) { Si[4] = -Si[4]; Si[5] = -Si[5]; }
    for (int k = 0; k < 6; ++k) stress[k] = S[k] + Si[k];
}

}  // namespace tdhs
}  // namespace qdfn
