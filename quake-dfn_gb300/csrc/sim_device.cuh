// Device side of the earthquake-cycle step loop: the per-patch friction
// solvers, the aging/slip evolution law and the external-stress interpolation.
//
//   EvolutionLaw                 scripts/Functions_Solvers.jl:2-15
//   Solver_HighV_D               scripts/Functions_Solvers.jl:26-182
//   Solver_LowV_D                scripts/Functions_Solvers.jl:185-327
//   InterpolateFromStressChange  scripts/Functions_Solvers.jl:465-540
//
// Every branch, iteration count and Dt-halving rule of the reference is kept:
// the step's outcome (accepted Dt, retries, solver switches) is decided by
// these branches, so reproducing them is what makes trajectories comparable.
// Julia's `log` throws on a negative argument; here that raises
// QDFN_ERR_DOMAIN.  Where the reference waits on stdin (`readline()` when
// Dt < 1e-10 in the high-V solver) the device code continues as if the user
// pressed Enter.
#pragma once
#include "qdfn_internal.h"

namespace qdfn {
namespace sim {

constexpr double kV0 = 1e-9;              // Main_D :42
constexpr double kConv = 1e-9;            // Main_D :46
constexpr int kHighVIterCap = 40000;      // tolerance*10 per 100 its reaches Inf by ~31700

struct PatchIn {
    double DispOld, FrictionOld, ThetaOld, VOld, Friction0, a, b, Dc, K_Self, Omega, Mass;
    double sigma, TLD, dtau, sigma_old, tau0;
    double ra, rDc, rDt;   // 1/a, 1/Dc, 1/Dt correctly rounded (Dt: the step the solve starts from)
};
struct PatchOut {
    double V, Friction, Disp, Theta, Dt;
    int Instab, Flag;
    int Iterations;      // secant iterations taken (diagnostics)
};

__device__ __forceinline__ double jlog(double x, int& err) {
    if (x < 0.0) err = QDFN_ERR_DOMAIN;
    return log(x);
}

// The normal-stress coupling term alpha * dsigma / Dt / b / sigma of the aging
// law is an exact (signed) zero when alpha == 0 and every operand is finite and
// nonzero; adding it then leaves a nonzero sum unchanged, so it is skipped
// (three FP64 divisions per call; Alpha_Evo is 0 in the reference,
// QUAKEDFN_RunARG.jl:170).  Otherwise it is evaluated as written.
__device__ __forceinline__ bool alpha_term_zero(double alpha, double Dt, double sig, double sig_old,
                                                double b) {
    return alpha == 0.0 && isfinite(Dt) && Dt != 0.0 && isfinite(sig) && sig != 0.0 &&
           isfinite(sig_old) && isfinite(b) && b != 0.0;
}

// Division by a divisor that stays fixed for a whole solve.  With y = 1/d
// correctly rounded (one IEEE division per solve), q0 = x*y is within two ulps
// of x/d, the remainder r = x - q0*d is exact in one FMA, and q0 + r*y is x/d
// up to an error of about 2^-52 ulp before its rounding (Markstein's correction
// step: P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990), so it rounds to the
// IEEE quotient unless x/d lies that close to a rounding boundary; the GPU
// test of this helper checks it bit for bit against IEEE division on random
// operands and on hard cases.  Three FP64 operations instead of the eight of a
// full division.  A
// zero dividend returns q0 = x * y, whose sign is IEEE's for x / d.  Operands
// whose magnitudes leave [2^-895, 2^896] (or a divisor that is zero, infinite
// or NaN) take the full division, so no step can overflow or underflow.
struct Recip {
    double d, y;
    bool ok;
};
__device__ __forceinline__ int exp_field(double v) { return (__double2hiint(v) >> 20) & 0x7ff; }
__device__ __forceinline__ bool in_safe_range(int e) { return (unsigned)(e - 128) <= 1791u; }
__device__ __forceinline__ Recip recip(double d) {
    Recip r;
    r.d = d;
    r.y = 1.0 / d;
    r.ok = in_safe_range(exp_field(d));
    return r;
}
// The same from a reciprocal formed earlier (y = 1/d correctly rounded).
__device__ __forceinline__ Recip recip_pre(double d, double y) {
    Recip r;
    r.d = d;
    r.y = y;
    r.ok = in_safe_range(exp_field(d));
    return r;
}
static __device__ __noinline__ double full_div(double x, double d) { return x / d; }
__device__ __forceinline__ double div_by(double x, const Recip& R) {
    const double q0 = x * R.y;
    const double r = fma(-q0, R.d, x);
    const double q = -fma(-r, R.y, -q0);
    const bool zero = (__double_as_longlong(x) << 1) == 0;
    const bool fast = R.ok && (zero || (in_safe_range(exp_field(x)) && in_safe_range(exp_field(q0))));
    if (fast) return zero ? q0 : q;   // a zero dividend: q0 = x * (1/d) carries the IEEE sign
    return full_div(x, R.d);   // out of line: never evaluated speculatively
}

// The alpha terms as written in the reference.  Out of line so that the
// compiler cannot evaluate them speculatively next to the (usual) skip path.
static __device__ __noinline__ double alpha_term_fast(double alpha, double sig, double sig_old, double Dt,
                                               double b) {
    return alpha * (sig - sig_old) / Dt / b / sig;
}
static __device__ __noinline__ double alpha_term_slow(double alpha, double sig, double sig_old, double Dt,
                                               double b) {
    return alpha * Dt * (sig - sig_old) / Dt / b / sig;
}

// `skip` = alpha_term_zero(alpha, Dt, sig, sig_old, b), evaluated once per
// solve by the caller: its operands do not change between the evolution calls
// of one solve (Dt is only halved on the way out of the secant loop).
__device__ __forceinline__ double evolution(double ThetaOld, double Dt, double V, const Recip& Rdc,
                                            double alpha, double sig, double sig_old, double b,
                                            int fast, int dr, bool skip, int& err) {
    if (dr == 1) {
        if (fast) {
            const double vd = div_by(V, Rdc);
            double Const_T = vd;
            if (!(skip && vd != 0.0)) Const_T = vd + alpha_term_fast(alpha, sig, sig_old, Dt, b);
            // (-V)/Dc == -(V/Dc) exactly, so the quotient is reused
            return (ThetaOld - 1 / Const_T) * exp(-vd * Dt) + 1 / Const_T;
        }
        const double den0 = 1 + div_by(Dt * V, Rdc);
        double den = den0;
        if (!(skip && den0 != 0.0)) den = den0 + alpha_term_slow(alpha, sig, sig_old, Dt, b);
        return (ThetaOld + Dt) / den;
    }
    const double w = div_by(V * ThetaOld, Rdc);
    return ThetaOld - w * jlog(w, err) * Dt;
}

// Semi-analytic harmonic-oscillator update with a secant iteration on V.
//
// As in the low-velocity solver below, an iteration's first evaluation is at
// the V of the previous iteration's update, whose Theta and Friction =
// mu0 + a ln(V/V0) + b ln(V0 Theta/Dc) are the first terms of that evaluation
// (same operations on the same operands), so they are reused.
#define QDFN_RESET() do { V = p.VOld; Theta = p.ThetaOld; Friction = p.FrictionOld; Disp = p.DispOld; } while (0)
// one evaluation of the oscillator map at Vx, given Theta and the friction
// prefix there: the V it returns
#define QDFN_OSC_V(Vx, Fpre)                                                            \
    ([&]() {                                                                            \
        const double Fr_ = (Fpre) + eta / p.sigma * (Vx) - p.dtau / p.sigma;            \
        const double F_ = p.TLD + (p.tau0 - Fr_ * p.sigma) / p.K_Self;                  \
        const double D_ = (p.DispOld - F_) * cO + (p.VOld / p.Omega) * sO + F_;         \
        return div_by(D_ - p.DispOld, Rdt) * 2 - p.VOld;                                \
    }())
#define QDFN_FPRE(Vx, Tx, errx) \
    (p.Friction0 + p.a * jlog((Vx) / kV0, errx) + p.b * jlog(div_by((Tx) * kV0, Rdc), errx))
// :87-134 -- both the negative and the NaN branch halve Dt; below Dt = 1e-5
// they also mark Instability = 4 (the V<0 branch) or do so after printing
// (the NaN branch)
#define QDFN_HV_NEG()                                                         \
    do {                                                                      \
        if (Dt > 1e-5) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; }  \
        else { Dt = Dt / 2; Instab = 4; QDFN_RESET(); maxDiff = 0; FLAG = 0; } \
    } while (0)
#define QDFN_HV_CAP()                                                         \
    do {                                                                      \
        if (Iteration % 100 == 0) {                                           \
            if (Dt < 1e-5) { crit = crit * 10; Instab = 2; }                  \
            else { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; }        \
        }                                                                     \
    } while (0)

static __device__ PatchOut solve_highv(const PatchIn& p, double Dt, double eta, double alpha, int dr,
                                int& err) {
    int FLAG = 1, Instab = 0, Iteration = 0;
    double maxDiff = 10, crit = kConv;
    const double DV = p.VOld / 100;
    double V = p.VOld / 1e10, Disp = p.DispOld, Friction = p.FrictionOld, Theta = p.ThetaOld;
    if (V < 0) V = 1e-100;
    const bool skip = dr == 1 && alpha_term_zero(alpha, Dt, p.sigma, p.sigma_old, p.b);
    // the reference evaluates cos/sin(Omega Dt) in every iteration; Dt is
    // constant for every iteration that reaches them, so once is the same
    const double cO = cos(p.Omega * Dt), sO = sin(p.Omega * Dt);
    // divisors fixed for the solve (Dt only changes on the way out of the loop)
    const Recip Rdc = recip_pre(p.Dc, p.rDc), Rdt = recip_pre(Dt, p.rDt);
    bool at_v = false;   // Theta and Friction are the update's values at V
    while (maxDiff > crit) {
        Iteration++;
        if (Iteration > kHighVIterCap) { err = QDFN_ERR_NO_CONVERGE; break; }
        const double VTest = V;
        if (!at_v) {
            Theta = evolution(p.ThetaOld, Dt, V, Rdc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, skip, err);
            if (Theta < 0) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; break; }
            Friction = QDFN_FPRE(V, Theta, err);
        }
        V = QDFN_OSC_V(VTest, Friction);
        const double FOriginal = VTest - V;
        V = VTest + DV;
        const double VTest2 = V;
        Theta = evolution(p.ThetaOld, Dt, V, Rdc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, skip, err);
        if (Theta < 0) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; break; }
        V = QDFN_OSC_V(VTest2, QDFN_FPRE(VTest2, Theta, err));
        const double FUpdated = VTest2 - V;
        V = VTest - FOriginal * DV / (FUpdated - FOriginal);
        if (V < 0 || isnan(V)) {
            QDFN_HV_NEG();
        } else {
            Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
            Theta = evolution(p.ThetaOld, Dt, V, Rdc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, skip, err);
            if (Theta < 0) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; break; }
            Friction = QDFN_FPRE(V, Theta, err);
            maxDiff = fabs(VTest / V - 1);
            Instab = 0;
        }
        QDFN_HV_CAP();
        if (err) break;
        at_v = true;
    }
    PatchOut o;
    o.V = V; o.Friction = Friction; o.Disp = Disp; o.Theta = Theta; o.Dt = Dt;
    o.Instab = Instab; o.Flag = FLAG; o.Iterations = Iteration;
    return o;
}

// One lane pair per patch (the even lane's result is the solve's), both lanes
// running the same instructions on different points: iteration 1 evaluates
// at V (even) and V + DV (odd); after each secant step the even lane evaluates
// at the new V -- its Theta and friction prefix are the update's -- and the
// odd lane at the new V + DV, the next iteration's two evaluations.  Errors
// count where the reference loop raises them: the update's (evolution law,
// friction logarithms) only when the update runs (V >= 0, not NaN); the
// second evaluation's only when the first passed.
static __device__ PatchOut solve_highv_pair(const PatchIn& p, double Dt, double eta, double alpha, int dr,
                                     int& err) {
    int FLAG = 1, Instab = 0, Iteration = 0;
    double maxDiff = 10, crit = kConv;
    const double DV = p.VOld / 100;
    double V = p.VOld / 1e10, Disp = p.DispOld, Friction = p.FrictionOld, Theta = p.ThetaOld;
    if (V < 0) V = 1e-100;
    const bool skip = dr == 1 && alpha_term_zero(alpha, Dt, p.sigma, p.sigma_old, p.b);
    const double cO = cos(p.Omega * Dt), sO = sin(p.Omega * Dt);
    const Recip Rdc = recip_pre(p.Dc, p.rDc), Rdt = recip_pre(Dt, p.rDt);
    const int lane = threadIdx.x & 31, base = lane & ~1;
    const bool odd = (lane & 1) != 0;
    const unsigned pmask = 3u << base;
    // one evaluation at Vh: Theta, the friction prefix and the residual
    double Th, Fp, FVh;
    int eh, tc;
    auto evaluate = [&](double Vh) {
        eh = 0;
        Fp = 0;
        FVh = 0;
        Th = evolution(p.ThetaOld, Dt, Vh, Rdc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, skip, eh);
        tc = Th < 0 ? 1 : 0;
        if (!tc) {
            Fp = QDFN_FPRE(Vh, Th, eh);
            FVh = Vh - QDFN_OSC_V(Vh, Fp);
        }
    };
    Iteration = 1;   // 1 <= kHighVIterCap
    double VTest = V;
    evaluate(odd ? VTest + DV : VTest);
    int fail0 = __shfl_sync(pmask, tc, base), fail1 = __shfl_sync(pmask, tc, base + 1);
    int err0 = __shfl_sync(pmask, eh, base), err1 = __shfl_sync(pmask, eh, base + 1);
    double FO = __shfl_sync(pmask, FVh, base), FU = __shfl_sync(pmask, FVh, base + 1);
    for (;;) {
        if (err0) err = err0;
        if (fail0) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; break; }
        if (err1) err = err1;
        if (fail1) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; break; }
        V = VTest - FO * DV / (FU - FO);
        if (V < 0 || isnan(V)) {
            QDFN_HV_NEG();
            QDFN_HV_CAP();
            break;   // maxDiff = 0 ends the loop (after the error check, which would too)
        }
        Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
        evaluate(odd ? V + DV : V);
        const int tcode = __shfl_sync(pmask, tc, base);
        const int erru = __shfl_sync(pmask, eh, base);
        const int f1 = __shfl_sync(pmask, tc, base + 1), e1 = __shfl_sync(pmask, eh, base + 1);
        const double FOn = __shfl_sync(pmask, FVh, base), FUn = __shfl_sync(pmask, FVh, base + 1);
        // the even lane's evaluation is the update at V
        Theta = Th;
        if (erru) err = erru;
        if (tcode) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; break; }
        Friction = Fp;
        maxDiff = fabs(VTest / V - 1);
        Instab = 0;
        QDFN_HV_CAP();
        if (err) break;
        if (!(maxDiff > crit)) break;
        Iteration++;
        if (Iteration > kHighVIterCap) { err = QDFN_ERR_NO_CONVERGE; break; }
        VTest = V;
        fail0 = 0; err0 = 0;   // the update's values: its errors are counted already
        fail1 = f1; err1 = e1;
        FO = FOn; FU = FUn;
    }
    PatchOut o;
    o.V = V; o.Friction = Friction; o.Disp = Disp; o.Theta = Theta; o.Dt = Dt;
    o.Instab = Instab; o.Flag = FLAG; o.Iterations = Iteration;
    return o;
}
#undef QDFN_OSC_V
#undef QDFN_FPRE
#undef QDFN_HV_NEG
#undef QDFN_HV_CAP

// Implicit trapezoidal update with a secant iteration on V and the friction
// inversion V = V0 exp((mu - mu0 - b ln(V0 theta/Dc))/a), all in FP64.
//
// One iteration of the reference loop: evaluate the residual at VTest = V and
// at V + DV (each: Accel, Theta, Disp, Friction, then the friction inversion),
// take the secant step to a new V, then update Accel, Disp, Theta, Friction and
// maxDiff at the new V.  The next iteration's first evaluation is at exactly
// that V, so its Accel, Theta, Disp and Friction are the values the update just
// formed (same operations on the same operands; with --fmad=false no
// contraction can differ), and they passed the update's Theta checks -- only
// the friction inversion is new.  Both solvers below reuse them and return what
// the reference loop returns, bit for bit.
#define QDFN_FAIL_A()                                                    \
    do {                                                                   \
        if (Dt < SwitchV) { Instab = 3; QDFN_RESET(); FLAG = 0; }          \
        else if (p.VOld == 0) { QDFN_RESET(); FLAG = 1; }                  \
        else { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; }         \
    } while (0)
#define QDFN_FRICTION(Vx, Dx, Ax) \
    (inv_sig * (p.K_Self * (p.TLD - (Dx)) + p.tau0 - eta * (Vx) + p.dtau - p.Mass * (Ax)))
#define QDFN_VEL(Fx, Tx, errx) \
    (kV0 * exp(div_by((Fx) - p.Friction0 - p.b * jlog(div_by(kV0 * (Tx), Rdc), errx), Ra)))
// Theta came out NaN in the update (Solvers :283-301)
#define QDFN_THETA_NAN()                                                                     \
    do {                                                                                     \
        if (p.VOld == 0) { QDFN_RESET(); FLAG = 1; }                                         \
        else if (Dt < 1e-3) {                                                                \
            if (p.VOld < 1e-7) {                                                             \
                V = 0; Theta = p.ThetaOld + Dt; Friction = p.FrictionOld; Disp = p.DispOld;  \
                maxDiff = 0; FLAG = 1;                                                       \
            } else { Instab = 3; QDFN_RESET(); FLAG = 0; }                                   \
        } else { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; }                         \
    } while (0)
// every 200 iterations (Solvers :309-318); always leaves the loop
#define QDFN_ITER_CAP()                                              \
    do {                                                             \
        if (Dt < 1e-4) { Instab = 3; QDFN_RESET(); FLAG = 0; }       \
        else if (Dt < 1e1) { crit = crit * 2; }                      \
        else { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; }   \
    } while (0)

// One lane per patch.
static __device__ PatchOut solve_lowv(const PatchIn& p, double Dt, double eta, double alpha, int dr,
                               double SwitchV, int& err) {
    int FLAG = 1, Instab = 0, Iteration = 0;
    double maxDiff = 10, crit = kConv;
    double V = p.VOld, Disp = p.DispOld, Friction = p.FrictionOld, Theta = p.ThetaOld;
    const double inv_sig = 1 / p.sigma;
    const bool skip = dr == 1 && alpha_term_zero(alpha, Dt, p.sigma, p.sigma_old, p.b);
    // divisors fixed for the solve (Dt only changes on the way out of the loop);
    // 1e-10 is the correctly rounded reciprocal of 1e10 (both are 10^-10 rounded)
    const Recip Rdc = recip_pre(p.Dc, p.rDc), Rdt = recip_pre(Dt, p.rDt), Ra = recip_pre(p.a, p.ra);
    const Recip R1e10 = {1e10, 1e-10, true};
    double Accel = 0;
    bool at_v = false;   // Accel, Theta, Disp, Friction are the update's values at V
    while (maxDiff > crit) {
        Iteration++;
        const double VTest = V;
        const double DV = div_by(VTest, R1e10);
        if (!at_v) {
            Accel = div_by(V - p.VOld, Rdt);
            Theta = evolution(p.ThetaOld, Dt, V, Rdc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, skip, err);
            if (Theta < 0 || isnan(Theta)) { QDFN_FAIL_A(); break; }
            Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
            Friction = QDFN_FRICTION(V, Disp, Accel);
        }
        const double FV = VTest - QDFN_VEL(Friction, Theta, err);
        V = V + DV;
        const double VTest2 = V;
        Accel = div_by(V - p.VOld, Rdt);
        Theta = evolution(p.ThetaOld, Dt, V, Rdc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, skip, err);
        if (Theta < 0 || isnan(Theta)) { QDFN_FAIL_A(); break; }
        Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
        Friction = QDFN_FRICTION(V, Disp, Accel);
        const double FV_DeV = VTest2 - QDFN_VEL(Friction, Theta, err);
        V = VTest - FV * DV / (FV_DeV - FV);
        if (dr != 1 && V < 0)
            V = exp(jlog(VTest, err) - FV * jlog(VTest2 / VTest, err) / (FV_DeV - FV));
        Accel = div_by(V - p.VOld, Rdt);
        Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
        Theta = evolution(p.ThetaOld, Dt, V, Rdc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, skip, err);
        if (Theta < 0) { QDFN_FAIL_A(); break; }
        if (isnan(Theta)) { QDFN_THETA_NAN(); break; }
        Friction = QDFN_FRICTION(V, Disp, Accel);
        maxDiff = fabs(VTest / V - 1);
        if (Iteration % 200 == 0) { QDFN_ITER_CAP(); break; }
        if (err) break;
        at_v = true;
    }
    PatchOut o;
    o.V = V; o.Friction = Friction; o.Disp = Disp; o.Theta = Theta; o.Dt = Dt;
    o.Instab = Instab; o.Flag = FLAG; o.Iterations = Iteration;
    return o;
}

// One lane pair per patch (lanes 2k, 2k+1 of the warp, same inputs; the even
// lane's result is the solve's).  Both lanes run the same instructions on
// different points -- an evaluation each -- so the warp never splits:
//   iteration 1: the even lane evaluates at V, the odd lane at V + DV;
//   every iteration: exchange the outcomes, take the secant step to the new V
//     (the same arithmetic on both lanes), then evaluate again: the even lane
//     at the new V -- its Accel, Disp, Theta and Friction are the update's, and
//     its friction inversion is the next iteration's first evaluation -- and
//     the odd lane at the new V + V/1e10, the next iteration's second;
//   exchange, then the update's decisions (Theta < 0, NaN, the 200-iteration
//     rule, errors, convergence) on the same values on both lanes.
// So an iteration's dependent chain is one evaluation and the secant step,
// instead of two evaluations' worth.  The next iteration's evaluations are
// formed before the decision to run it and dropped if the loop ends.  Errors
// count where the reference loop raises them: the update's evolution-law error
// at once, an evaluation's when its iteration runs (the second only when the
// first passed).  A lone warp issues one FP64 instruction per ~70 cycles on
// this part, so the chain sets the solve time where few warps are left to run
// (the last row blocks of a step).
static __device__ PatchOut solve_lowv_pair(const PatchIn& p, double Dt, double eta, double alpha, int dr,
                                    double SwitchV, int& err) {
    int FLAG = 1, Instab = 0, Iteration = 0;
    double maxDiff = 10, crit = kConv;
    double V = p.VOld, Disp = p.DispOld, Friction = p.FrictionOld, Theta = p.ThetaOld;
    const double inv_sig = 1 / p.sigma;
    const bool skip = dr == 1 && alpha_term_zero(alpha, Dt, p.sigma, p.sigma_old, p.b);
    const Recip Rdc = recip_pre(p.Dc, p.rDc), Rdt = recip_pre(Dt, p.rDt), Ra = recip_pre(p.a, p.ra);
    const Recip R1e10 = {1e10, 1e-10, true};
    const int lane = threadIdx.x & 31, base = lane & ~1;
    const bool odd = (lane & 1) != 0;
    const unsigned pmask = 3u << base;
    // one evaluation at Vh: Theta, Disp and -- if Theta passed -- Friction and
    // the residual; the evolution law's and the inversion's errors apart
    double Th, Dh, Frh, FVh;
    int errT, errV, tc;
    auto evaluate = [&](double Vh) {
        errT = 0;
        errV = 0;
        FVh = 0;
        Frh = 0;
        const double Ah = div_by(Vh - p.VOld, Rdt);
        Th = evolution(p.ThetaOld, Dt, Vh, Rdc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, skip, errT);
        Dh = p.DispOld + (p.VOld + Vh) / 2 * Dt;
        tc = Th < 0 ? 1 : (isnan(Th) ? 2 : 0);
        if (tc == 0) {
            Frh = QDFN_FRICTION(Vh, Dh, Ah);
            FVh = Vh - QDFN_VEL(Frh, Th, errV);
        }
    };
    Iteration = 1;
    double VTest = V;
    double DV = div_by(VTest, R1e10);
    evaluate(odd ? VTest + DV : VTest);
    int fail0 = __shfl_sync(pmask, tc != 0 ? 1 : 0, base), fail1 = __shfl_sync(pmask, tc != 0 ? 1 : 0, base + 1);
    int err0 = __shfl_sync(pmask, errT ? errT : errV, base), err1 = __shfl_sync(pmask, errT ? errT : errV, base + 1);
    double FV = __shfl_sync(pmask, FVh, base), FV_DeV = __shfl_sync(pmask, FVh, base + 1);
    for (;;) {
        if (err0) err = err0;
        if (fail0) { QDFN_FAIL_A(); break; }
        if (err1) err = err1;        // the second evaluation runs only after the first passed
        if (fail1) { QDFN_FAIL_A(); break; }
        const double VTest2 = VTest + DV;
        V = VTest - FV * DV / (FV_DeV - FV);
        if (dr != 1 && V < 0)
            V = exp(jlog(VTest, err) - FV * jlog(VTest2 / VTest, err) / (FV_DeV - FV));
        const double DVn = div_by(V, R1e10);
        evaluate(odd ? V + DVn : V);
        maxDiff = fabs(VTest / V - 1);
        // the even lane's evaluation is the update at V
        Theta = Th;
        Disp = Dh;
        if (tc == 0) Friction = Frh;
        const int tcode = __shfl_sync(pmask, tc, base);
        const int erru = __shfl_sync(pmask, errT, base);
        const int e0 = __shfl_sync(pmask, errV, base);
        const int f1 = __shfl_sync(pmask, tc != 0 ? 1 : 0, base + 1);
        const int e1 = __shfl_sync(pmask, errT ? errT : errV, base + 1);
        const double FVn = __shfl_sync(pmask, FVh, base), FV_DeVn = __shfl_sync(pmask, FVh, base + 1);
        if (erru) err = erru;
        if (tcode == 1) { QDFN_FAIL_A(); break; }
        if (tcode == 2) { QDFN_THETA_NAN(); break; }
        if (Iteration % 200 == 0) { QDFN_ITER_CAP(); break; }
        if (err) break;
        if (!(maxDiff > crit)) break;
        Iteration++;
        VTest = V;
        DV = DVn;
        fail0 = 0; err0 = e0;
        fail1 = f1; err1 = e1;
        FV = FVn; FV_DeV = FV_DeVn;
    }
    PatchOut o;
    o.V = V; o.Friction = Friction; o.Disp = Disp; o.Theta = Theta; o.Dt = Dt;
    o.Instab = Instab; o.Flag = FLAG; o.Iterations = Iteration;
    return o;
}
#undef QDFN_FAIL_A
#undef QDFN_FRICTION
#undef QDFN_VEL
#undef QDFN_THETA_NAN
#undef QDFN_ITER_CAP
#undef QDFN_RESET

// InterpolateFromStressChange for one patch column.
__device__ __forceinline__ void interp_ext(int64_t nt, const double* __restrict__ t,
                                           const double* __restrict__ en,
                                           const double* __restrict__ es,
                                           const double* __restrict__ ep, int64_t N, int64_t i,
                                           double Time, double& dn, double& ds, double& dp) {
    int64_t idx = 0;
    for (int64_t k = 1; k <= nt; ++k)
        if (Time >= t[k - 1]) idx = k;
    if (idx == 0) {
        const double f = Time / t[0];
        dn = f * (en[i] - 0.0) + 0.0;
        ds = f * (es[i] - 0.0) + 0.0;
        dp = f * (ep[i] - 0.0) + 0.0;
    } else if (idx == nt) {
        dn = en[(nt - 1) * N + i];
        ds = es[(nt - 1) * N + i];
        dp = ep[(nt - 1) * N + i];
    } else {
        const double f = (Time - t[idx - 1]) / (t[idx] - t[idx - 1]);
        const int64_t lo = (idx - 1) * N + i, hi = idx * N + i;
        dn = f * (en[hi] - en[lo]) + en[lo];
        ds = f * (es[hi] - es[lo]) + es[lo];
        dp = f * (ep[hi] - ep[lo]) + ep[lo];
    }
}

}  // namespace sim
}  // namespace qdfn
