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
// correctly rounded (one IEEE division per solve), q0 = x*y is within an ulp
// of x/d, the remainder r = x - q0*d is exact in one FMA, and q0 + r*y rounds
// to x/d (Markstein's correction step: P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990).  Three FP64 operations instead of the eight of a full division.  The
// sum is formed as -fma(-r, y, -q0) so that x = -0 keeps its sign.  Operands
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
__device__ __noinline__ double full_div(double x, double d) { return x / d; }
__device__ __forceinline__ double div_by(double x, const Recip& R) {
    const double q0 = x * R.y;
    const double r = fma(-q0, R.d, x);
    const double q = -fma(-r, R.y, -q0);
    const bool zero = (__double_as_longlong(x) << 1) == 0;
    const bool fast = R.ok && (zero || (in_safe_range(exp_field(x)) && in_safe_range(exp_field(q0))));
    if (fast) return q;
    return full_div(x, R.d);   // out of line: never evaluated speculatively
}

// The alpha terms as written in the reference.  Out of line so that the
// compiler cannot evaluate them speculatively next to the (usual) skip path.
__device__ __noinline__ double alpha_term_fast(double alpha, double sig, double sig_old, double Dt,
                                               double b) {
    return alpha * (sig - sig_old) / Dt / b / sig;
}
__device__ __noinline__ double alpha_term_slow(double alpha, double sig, double sig_old, double Dt,
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
__device__ PatchOut solve_highv(const PatchIn& p, double Dt, double eta, double alpha, int dr,
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
    const Recip Rdc = recip(p.Dc), Rdt = recip(Dt);
#define QDFN_RESET() do { V = p.VOld; Theta = p.ThetaOld; Friction = p.FrictionOld; Disp = p.DispOld; } while (0)
    while (maxDiff > crit) {
        Iteration++;
        if (Iteration > kHighVIterCap) { err = QDFN_ERR_NO_CONVERGE; break; }
        const double VTest = V;
        Theta = evolution(p.ThetaOld, Dt, V, Rdc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, skip, err);
        if (Theta < 0) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; break; }
        double Fr = p.Friction0 + p.a * jlog(V / kV0, err) + p.b * jlog(div_by(Theta * kV0, Rdc), err) +
                    eta / p.sigma * V - p.dtau / p.sigma;
        double F = p.TLD + (p.tau0 - Fr * p.sigma) / p.K_Self;
        Disp = (p.DispOld - F) * cO + (p.VOld / p.Omega) * sO + F;
        V = div_by(Disp - p.DispOld, Rdt) * 2 - p.VOld;
        const double FOriginal = VTest - V;
        V = VTest + DV;
        const double VTest2 = V;
        Theta = evolution(p.ThetaOld, Dt, V, Rdc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, skip, err);
        if (Theta < 0) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; break; }
        Fr = p.Friction0 + p.a * jlog(V / kV0, err) + p.b * jlog(div_by(Theta * kV0, Rdc), err) +
             eta / p.sigma * V - p.dtau / p.sigma;
        F = p.TLD + (p.tau0 - Fr * p.sigma) / p.K_Self;
        Disp = (p.DispOld - F) * cO + (p.VOld / p.Omega) * sO + F;
        V = div_by(Disp - p.DispOld, Rdt) * 2 - p.VOld;
        const double FUpdated = VTest2 - V;
        V = VTest - FOriginal * DV / (FUpdated - FOriginal);
        if (V < 0 || isnan(V)) {
            // :87-134 -- both the negative and the NaN branch halve Dt; below
            // Dt = 1e-5 they also mark Instability = 4 (the V<0 branch) or do so
            // after printing (the NaN branch)
            if (Dt > 1e-5) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; }
            else { Dt = Dt / 2; Instab = 4; QDFN_RESET(); maxDiff = 0; FLAG = 0; }
        } else {
            Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
            Theta = evolution(p.ThetaOld, Dt, V, Rdc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, skip, err);
            if (Theta < 0) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; break; }
            Friction = p.Friction0 + p.a * jlog(V / kV0, err) + p.b * jlog(div_by(Theta * kV0, Rdc), err);
            maxDiff = fabs(VTest / V - 1);
            Instab = 0;
        }
        if (Iteration % 100 == 0) {
            if (Dt < 1e-5) { crit = crit * 10; Instab = 2; }
            else { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; }
        }
        if (err) break;
    }
    PatchOut o;
    o.V = V; o.Friction = Friction; o.Disp = Disp; o.Theta = Theta; o.Dt = Dt;
    o.Instab = Instab; o.Flag = FLAG; o.Iterations = Iteration;
    return o;
}

// Implicit trapezoidal update with a secant iteration on V and the friction
// inversion V = V0 exp((mu - mu0 - b ln(V0 theta/Dc))/a), all in FP64.
//
// kPair: the solve of one patch runs on a lane pair (lanes 2k, 2k+1 of the
// warp, same inputs).  The two evaluations of the secant step -- at V and at
// V + DV -- are independent, so lane 2k evaluates at V and lane 2k+1 at V + DV,
// and they exchange the residuals; everything else runs on both lanes alike.
// The arithmetic and every branch decision are those of the one-lane solve
// (an evaluation's error counts only when the one before it passed, as in the
// sequential order), so both return the same result.  A lone warp issues one
// FP64 instruction per ~70 cycles on this part, so halving the dependent chain
// of an iteration matters where few warps are left to run (the last row
// blocks of a step).
template <bool kPair>
__device__ PatchOut solve_lowv_t(const PatchIn& p, double Dt, double eta, double alpha, int dr,
                                 double SwitchV, int& err) {
    int FLAG = 1, Instab = 0, Iteration = 0;
    double maxDiff = 10, crit = kConv;
    double V = p.VOld, Disp = p.DispOld, Friction = p.FrictionOld, Theta = p.ThetaOld;
    const double inv_sig = 1 / p.sigma;
    const bool skip = dr == 1 && alpha_term_zero(alpha, Dt, p.sigma, p.sigma_old, p.b);
    // divisors fixed for the solve (Dt only changes on the way out of the loop);
    // 1e-10 is the correctly rounded reciprocal of 1e10 (both are 10^-10 rounded)
    const Recip Rdc = recip(p.Dc), Rdt = recip(Dt), Ra = recip(p.a);
    const Recip R1e10 = {1e10, 1e-10, true};
#define QDFN_FAIL_A()                                                    \
    do {                                                                   \
        if (Dt < SwitchV) { Instab = 3; QDFN_RESET(); FLAG = 0; }          \
        else if (p.VOld == 0) { QDFN_RESET(); FLAG = 1; }                  \
        else { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; }         \
    } while (0)
#define QDFN_FRICTION(Vx, Dx, Ax) \
    (inv_sig * (p.K_Self * (p.TLD - (Dx)) + p.tau0 - eta * (Vx) + p.dtau - p.Mass * (Ax)))
    const int lane = threadIdx.x & 31, base = lane & ~1;
    const unsigned pmask = 3u << base;
    (void)lane; (void)pmask;
    while (maxDiff > crit) {
        Iteration++;
        const double VTest = V;
        const double DV = div_by(VTest, R1e10);
        double FV, FV_DeV, VTest2, Accel;
        if constexpr (!kPair) {
            Accel = div_by(V - p.VOld, Rdt);
            Theta = evolution(p.ThetaOld, Dt, V, Rdc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, skip, err);
            if (Theta < 0 || isnan(Theta)) { QDFN_FAIL_A(); break; }
            Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
            Friction = QDFN_FRICTION(V, Disp, Accel);
            double Vel = kV0 * exp(div_by(Friction - p.Friction0 - p.b * jlog(div_by(kV0 * Theta, Rdc), err), Ra));
            FV = VTest - Vel;
            V = V + DV;
            VTest2 = V;
            Accel = div_by(V - p.VOld, Rdt);
            Theta = evolution(p.ThetaOld, Dt, V, Rdc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, skip, err);
            if (Theta < 0 || isnan(Theta)) { QDFN_FAIL_A(); break; }
            Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
            Friction = QDFN_FRICTION(V, Disp, Accel);
            Vel = kV0 * exp(div_by(Friction - p.Friction0 - p.b * jlog(div_by(kV0 * Theta, Rdc), err), Ra));
            FV_DeV = VTest2 - Vel;
        } else {
            // this lane's evaluation point: V (even lane) or V + DV (odd lane)
            const double Vh = (lane & 1) ? VTest + DV : VTest;
            int errh = 0;
            const double Ah = div_by(Vh - p.VOld, Rdt);
            const double Th = evolution(p.ThetaOld, Dt, Vh, Rdc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, skip, errh);
            const int failh = (Th < 0 || isnan(Th)) ? 1 : 0;
            double FVh = 0;
            if (!failh) {
                const double Dh = p.DispOld + (p.VOld + Vh) / 2 * Dt;
                const double Frh = QDFN_FRICTION(Vh, Dh, Ah);
                const double Velh = kV0 * exp(div_by(Frh - p.Friction0 - p.b * jlog(div_by(kV0 * Th, Rdc), errh), Ra));
                FVh = Vh - Velh;
            }
            const int fail0 = __shfl_sync(pmask, failh, base), fail1 = __shfl_sync(pmask, failh, base + 1);
            const int err0 = __shfl_sync(pmask, errh, base), err1 = __shfl_sync(pmask, errh, base + 1);
            FV = __shfl_sync(pmask, FVh, base);
            FV_DeV = __shfl_sync(pmask, FVh, base + 1);
            if (err0) err = err0;
            if (fail0) { QDFN_FAIL_A(); break; }
            if (err1) err = err1;        // the second evaluation runs only after the first passed
            if (fail1) { QDFN_FAIL_A(); break; }
            VTest2 = VTest + DV;
        }
        V = VTest - FV * DV / (FV_DeV - FV);
        if (dr != 1 && V < 0)
            V = exp(jlog(VTest, err) - FV * jlog(VTest2 / VTest, err) / (FV_DeV - FV));
        Accel = div_by(V - p.VOld, Rdt);
        Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
        Theta = evolution(p.ThetaOld, Dt, V, Rdc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, skip, err);
        if (Theta < 0) { QDFN_FAIL_A(); break; }
        if (isnan(Theta)) {
            if (p.VOld == 0) { QDFN_RESET(); FLAG = 1; }
            else if (Dt < 1e-3) {
                if (p.VOld < 1e-7) {
                    V = 0; Theta = p.ThetaOld + Dt; Friction = p.FrictionOld; Disp = p.DispOld;
                    maxDiff = 0; FLAG = 1;
                } else { Instab = 3; QDFN_RESET(); FLAG = 0; }
            } else { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; }
            break;
        }
        Friction = QDFN_FRICTION(V, Disp, Accel);
        maxDiff = fabs(VTest / V - 1);
        if (Iteration % 200 == 0) {
            if (Dt < 1e-4) { Instab = 3; QDFN_RESET(); FLAG = 0; break; }
            else if (Dt < 1e1) { crit = crit * 2; }
            else { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; }
            break;
        }
        if (err) break;
    }
#undef QDFN_FAIL_A
#undef QDFN_FRICTION
#undef QDFN_RESET
    PatchOut o;
    o.V = V; o.Friction = Friction; o.Disp = Disp; o.Theta = Theta; o.Dt = Dt;
    o.Instab = Instab; o.Flag = FLAG; o.Iterations = Iteration;
    return o;
}
__device__ __forceinline__ PatchOut solve_lowv(const PatchIn& p, double Dt, double eta, double alpha, int dr,
                                               double SwitchV, int& err) {
    return solve_lowv_t<false>(p, Dt, eta, alpha, dr, SwitchV, err);
}

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
