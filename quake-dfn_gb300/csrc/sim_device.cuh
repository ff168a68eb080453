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

__device__ __forceinline__ double evolution(double ThetaOld, double Dt, double V, double Dc,
                                            double alpha, double sig, double sig_old, double b,
                                            int fast, int dr, int& err) {
    if (dr == 1) {
        const bool skip = alpha_term_zero(alpha, Dt, sig, sig_old, b);
        if (fast) {
            const double vd = V / Dc;
            const double Const_T = (skip && vd != 0.0) ? vd : vd + alpha * (sig - sig_old) / Dt / b / sig;
            // (-V)/Dc == -(V/Dc) exactly, so the quotient is reused
            return (ThetaOld - 1 / Const_T) * exp(-vd * Dt) + 1 / Const_T;
        }
        const double den0 = 1 + Dt * V / Dc;
        const double den = (skip && den0 != 0.0) ? den0 : den0 + alpha * Dt * (sig - sig_old) / Dt / b / sig;
        return (ThetaOld + Dt) / den;
    }
    return ThetaOld - V * ThetaOld / Dc * jlog(V * ThetaOld / Dc, err) * Dt;
}

// Semi-analytic harmonic-oscillator update with a secant iteration on V.
__device__ PatchOut solve_highv(const PatchIn& p, double Dt, double eta, double alpha, int dr,
                                int& err) {
    int FLAG = 1, Instab = 0, Iteration = 0;
    double maxDiff = 10, crit = kConv;
    const double DV = p.VOld / 100;
    double V = p.VOld / 1e10, Disp = p.DispOld, Friction = p.FrictionOld, Theta = p.ThetaOld;
    if (V < 0) V = 1e-100;
#define QDFN_RESET() do { V = p.VOld; Theta = p.ThetaOld; Friction = p.FrictionOld; Disp = p.DispOld; } while (0)
    while (maxDiff > crit) {
        Iteration++;
        if (Iteration > kHighVIterCap) { err = QDFN_ERR_NO_CONVERGE; break; }
        const double VTest = V;
        Theta = evolution(p.ThetaOld, Dt, V, p.Dc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, err);
        if (Theta < 0) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; break; }
        const double cO = cos(p.Omega * Dt), sO = sin(p.Omega * Dt);
        double Fr = p.Friction0 + p.a * jlog(V / kV0, err) + p.b * jlog(Theta * kV0 / p.Dc, err) +
                    eta / p.sigma * V - p.dtau / p.sigma;
        double F = p.TLD + (p.tau0 - Fr * p.sigma) / p.K_Self;
        Disp = (p.DispOld - F) * cO + (p.VOld / p.Omega) * sO + F;
        V = (Disp - p.DispOld) / Dt * 2 - p.VOld;
        const double FOriginal = VTest - V;
        V = VTest + DV;
        const double VTest2 = V;
        Theta = evolution(p.ThetaOld, Dt, V, p.Dc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, err);
        if (Theta < 0) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; break; }
        Fr = p.Friction0 + p.a * jlog(V / kV0, err) + p.b * jlog(Theta * kV0 / p.Dc, err) +
             eta / p.sigma * V - p.dtau / p.sigma;
        F = p.TLD + (p.tau0 - Fr * p.sigma) / p.K_Self;
        Disp = (p.DispOld - F) * cO + (p.VOld / p.Omega) * sO + F;
        V = (Disp - p.DispOld) / Dt * 2 - p.VOld;
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
            Theta = evolution(p.ThetaOld, Dt, V, p.Dc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, err);
            if (Theta < 0) { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; break; }
            Friction = p.Friction0 + p.a * jlog(V / kV0, err) + p.b * jlog(Theta * kV0 / p.Dc, err);
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
    o.Instab = Instab; o.Flag = FLAG;
    return o;
}

// Implicit trapezoidal update with a secant iteration on V and the friction
// inversion V = V0 exp((mu - mu0 - b ln(V0 theta/Dc))/a), all in FP64.
__device__ PatchOut solve_lowv(const PatchIn& p, double Dt, double eta, double alpha, int dr,
                               double SwitchV, int& err) {
    int FLAG = 1, Instab = 0, Iteration = 0;
    double maxDiff = 10, crit = kConv;
    double V = p.VOld, Disp = p.DispOld, Friction = p.FrictionOld, Theta = p.ThetaOld;
    const double inv_sig = 1 / p.sigma;
#define QDFN_FAIL_A()                                                      \
    do {                                                                   \
        if (Dt < SwitchV) { Instab = 3; QDFN_RESET(); FLAG = 0; }          \
        else if (p.VOld == 0) { QDFN_RESET(); FLAG = 1; }                  \
        else { Dt = Dt / 2; QDFN_RESET(); maxDiff = 0; FLAG = 0; }         \
    } while (0)
#define QDFN_FRICTION(Vx, Dx, Ax) \
    (inv_sig * (p.K_Self * (p.TLD - (Dx)) + p.tau0 - eta * (Vx) + p.dtau - p.Mass * (Ax)))
    while (maxDiff > crit) {
        Iteration++;
        const double VTest = V;
        const double DV = VTest / 1e10;
        double Accel = (V - p.VOld) / Dt;
        Theta = evolution(p.ThetaOld, Dt, V, p.Dc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, err);
        if (Theta < 0 || isnan(Theta)) { QDFN_FAIL_A(); break; }
        Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
        Friction = QDFN_FRICTION(V, Disp, Accel);
        double Vel = kV0 * exp((Friction - p.Friction0 - p.b * jlog(kV0 * Theta / p.Dc, err)) / p.a);
        const double FV = VTest - Vel;
        V = V + DV;
        const double VTest2 = V;
        Accel = (V - p.VOld) / Dt;
        Theta = evolution(p.ThetaOld, Dt, V, p.Dc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, err);
        if (Theta < 0 || isnan(Theta)) { QDFN_FAIL_A(); break; }
        Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
        Friction = QDFN_FRICTION(V, Disp, Accel);
        Vel = kV0 * exp((Friction - p.Friction0 - p.b * jlog(kV0 * Theta / p.Dc, err)) / p.a);
        const double FV_DeV = VTest2 - Vel;
        V = VTest - FV * DV / (FV_DeV - FV);
        if (dr != 1 && V < 0)
            V = exp(jlog(VTest, err) - FV * jlog(VTest2 / VTest, err) / (FV_DeV - FV));
        Accel = (V - p.VOld) / Dt;
        Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
        Theta = evolution(p.ThetaOld, Dt, V, p.Dc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, err);
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
    o.Instab = Instab; o.Flag = FLAG;
    return o;
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
