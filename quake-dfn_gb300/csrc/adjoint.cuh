// Local Jacobian of one patch's converged time step, for the adjoint.
//
// An accepted step leaves every non-loading patch at the root V* of its
// solver's residual (the secant loops of scripts/Functions_Solvers.jl stop at
// |V_test/V - 1| < 1e-9):
//   low velocity  (Solver_LowV_D, :185-327)
//     g(V) = V - V0 exp((mu(V) - F0 - b ln(V0 theta_s(V)/Dc)) / a)
//     mu(V) = [K (TLD - D(V)) + tau0 - eta V + dtau - M (V - V_old)/dt] / sigma
//   high velocity (Solver_HighV_D, :26-182)
//     g(V) = V - W(V),  W = 2 (X(V) - D_old)/dt - V_old
//     X = (D_old - F) cos(Omega dt) + (V_old/Omega) sin(Omega dt) + F
//     F = TLD + (tau0 - mu_rad sigma)/K
//     mu_rad = F0 + a ln(V/V0) + b ln(theta_f(V) V0/Dc) + eta V/sigma - dtau/sigma
// with D(V) = D_old + (V_old + V) dt/2 and the aging law theta_s (slow form)
// or theta_f (semi-analytic fast form), or the slip law (EvolutionLaw, :2-15,
// Alpha_Evo = 0).  The step's outputs are V*, D(V*), theta(V*) and
// Accel = (V* - V_old)/dt.  By the implicit-function theorem
// dV*/dx = -g_x / g_V, so the local Jacobian of the outputs with respect to the
// step's inputs x = (D_old, V_old, theta_old, TLD, sigma, dtau, dt, a, b, Dc)
// follows from one forward-mode evaluation of g and of the outputs at V*
// (dual numbers, direction 0 = V).  F0 = f_i - a ln(V_i/V0) - b ln(theta_i V0/Dc)
// (Main_D :80) carries the parameters' dependence through the run constants.
#pragma once
#include "dual.cuh"
#include "sim_device.cuh"

namespace qdfn {
namespace adj {

constexpr int kDirs = 11;   // V, D_old, V_old, theta_old, TLD, sigma, dtau, dt, a, b, Dc
enum { dV = 0, dDold, dVold, dThold, dTLD, dSig, dDtau, dDt, dA, dB, dDc };

using D11 = ad::Dual<kDirs>;

__host__ __device__ inline double f_exp(double x) { return ::exp(x); }
__host__ __device__ inline double f_log(double x) { return ::log(x); }
__host__ __device__ inline double f_cos(double x) { return ::cos(x); }
__host__ __device__ inline double f_sin(double x) { return ::sin(x); }
template <int K>
__host__ __device__ inline ad::Dual<K> f_exp(const ad::Dual<K>& x) { return ad::exp(x); }
template <int K>
__host__ __device__ inline ad::Dual<K> f_log(const ad::Dual<K>& x) { return ad::log(x); }
template <int K>
__host__ __device__ inline ad::Dual<K> f_cos(const ad::Dual<K>& x) { return ad::cos(x); }
template <int K>
__host__ __device__ inline ad::Dual<K> f_sin(const ad::Dual<K>& x) { return ad::sin(x); }

// EvolutionLaw with Alpha_Evo = 0: aging law (slow: fast1_slow0 = 0, or the
// semi-analytic fast form) or, for evolution_dr != 1, the slip law
template <class T>
__host__ __device__ inline T theta_law(const T& th_old, const T& dt, const T& V, const T& Dc, int fast,
                                       int dr) {
    if (dr == 1) {
        if (fast) {
            const T C = V / Dc;
            return (th_old - 1.0 / C) * f_exp(-V / Dc * dt) + 1.0 / C;
        }
        return (th_old + dt) / (1.0 + dt * V / Dc);
    }
    return th_old - V * th_old / Dc * f_log(V * th_old / Dc) * dt;
}

// Everything about one patch the local derivatives need.
struct PatchX {
    double V;                                  // the accepted V*
    double Dold, Vold, thold, TLD, sig, dtau, dt, a, b, Dc;
    double F0, la, lth;                        // F0 and ln(V_i/V0), ln(theta_i V0/Dc) (its derivatives)
    double K, M, Omega, eta, tau0;
    int high, dr;
};

// Residual and outputs (D, theta, Accel) at V*, with derivatives in the 11
// directions.
__host__ __device__ inline void local_eval(const PatchX& x, D11& g, D11& D, D11& th, D11& A) {
    const D11 V = D11::var(x.V, dV), Dold = D11::var(x.Dold, dDold), Vold = D11::var(x.Vold, dVold);
    const D11 thold = D11::var(x.thold, dThold), TLD = D11::var(x.TLD, dTLD), sig = D11::var(x.sig, dSig);
    const D11 dtau = D11::var(x.dtau, dDtau), dt = D11::var(x.dt, dDt);
    const D11 a = D11::var(x.a, dA), b = D11::var(x.b, dB), Dc = D11::var(x.Dc, dDc);
    D11 F0(x.F0);                              // dF0/da = -la, dF0/db = -lth, dF0/dDc = b/Dc
    F0.d[dA] = -x.la;
    F0.d[dB] = -x.lth;
    F0.d[dDc] = x.b / x.Dc;
    const double V0 = sim::kV0;
    D = Dold + (Vold + V) / 2.0 * dt;
    A = (V - Vold) / dt;
    if (!x.high) {
        th = theta_law(thold, dt, V, Dc, 0, x.dr);
        const D11 mu = 1.0 / sig * (x.K * (TLD - D) + x.tau0 - x.eta * V + dtau - x.M * A);
        const D11 Vel = V0 * f_exp((mu - F0 - b * f_log(V0 * th / Dc)) / a);
        g = V - Vel;
    } else {
        th = theta_law(thold, dt, V, Dc, 1, x.dr);
        const D11 mu_rad = F0 + a * f_log(V / V0) + b * f_log(th * V0 / Dc) + x.eta / sig * V - dtau / sig;
        const D11 F = TLD + (x.tau0 - mu_rad * sig) / x.K;
        const D11 X = (Dold - F) * f_cos(x.Omega * dt) + (Vold / x.Omega) * f_sin(x.Omega * dt) + F;
        const D11 W = (X - Dold) / dt * 2.0 - Vold;
        g = V - W;
    }
}

// Vector-Jacobian product of one patch's step: given the adjoints of its
// outputs (lV, lD, lth, lA), the adjoints of its inputs in the 10 input
// directions (index k - 1 of out[] for direction k = 1..10).  Returns false
// when the residual's derivative g_V is zero or not finite.
__host__ __device__ inline bool local_vjp(const PatchX& x, double lV, double lD, double lth, double lA,
                                          double out[kDirs - 1]) {
    D11 g, D, th, A;
    local_eval(x, g, D, th, A);
    const double gV = g.d[dV];
    if (!(gV != 0.0) || !isfinite(gV)) return false;
    // dy/dx_k = y_k + y_V s_k with s_k = -g_k / g_V
    const double w = lV + lD * D.d[dV] + lth * th.d[dV] + lA * A.d[dV];
    for (int k = 1; k < kDirs; ++k) {
        const double s = -g.d[k] / gV;
        out[k - 1] = lD * D.d[k] + lth * th.d[k] + lA * A.d[k] + w * s;
    }
    return true;
}

}  // namespace adj
}  // namespace qdfn
