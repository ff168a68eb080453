// Oracle: the quasi-dynamic earthquake-cycle step loop, restated from
//   scripts/Functions_Solvers.jl
//     EvolutionLaw                 :2-15
//     Solver_HighV_D               :26-182
//     Solver_LowV_D                :185-327
//     SolveOneTimeStep             :334-380
//     InterpolateFromStressChange  :465-540
//   scripts/Functions_RSFDFN3DMain_D.jl  main    :2-324 (dense)
//   scripts/Functions_RSFDFN3DMain_H.jl  main_H  :2-383 (H-matrix: TLD divides by
//       -K_Self after the product, external stress is sampled at TOld, :241-261)
//   scripts/Functions_Hmatrix.jl
//     HmatSolver_Pararllel         :631-646, StiffnessTransitionToLoading :459-477
// Where the reference blocks on stdin (`readline()`, Main_D :255-258 after 100
// retries, Solvers :123-125 when Dt < 1e-10) this restatement behaves as if the
// user pressed Enter and continues; the hard caps below only turn a run that
// would loop for ever into an error code.
//
// TEST INFRASTRUCTURE ONLY (CPU oracle); not part of the shipped library.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "oracle.h"

namespace {

const double V0 = 1e-9;                 // Main_D :42
const double CONV = 1e-9;               // Main_D :46
const int64_t RETRY_CAP = 10000;        // retries of one step before giving up
const int64_t HIGHV_ITER_CAP = 40000;   // crit*10 every 100 its reaches Inf by ~31700

struct Err { int code = 0; };

inline double jlog(double x, Err& e) {
    if (x < 0) { e.code = ORACLE_ERR_DOMAIN; return NAN; }
    return std::log(x);
}

// EvolutionLaw (:2-15)
inline double evolution(double ThetaOld, double Dt, double V, double Dc, double alpha,
                        double sig, double sig_old, double b, int fast, int dr, Err& e) {
    if (dr == 1) {
        if (fast == 1) {
            double Const_T = V / Dc + alpha * (sig - sig_old) / Dt / b / sig;
            return (ThetaOld - 1 / Const_T) * std::exp(-V / Dc * Dt) + 1 / Const_T;
        }
        return (ThetaOld + Dt) / (1 + Dt * V / Dc + alpha * Dt * (sig - sig_old) / Dt / b / sig);
    }
    return ThetaOld - V * ThetaOld / Dc * jlog(V * ThetaOld / Dc, e) * Dt;
}

struct PatchIn {
    double DispOld, FrictionOld, ThetaOld, VOld, Friction0, a, b, Dc, K_Self, Omega, Mass;
    double sigma, TLD, dtau, sigma_old, tau0;
};
struct PatchOut {
    double V, Friction, Disp, Theta, Dt;
    int Instab, Flag;
};

// Solver_HighV_D (:26-182)
PatchOut solve_highv(const PatchIn& p, double Dt, double G, double rho, double alpha, int dr,
                     Err& e) {
    const double eta = G / 2 / std::sqrt(G / rho);
    int FLAG = 1, Instab = 0;
    int64_t Iteration = 0;
    double maxDiff = 10, crit = CONV;
    double DV = p.VOld / 100;
    double V = p.VOld / 1e10, Disp = p.DispOld, Friction = p.FrictionOld, Theta = p.ThetaOld;
    if (V < 0) V = 1e-100;
    auto reset = [&]() { V = p.VOld; Theta = p.ThetaOld; Friction = p.FrictionOld; Disp = p.DispOld; };
    while (maxDiff > crit) {
        Iteration++;
        if (Iteration > HIGHV_ITER_CAP) { e.code = ORACLE_ERR_NO_CONVERGE; break; }
        double VTest = V;
        Theta = evolution(p.ThetaOld, Dt, V, p.Dc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, e);
        if (Theta < 0) { Dt = Dt / 2; reset(); maxDiff = 0; FLAG = 0; break; }
        double Fr = p.Friction0 + p.a * jlog(V / V0, e) + p.b * jlog(Theta * V0 / p.Dc, e) +
                    eta / p.sigma * V - p.dtau / p.sigma;
        double F = p.TLD + (p.tau0 - Fr * p.sigma) / p.K_Self;
        Disp = (p.DispOld - F) * std::cos(p.Omega * Dt) + (p.VOld / p.Omega) * std::sin(p.Omega * Dt) + F;
        V = (Disp - p.DispOld) / Dt * 2 - p.VOld;
        double FOriginal = VTest - V;
        V = VTest + DV;
        double VTest2 = V;
        Theta = evolution(p.ThetaOld, Dt, V, p.Dc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, e);
        if (Theta < 0) { Dt = Dt / 2; reset(); maxDiff = 0; FLAG = 0; break; }
        Fr = p.Friction0 + p.a * jlog(V / V0, e) + p.b * jlog(Theta * V0 / p.Dc, e) +
             eta / p.sigma * V - p.dtau / p.sigma;
        F = p.TLD + (p.tau0 - Fr * p.sigma) / p.K_Self;
        Disp = (p.DispOld - F) * std::cos(p.Omega * Dt) + (p.VOld / p.Omega) * std::sin(p.Omega * Dt) + F;
        V = (Disp - p.DispOld) / Dt * 2 - p.VOld;
        double FUpdated = VTest2 - V;
        V = VTest - FOriginal * DV / (FUpdated - FOriginal);
        if (V < 0) {
            if (Dt > 1e-5) { Dt = Dt / 2; reset(); maxDiff = 0; FLAG = 0; }
            else { Dt = Dt / 2; Instab = 4; reset(); maxDiff = 0; FLAG = 0; }
        } else if (std::isnan(V)) {
            if (Dt > 1e-5) { Dt = Dt / 2; reset(); maxDiff = 0; FLAG = 0; }
            else { Dt = Dt / 2; Instab = 4; reset(); maxDiff = 0; FLAG = 0; }
        } else {
            Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
            Theta = evolution(p.ThetaOld, Dt, V, p.Dc, alpha, p.sigma, p.sigma_old, p.b, 1, dr, e);
            if (Theta < 0) { Dt = Dt / 2; reset(); maxDiff = 0; FLAG = 0; break; }
            Friction = p.Friction0 + p.a * jlog(V / V0, e) + p.b * jlog(Theta * V0 / p.Dc, e);
            maxDiff = std::fabs(VTest / V - 1);
            Instab = 0;
        }
        if (Iteration % 100 == 0) {
            if (Dt < 1e-5) { crit = crit * 10; Instab = 2; }
            else { Dt = Dt / 2; reset(); maxDiff = 0; FLAG = 0; }
        }
        if (e.code) break;
    }
    return PatchOut{V, Friction, Disp, Theta, Dt, Instab, FLAG};
}

// Solver_LowV_D (:185-327)
PatchOut solve_lowv(const PatchIn& p, double Dt, double G, double rho, double alpha, int dr,
                    double SwitchV, Err& e) {
    const double eta = G / 2 / std::sqrt(G / rho);
    int FLAG = 1, Instab = 0;
    int64_t Iteration = 0;
    double maxDiff = 10, crit = CONV;
    double V = p.VOld, Disp = p.DispOld, Friction = p.FrictionOld, Theta = p.ThetaOld;
    auto reset = [&]() { V = p.VOld; Theta = p.ThetaOld; Friction = p.FrictionOld; Disp = p.DispOld; };
    // failure handling shared by the Theta<0 / NaN checks (:210-222 etc.)
    auto fail_a = [&]() {
        if (Dt < SwitchV) { Instab = 3; reset(); FLAG = 0; }
        else if (p.VOld == 0) { reset(); FLAG = 1; }
        else { Dt = Dt / 2; reset(); maxDiff = 0; FLAG = 0; }
    };
    auto friction_of = [&](double Vx, double Dispx, double Accelx) {
        return 1 / p.sigma * (p.K_Self * (p.TLD - Dispx) + p.tau0 - eta * Vx + p.dtau - p.Mass * Accelx);
    };
    while (maxDiff > crit) {
        Iteration++;
        double VTest = V;
        double DV = VTest / 1e10;
        double Accel = (V - p.VOld) / Dt;
        Theta = evolution(p.ThetaOld, Dt, V, p.Dc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, e);
        if (Theta < 0 || std::isnan(Theta)) { fail_a(); break; }
        Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
        Friction = friction_of(V, Disp, Accel);
        double Vel = V0 * std::exp((Friction - p.Friction0 - p.b * jlog(V0 * Theta / p.Dc, e)) / p.a);
        double FV = VTest - Vel;
        V = V + DV;
        double VTest2 = V;
        Accel = (V - p.VOld) / Dt;
        Theta = evolution(p.ThetaOld, Dt, V, p.Dc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, e);
        if (Theta < 0 || std::isnan(Theta)) { fail_a(); break; }
        Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
        Friction = friction_of(V, Disp, Accel);
        Vel = V0 * std::exp((Friction - p.Friction0 - p.b * jlog(V0 * Theta / p.Dc, e)) / p.a);
        double FV_DeV = VTest2 - Vel;
        V = VTest - FV * DV / (FV_DeV - FV);
        if (dr != 1 && V < 0)
            V = std::exp(jlog(VTest, e) - FV * jlog(VTest2 / VTest, e) / (FV_DeV - FV));
        Accel = (V - p.VOld) / Dt;
        Disp = p.DispOld + (p.VOld + V) / 2 * Dt;
        Theta = evolution(p.ThetaOld, Dt, V, p.Dc, alpha, p.sigma, p.sigma_old, p.b, 0, dr, e);
        if (Theta < 0) { fail_a(); break; }
        if (std::isnan(Theta)) {
            if (p.VOld == 0) { reset(); FLAG = 1; }
            else if (Dt < 1e-3) {
                if (p.VOld < 1e-7) {
                    V = 0; Theta = p.ThetaOld + Dt; Friction = p.FrictionOld; Disp = p.DispOld;
                    maxDiff = 0; FLAG = 1;
                } else { Instab = 3; reset(); FLAG = 0; }
            } else { Dt = Dt / 2; reset(); maxDiff = 0; FLAG = 0; }
            break;
        }
        Friction = friction_of(V, Disp, Accel);
        maxDiff = std::fabs(VTest / V - 1);
        if (Iteration % 200 == 0) {
            if (Dt < 1e-4) { Instab = 3; reset(); FLAG = 0; break; }
            else if (Dt < 1e1) { crit = crit * 2; }
            else { Dt = Dt / 2; reset(); maxDiff = 0; FLAG = 0; }
            break;
        }
        if (e.code) break;
    }
    return PatchOut{V, Friction, Disp, Theta, Dt, Instab, FLAG};
}

// InterpolateFromStressChange (:465-540), one patch column
inline void interp_ext(const oracle_problem* p, double Time, int64_t i, double& dn, double& ds,
                       double& dp) {
    int64_t nt = p->n_ext, N = p->N;
    int64_t timeIdx = 0;  // 1-based index of the last sample <= Time, 0 if none
    for (int64_t k = 1; k <= nt; ++k)
        if (Time >= p->ext_t[k - 1]) timeIdx = k;
    if (timeIdx == 0) {
        double timediff = Time;
        double f = timediff / p->ext_t[0];
        dn = f * (p->ext_n[i] - 0.0) + 0.0;
        ds = f * (p->ext_s[i] - 0.0) + 0.0;
        dp = f * (p->ext_p[i] - 0.0) + 0.0;
    } else if (timeIdx == nt) {
        dn = p->ext_n[(nt - 1) * N + i];
        ds = p->ext_s[(nt - 1) * N + i];
        dp = p->ext_p[(nt - 1) * N + i];
    } else {
        double timediff = Time - p->ext_t[timeIdx - 1];
        double f = timediff / (p->ext_t[timeIdx] - p->ext_t[timeIdx - 1]);
        const int64_t lo = (timeIdx - 1) * N + i, hi = timeIdx * N + i;
        dn = f * (p->ext_n[hi] - p->ext_n[lo]) + p->ext_n[lo];
        ds = f * (p->ext_s[hi] - p->ext_s[lo]) + p->ext_s[lo];
        dp = f * (p->ext_p[hi] - p->ext_p[lo]) + p->ext_p[lo];
    }
}

}  // namespace

// ----------------------------------------------------------------------------
// elastic operators
struct oracle_operator {
    int64_t N;
    int hmat;
    int nthreads;
    std::vector<double> elsm, kn;   // dense
    std::vector<double> kself;
    // H
    int64_t nb = 0;
    std::vector<int64_t> range, rank_s, rank_n;
    std::vector<std::vector<double>> Us, Vts, Ds, Un, Vtn, Dn;
};

extern "C" oracle_operator* oracle_op_dense(int64_t N, const double* Ks, const double* Kn,
                                            int nthreads) {
    auto* op = new oracle_operator();
    op->N = N;
    op->hmat = 0;
    op->nthreads = nthreads > 0 ? nthreads : 1;
    op->elsm.assign((size_t)N * N, 0.0);
    op->kn.assign(Kn, Kn + (size_t)N * N);
    op->kself.assign(N, 0.0);
    for (int64_t i = 0; i < N; ++i) {  // Main_D :54-63
        op->kself[i] = std::fabs(Ks[i * N + i]);
        for (int64_t j = 0; j < N; ++j)
            op->elsm[i * N + j] = (i == j) ? 0.0 : Ks[i * N + j] / Ks[i * N + i];
    }
    return op;
}

extern "C" oracle_operator* oracle_op_hmat(int64_t N, int64_t nb, const int64_t* range,
                                           const int64_t* rank_s, const double* const* Us,
                                           const double* const* Vts, const double* const* Ds,
                                           const int64_t* rank_n, const double* const* Un,
                                           const double* const* Vtn, const double* const* Dn,
                                           int nthreads) {
    auto* op = new oracle_operator();
    op->N = N;
    op->hmat = 1;
    op->nthreads = nthreads > 0 ? nthreads : 1;
    op->nb = nb;
    op->range.assign(range, range + 4 * nb);
    op->rank_s.assign(rank_s, rank_s + nb);
    op->rank_n.assign(rank_n, rank_n + nb);
    op->Us.resize(nb); op->Vts.resize(nb); op->Ds.resize(nb);
    op->Un.resize(nb); op->Vtn.resize(nb); op->Dn.resize(nb);
    op->kself.assign(N, 0.0);
    for (int64_t b = 0; b < nb; ++b) {
        int64_t ns = range[4 * b + 1] - range[4 * b] + 1, nr = range[4 * b + 3] - range[4 * b + 2] + 1;
        if (rank_s[b] < 0) {
            op->Ds[b].assign(Ds[b], Ds[b] + nr * ns);
            // StiffnessTransitionToLoading :459-477: diagonal blocks give K_Self = -K_ii
            // and have their diagonal zeroed
            if (range[4 * b] == range[4 * b + 2] && range[4 * b + 1] == range[4 * b + 3]) {
                for (int64_t j = 0; j < nr; ++j) {
                    op->kself[range[4 * b] + j] = -op->Ds[b][j * ns + j];
                    op->Ds[b][j * ns + j] = 0.0;
                }
            }
        } else {
            op->Us[b].assign(Us[b], Us[b] + nr * rank_s[b]);
            op->Vts[b].assign(Vts[b], Vts[b] + rank_s[b] * ns);
        }
        if (rank_n[b] < 0) op->Dn[b].assign(Dn[b], Dn[b] + nr * ns);
        else {
            op->Un[b].assign(Un[b], Un[b] + nr * rank_n[b]);
            op->Vtn[b].assign(Vtn[b], Vtn[b] + rank_n[b] * ns);
        }
    }
    return op;
}

extern "C" void oracle_op_free(oracle_operator* op) { delete op; }

extern "C" void oracle_op_kself(const oracle_operator* op, double* kself) {
    std::memcpy(kself, op->kself.data(), sizeof(double) * op->N);
}

static void hmat_apply(const oracle_operator* op, int64_t b, int shear, const double* x,
                       double* y) {
    const int64_t s0 = op->range[4 * b], s1 = op->range[4 * b + 1];
    const int64_t r0 = op->range[4 * b + 2], r1 = op->range[4 * b + 3];
    const int64_t ns = s1 - s0 + 1, nr = r1 - r0 + 1;
    const int64_t rank = shear ? op->rank_s[b] : op->rank_n[b];
    if (rank < 0) {
        const double* Dm = shear ? op->Ds[b].data() : op->Dn[b].data();
        for (int64_t i = 0; i < nr; ++i) {
            double acc = 0;
            for (int64_t j = 0; j < ns; ++j) acc += Dm[i * ns + j] * x[s0 + j];
            y[r0 + i] += acc;
        }
    } else {
        const double* U = shear ? op->Us[b].data() : op->Un[b].data();
        const double* Vt = shear ? op->Vts[b].data() : op->Vtn[b].data();
        std::vector<double> t(rank, 0.0);
        for (int64_t k = 0; k < rank; ++k) {
            double acc = 0;
            for (int64_t j = 0; j < ns; ++j) acc += Vt[k * ns + j] * x[s0 + j];
            t[k] = acc;
        }
        for (int64_t i = 0; i < nr; ++i) {
            double acc = 0;
            for (int64_t k = 0; k < rank; ++k) acc += U[i * rank + k] * t[k];
            y[r0 + i] += acc;
        }
    }
}

extern "C" void oracle_op_apply(const oracle_operator* op, const double* D, double* tld,
                                double* knd) {
    const int64_t N = op->N;
    std::vector<double> x(N);
    for (int64_t j = 0; j < N; ++j) x[j] = 0.0 - D[j];  // Far_Load_Disp_Initial - DispOld
    if (!op->hmat) {
        // dgemv-like: rows in parallel, each dot product vectorised (the
        // reference's BLAS dgemv also reorders the sum)
#pragma omp parallel for schedule(static) num_threads(op->nthreads)
        for (int64_t i = 0; i < N; ++i) {
            const double* e = op->elsm.data() + i * N;
            const double* k = op->kn.data() + i * N;
            double a = 0, c = 0;
#pragma omp simd reduction(+ : a, c)
            for (int64_t j = 0; j < N; ++j) { a += e[j] * x[j]; c += k[j] * D[j]; }
            tld[i] = a;
            knd[i] = c;
        }
    } else {
        std::fill(tld, tld + N, 0.0);
        std::fill(knd, knd + N, 0.0);
        for (int64_t b = 0; b < op->nb; ++b) {
            hmat_apply(op, b, 1, x.data(), tld);
            hmat_apply(op, b, 0, D, knd);
        }
        for (int64_t i = 0; i < N; ++i) tld[i] = tld[i] / -op->kself[i];  // Main_H :241-243
    }
}

// ----------------------------------------------------------------------------
extern "C" void oracle_state_init(const oracle_problem* p, oracle_state* s) {
    const int64_t N = p->N;
    s->T = 0.0;
    s->dt = 1.0;
    s->step = 0;
    for (int64_t i = 0; i < N; ++i) {
        s->V[i] = p->V_i[i];
        s->D[i] = 0.0;
        s->theta[i] = p->theta_i[i];
        s->friction[i] = p->f_i[i];
        s->accel[i] = 0.0;
        s->sigma_old[i] = p->sigma0[i];
    }
}

extern "C" int oracle_run(const oracle_problem* p, const oracle_operator* op, oracle_state* s,
                          int64_t nsteps, int64_t record_step, int64_t max_rec, double* hist_t,
                          double* hist_dt, double* hist_V, double* hist_D, double* hist_theta,
                          double* hist_sigma, int64_t* n_rec, int nthreads) {
    const int64_t N = p->N, Nl = p->Nload, Ns = N - Nl;
    const int nth = nthreads > 0 ? nthreads : 1;
    std::vector<double> kself(N), omega(N), F0(N), tau0(N);
    oracle_op_kself(op, kself.data());
    Err gerr;
    for (int64_t i = 0; i < N; ++i) {
        if (kself[i] / p->mass[i] < 0) return ORACLE_ERR_DOMAIN;
        omega[i] = std::sqrt(kself[i] / p->mass[i]);
        tau0[i] = p->sigma0[i] * p->f_i[i];  // InitialShearStress
        F0[i] = p->f_i[i] - p->a[i] * jlog(p->V_i[i] / V0, gerr) -
                p->b[i] * jlog(p->theta_i[i] * V0 / p->Dc[i], gerr);
    }
    if (gerr.code) return gerr.code;
    std::vector<int64_t> unstable;
    for (int64_t i = 0; i < N; ++i)
        if (p->a[i] - p->b[i] < 0) unstable.push_back(i);
    const bool by_unstable = !unstable.empty();
    const double G = p->G, rho = p->rho;
    std::vector<double> tld(N), knd(N), sig_i(N), dsn(N, 0.0), dss(N, 0.0), dsp(N, 0.0);
    std::vector<double> Vn(N), Fn(N), Dn(N), Thn(N), Sn(N), DtAll(N);
    std::vector<int> Switch(N), Instab(N), Flag(N);
    double Dt = s->dt;
    for (int64_t it = 0; it < nsteps; ++it) {
        const int64_t gstep = s->step + 1;
        const double TOld = s->T;
        for (int64_t i = 0; i < N; ++i) Switch[i] = s->V[i] > p->switch_v ? 1 : 0;
        // time step control (Main_D :163-187)
        double Vmax = -INFINITY, Dtmin = INFINITY;
        bool vnan = false, any = false;
        auto consider = [&](int64_t i) {
            double v = s->V[i];
            if (std::isnan(v)) vnan = true;
            else if (v > Vmax) Vmax = v;
            double q = std::fabs(v / s->accel[i]);
            if (!std::isnan(q) && q != 0) { any = true; if (q < Dtmin) Dtmin = q; }
        };
        if (by_unstable) for (int64_t i : unstable) consider(i);
        else for (int64_t i = 0; i < Ns; ++i) consider(i);
        if (vnan) Vmax = NAN;
        if (!any) return ORACLE_ERR_EMPTY;
        Dtmin = Dtmin / p->dt_cut;
        double DtRef;
        if (Vmax > p->switch_v) DtRef = p->rupture_dt;
        else if (Dtmin > p->max_dt) DtRef = p->max_dt;
        else DtRef = Dtmin;
        if (DtRef <= p->rupture_dt) Dt = DtRef;
        else if (Dt < DtRef / 1.2) Dt = Dt * 1.2;
        else Dt = DtRef;
        oracle_op_apply(op, s->D, tld.data(), knd.data());
        int64_t Iteration = 0;
        while (true) {
            Iteration++;
            if (Iteration > RETRY_CAP) return ORACLE_ERR_RETRIES;
            const double tq = p->interp_at_told ? TOld : TOld + Dt;
            for (int64_t i = 0; i < N; ++i) {
                if (p->n_ext > 0) interp_ext(p, tq, i, dsn[i], dss[i], dsp[i]);
                double sg = knd[i] + p->sigma0[i] + dsn[i];
                sig_i[i] = sg < p->sigma_min ? p->sigma_min : sg;
            }
            std::vector<int> errs(nth, 0);
            const double DtOld = Dt;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nth)
            for (int64_t i = 0; i < Ns; ++i) {
                PatchIn pin{s->D[i], s->friction[i], s->theta[i], s->V[i], F0[i], p->a[i],
                            p->b[i], p->Dc[i], kself[i], omega[i], p->mass[i], sig_i[i],
                            0.0 + tld[i], dss[i], s->sigma_old[i], tau0[i]};
                Err e;
                PatchOut o = Switch[i] == 1
                                 ? solve_highv(pin, DtOld, G, rho, p->alpha_evo, p->evolution_dr, e)
                                 : solve_lowv(pin, DtOld, G, rho, p->alpha_evo, p->evolution_dr,
                                              p->switch_v, e);
                Vn[i] = o.V; Fn[i] = o.Friction; Dn[i] = o.Disp; Thn[i] = o.Theta;
                Sn[i] = sig_i[i]; DtAll[i] = o.Dt; Instab[i] = o.Instab; Flag[i] = o.Flag;
                if (e.code) {
#pragma omp critical
                    gerr.code = e.code;
                }
            }
            if (gerr.code) return gerr.code;
            for (int64_t i = Ns; i < N; ++i) {  // loading faults (Solvers :370-377)
                Vn[i] = p->V_const[i];
                Fn[i] = s->friction[i];
                Dn[i] = s->D[i] + Vn[i] * Dt;
                Thn[i] = s->theta[i];
                Sn[i] = 1e10;
                DtAll[i] = Dt;
                Instab[i] = 0;
                Flag[i] = 1;
            }
            int minflag = 1;
            for (int64_t i = 0; i < N; ++i) minflag = std::min(minflag, Flag[i]);
            if (minflag == 0) {
                double m = INFINITY;
                for (int64_t i = 0; i < N; ++i) m = std::min(m, DtAll[i]);
                Dt = m;
                for (int64_t i = 0; i < N; ++i) {
                    if (Instab[i] == 3) Switch[i] = 1;
                    else if (Instab[i] == 4) { Switch[i] = 0; Dt = 1e-3; }
                }
                continue;
            }
            break;
        }
        {
            double m = INFINITY;
            for (int64_t i = 0; i < N; ++i) m = std::min(m, DtAll[i]);
            Dt = m;
        }
        if (record_step > 0 && gstep % record_step == 0 && n_rec && *n_rec < max_rec) {
            int64_t r = *n_rec;
            if (hist_t) hist_t[r] = TOld;
            if (hist_dt) hist_dt[r] = Dt;
            for (int64_t i = 0; i < N; ++i) {
                if (hist_V) hist_V[r * N + i] = Vn[i];
                if (hist_D) hist_D[r * N + i] = Dn[i];
                if (hist_theta) hist_theta[r * N + i] = Thn[i];
                if (hist_sigma) hist_sigma[r * N + i] = Sn[i];
            }
            *n_rec = r + 1;
        }
        s->T = TOld + Dt;
        for (int64_t i = 0; i < N; ++i) {
            s->accel[i] = (Vn[i] - s->V[i]) / Dt;
            s->D[i] = Dn[i];
            s->theta[i] = Thn[i];
            s->V[i] = Vn[i];
            s->friction[i] = Fn[i];
            s->sigma_old[i] = Sn[i];
        }
        s->dt = Dt;
        s->step = gstep;
    }
    return ORACLE_OK;
}
