"""The mixed-precision contract against the FP64 oracle: with the elastic
operator stored in FP32 (FP64 state, friction inversion, time and step
control), the relative slip error max|D - D_oracle| / max|D_oracle| stays at
or below 1e-6 at matched simulated times (every oracle step of the
interseismic horizon, the GPU slip interpolated in time) -- until the first patch accelerates past twice the
largest starting slip rate (the onset of nucleation).  From there on the trajectories are
unstable: a nucleating patch's slip-rate runaway amplifies any perturbation
exponentially (a 1e-15 perturbation of the FP64 operator already grows to
~1e-7 in slip through the first event of the single fault), so the contract is
stated over that horizon, which each test measures from the oracle's own run
and requires to be long.

Runs: the C1 single fault (the dense FP32 product, one instance), a reduced C2
network (dense FP32, 4 friction draws in one context), and an H-matrix network
(FP32 blocks against the oracle's FP64 product of the same blocks).  The BF16
hi+lo operator (~16 significant bits) is held to its own, stated bound."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
G, NU = 32e9, 0.25


def pre_nucleation_records(hist, ns, v_start, factor=2.0):
    """Leading records in which no patch among the first `ns` has accelerated
    past `factor` times the largest starting slip rate `v_start`."""
    vmax = np.max(hist["V"][:, :ns], axis=1)
    bad = np.nonzero(vmax > factor * v_start)[0]
    return int(bad[0]) if bad.size else int(vmax.shape[0])


def matched_time_err(gh, oh, n):
    """Relative slip error at matched simulated times (the reference records on
    step counts, and the two runs' adaptive steps may differ in the last bits,
    or by a branch of the step control): the GPU history's slip interpolated
    linearly in time at each of the first n oracle record times, against the
    oracle's, over max |D_oracle| of those records."""
    Tg, Dg = gh["T"], gh["D"]
    err = 0.0
    for j in range(n):
        t = oh["T"][j]
        k = int(np.searchsorted(Tg, t))
        if k == 0:
            d = Dg[0] if t == Tg[0] else Dg[0] * (t / Tg[0])   # before the first record: from D = 0 at T = 0
        elif k >= len(Tg):
            return float("inf")                              # past the GPU's window
        else:
            w = (t - Tg[k - 1]) / (Tg[k] - Tg[k - 1])
            d = Dg[k - 1] + w * (Dg[k] - Dg[k - 1])
        err = max(err, float(np.max(np.abs(d - oh["D"][j]))))
    return err / max(float(np.max(np.abs(oh["D"][:n]))), 1e-300)


def _oracle(oracle_mod, prob, ext, op, nsteps, rstep, r=None):
    p = dict(prob, ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
    if r is not None:
        N = prob["N"]
        for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
            p[k] = np.asarray(prob[k])[r * N:(r + 1) * N]
        for k in ("sigma0", "V_const", "mass"):
            p[k] = np.asarray(prob[k])[:N]
    o = oracle_mod.Simulation(p, op)
    return o.run(nsteps, record_step=rstep, max_rec=nsteps // rstep)


def test_c1_single_fault_fp32_within_1e6_of_the_oracle(qdfn_mod, oracle_mod):
    from qdfn import assemble, simulate, synth
    sysd = synth.single_fault()
    rec = sysd["records"]
    Ks, Kn = assemble.assemble_rect(rec, rec, sysd["G"], sysd["nu"])
    prob = synth.problem_dict(sysd, np.diag(Ks))
    ext = synth.external_ramp(sysd["N"], sysd["stressing_rate"], 1e12)
    steps, rstep = 300, 1
    oh = _oracle(oracle_mod, prob, ext, ("dense", Ks, Kn), steps, rstep)
    n = pre_nucleation_records(oh, sysd["N"], np.max(prob["V_i"]))
    assert n * rstep >= 40, n * rstep
    sim = simulate.Simulation(prob, record_step=rstep, max_records=steps // rstep)
    sim.set_dense(Ks, Kn, "fp32")
    sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    sim.run(steps, timeout_s=120)
    d = matched_time_err(sim.history(0), oh, n)
    assert d <= 1e-6, (d, n)
    sim.close()


def _network(seed=2, n_faults=6, patch=100.0):
    from qdfn import assemble, synth
    sysd = synth.fault_network(seed=seed, n_faults=n_faults, patch=patch)
    rec = sysd["records"]
    Ks, Kn = assemble.assemble_rect(rec, rec, sysd["G"], sysd["nu"])
    draws = synth.friction_draws(sysd, 4, seed=1)
    prob = synth.problem_dict(sysd, np.diag(Ks), n_inst=4, draws=draws)
    ext = synth.external_ramp(sysd["N"], sysd["stressing_rate"], 1e12)
    return sysd, rec, Ks, Kn, prob, ext


@pytest.mark.parametrize("precision,bound", [("fp32", 1e-6), ("bf16x2", 1e-4)])
def test_reduced_network_four_draws_within_bound_of_the_oracle(qdfn_mod, oracle_mod, precision, bound):
    """A reduced C2 network (6 faults of the C2 distributions, 100 m patches)
    with 4 friction draws in one context, 400 steps: every draw against its own
    FP64 oracle run over its interseismic horizon.  FP32: 1e-6 (the contract).
    BF16 hi+lo: 1e-4 (its ~16 significant bits; not the contract's format)."""
    from qdfn import simulate
    sysd, rec, Ks, Kn, prob, ext = _network()
    N = sysd["N"]
    steps, rstep = 400, 1
    sim = simulate.Simulation(prob, n_inst=4, record_step=rstep, max_records=steps // rstep)
    sim.set_dense(Ks, Kn, precision)
    sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    sim.run(steps, timeout_s=120)
    worst, horizons = 0.0, []
    for r in range(4):
        oh = _oracle(oracle_mod, prob, ext, ("dense", Ks, Kn), steps, rstep, r=r)
        n = pre_nucleation_records(oh, N - sysd["Nload"], np.max(prob["V_i"]))
        horizons.append(n * rstep)
        if n:
            worst = max(worst, matched_time_err(sim.history(r), oh, n))
    assert sorted(horizons)[1] >= 40, horizons        # at least three draws compared over >= 40 steps
    assert worst <= bound, (worst, horizons)
    sim.close()


def test_hmatrix_fp32_within_1e6_of_the_oracle_h_product(qdfn_mod, oracle_mod):
    """The same kind of network through the H-matrix path (ACA blocks at
    1e-8): FP32 block storage on the GPU against the oracle's FP64 product of
    the same blocks, 300 steps, interseismic horizon."""
    from qdfn import hmatrix, simulate, synth
    from _systems import problem_for, small_network
    sysd = small_network(seed=5, n_faults=6, patch=250.0)
    rec = sysd["records"]
    H, perm = hmatrix.build_rect(rec, G, NU, leaf=32, eta=2.0, tol=1e-8)
    recp = rec[perm]
    Hs, _ = H.to_dense(rec.shape[0])
    prob = problem_for(recp, Hs, seed=3)
    prob["interp_at_told"] = 1
    ext = synth.external_ramp(rec.shape[0], 1e6, 1e11)
    steps, rstep = 300, 1
    blocks = dict(range=H.ranges, sD=H.dense_s, sU=H.U_s, sVt=H.Vt_s, nD=H.dense_n, nU=H.U_n, nVt=H.Vt_n)
    oh = _oracle(oracle_mod, prob, ext, ("hmat", blocks), steps, rstep)
    n = pre_nucleation_records(oh, rec.shape[0], np.max(prob["V_i"]))
    assert n * rstep >= 30, n * rstep
    sim = simulate.Simulation(prob, record_step=rstep, max_records=steps // rstep)
    hmatrix.set_hmatrix(sim, H, "fp32")
    sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    sim.run(steps, timeout_s=120)
    d = matched_time_err(sim.history(0), oh, n)
    assert d <= 1e-6, (d, n)
    sim.close()
