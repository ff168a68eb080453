"""Cycle simulation on the GPU (persistent kernel) vs the FP64 oracle.

FP64 path: same step decisions and slip/slip-rate/time within 1e-9 relative over
the stated horizons (the matvec sums in a different order than the oracle, so
agreement is to rounding, amplified by the dynamics; horizons stop before the
differences reach the branch decisions).
"""
import numpy as np
import pytest

from _systems import cols, mixed_rects, problem_for, small_network

pytestmark = pytest.mark.gpu
G, NU = 32e9, 0.25


def _setup(oracle_mod, rec, seed=None, rate=1e6, **kw):
    from qdfn import assemble, synth
    Ks, Kn = assemble.assemble_rect(rec, rec, G, NU)
    prob = problem_for(rec, Ks, seed=seed, **kw)
    ext = synth.external_ramp(rec.shape[0], rate, 1e11)
    oprob = dict(prob, ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
    return Ks, Kn, prob, ext, oprob


def _gpu_sim(prob, Ks, Kn, ext, precision="fp64", n_inst=1, record_step=0, max_records=0):
    from qdfn import simulate
    sim = simulate.Simulation(prob, n_inst=n_inst, record_step=record_step, max_records=max_records)
    sim.set_dense(Ks, Kn, precision)
    sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    return sim


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_operator_fp64_matches_oracle(qdfn_mod, oracle_mod):
    rec = mixed_rects()
    Ks, Kn, prob, ext, _ = _setup(oracle_mod, rec)
    sim = _gpu_sim(prob, Ks, Kn, ext)
    D = np.random.default_rng(0).uniform(-1, 2, rec.shape[0])
    tld, knd = sim.apply(D)
    o = oracle_mod.Simulation(dict(prob), ("dense", Ks, Kn))
    otld, oknd = o.apply(D)
    assert _rel(tld[0], otld) < 1e-12 and _rel(knd[0], oknd) < 1e-12
    assert np.array_equal(sim.kself(), o.kself())


@pytest.mark.parametrize("precision,tol", [("fp32", 2e-6), ("bf16x2", 2e-4)])
def test_operator_mixed_precision_error(qdfn_mod, oracle_mod, precision, tol):
    rec = small_network()["records"]
    Ks, Kn, prob, ext, _ = _setup(oracle_mod, rec)
    sim = _gpu_sim(prob, Ks, Kn, ext, precision=precision)
    D = np.random.default_rng(1).uniform(0.0, 1.0, rec.shape[0])
    tld, knd = sim.apply(D)
    o = oracle_mod.Simulation(dict(prob), ("dense", Ks, Kn))
    otld, oknd = o.apply(D)
    assert _rel(tld[0], otld) < tol and _rel(knd[0], oknd) < tol


def test_fp64_trajectory_matches_oracle(qdfn_mod, oracle_mod):
    rec = mixed_rects()
    Ks, Kn, prob, ext, oprob = _setup(oracle_mod, rec)
    nsteps = 300
    sim = _gpu_sim(prob, Ks, Kn, ext, record_step=10, max_records=nsteps // 10)
    sim.run(nsteps, timeout_s=120)
    o = oracle_mod.Simulation(oprob, ("dense", Ks, Kn))
    oh = o.run(nsteps, record_step=10, max_rec=nsteps // 10)
    st = sim.state(0)
    h = sim.history(0)
    assert st["step"] == o.step == nsteps
    assert abs(st["T"] / o.T - 1) < 1e-9
    assert np.array_equal(h["Dt"] > 0, oh["Dt"] > 0) and h["T"].shape == oh["T"].shape
    assert _rel(h["T"], oh["T"]) < 1e-9
    assert _rel(st["D"], o.state["D"]) < 1e-9
    assert _rel(st["V"], o.state["V"]) < 1e-9
    assert _rel(h["sigma"], oh["sigma"]) < 1e-12


def test_fp64_trajectory_through_rupture(qdfn_mod, oracle_mod):
    """Fast loading (1 MPa/yr on 1 MPa normal-stress scale faults) drives the
    velocity-weakening patches through SwitchV: the high-V solver, the rupture
    time step and the retries are exercised."""
    rec = mixed_rects()
    Ks, Kn, prob, ext, oprob = _setup(oracle_mod, rec, rate=2e7)
    o = oracle_mod.Simulation(oprob, ("dense", Ks, Kn))
    sim = _gpu_sim(prob, Ks, Kn, ext)
    vmax_o = 0.0
    for _ in range(40):
        o.run(25)
        sim.run(25, timeout_s=120)
        vmax_o = max(vmax_o, float(np.max(o.state["V"])))
        st = sim.state(0)
        assert st["step"] == o.step
        assert abs(st["T"] / o.T - 1) < 1e-6
        assert _rel(st["D"], o.state["D"]) < 1e-6
        if vmax_o > prob["switch_v"]:
            break
    assert vmax_o > prob["switch_v"], "horizon did not reach a rupture"


@pytest.mark.parametrize("n_inst", [2, 3])
def test_instances_match_independent_oracle_runs(qdfn_mod, oracle_mod, n_inst):
    from qdfn import synth
    rec = small_network()["records"]
    Ks, Kn, prob, ext, oprob = _setup(oracle_mod, rec)
    draws = synth.friction_draws(dict(prob, N=rec.shape[0]), n_inst, seed=5)
    mprob = dict(prob)
    for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
        mprob[k] = draws[k]
    sim = _gpu_sim(mprob, Ks, Kn, ext, n_inst=n_inst)
    sim.run(150, timeout_s=120)
    N = rec.shape[0]
    for r in range(n_inst):
        op = dict(oprob)
        for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
            op[k] = draws[k][r * N:(r + 1) * N]
        o = oracle_mod.Simulation(op, ("dense", Ks, Kn))
        o.run(150)
        st = sim.state(r)
        assert abs(st["T"] / o.T - 1) < 1e-9
        assert _rel(st["D"], o.state["D"]) < 1e-9


@pytest.mark.parametrize("precision", ["fp64", "fp32", "bf16x2"])
@pytest.mark.parametrize("n_inst", [1, 3])
def test_odd_sized_system_tracks_the_oracle(qdfn_mod, oracle_mod, precision, n_inst):
    """N = 49 (odd) with 1 and 3 instances: the step loop's second state
    buffer and the operator's second copy of D start at an odd element offset
    unless padded, which bulk copies cannot read.  FP32 runs the overlapped
    operator/solve phase (lane-pair solves), as does BF16x2; FP64 the sequential
    one.  All follow the FP64 oracle: FP64 to rounding, FP32 and BF16x2 within
    their operator error."""
    from qdfn import synth
    rec = small_network(seed=1)["records"]
    assert rec.shape[0] % 2 == 1
    Ks, Kn, prob, ext, oprob = _setup(oracle_mod, rec)
    N = rec.shape[0]
    draws = synth.friction_draws(dict(prob, N=N), n_inst, seed=9)
    mprob = dict(prob)
    for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
        mprob[k] = draws[k]
    sim = _gpu_sim(mprob, Ks, Kn, ext, precision=precision, n_inst=n_inst)
    nsteps, tol = {"fp64": (101, 1e-9), "fp32": (41, 1e-4), "bf16x2": (41, 2e-3)}[precision]
    sim.run(nsteps, timeout_s=120)
    for r in range(n_inst):
        op = dict(oprob)
        for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
            op[k] = draws[k][r * N:(r + 1) * N]
        o = oracle_mod.Simulation(op, ("dense", Ks, Kn))
        o.run(nsteps)
        st = sim.state(r)
        assert st["step"] == o.step == nsteps
        assert abs(st["T"] / o.T - 1) < tol
        assert _rel(st["D"], o.state["D"]) < tol
        assert _rel(st["V"], o.state["V"]) < tol


def test_ensemble_state_transfer_matches_per_instance_api(qdfn_mod, oracle_mod):
    """qdfn_get_state_all / qdfn_set_state_all move the same bytes as the
    per-instance calls, and set_state_all -> run_async -> get_state_all (one
    synchronisation) continues a run exactly like set_state -> run -> state."""
    from qdfn import synth
    rec = small_network()["records"]
    Ks, Kn, prob, ext, _ = _setup(oracle_mod, rec)
    N, R = rec.shape[0], 3
    draws = synth.friction_draws(dict(prob, N=N), R, seed=4)
    mprob = dict(prob)
    for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
        mprob[k] = draws[k]
    a = _gpu_sim(mprob, Ks, Kn, ext, n_inst=R)
    a.run(30)
    names = a.STATE_FIELDS
    arr = {k: np.full(R * N, np.nan) for k in names}
    T, dt, step = np.zeros(R), np.zeros(R), np.zeros(R, dtype=np.int64)
    a.get_state_all(arr, T, dt, step)
    for r in range(R):
        st = a.state(r)
        for k in names:
            assert np.array_equal(arr[k][r * N:(r + 1) * N], st[k])
        assert T[r] == st["T"] and dt[r] == st["dt"] and step[r] == st["step"]
    b = _gpu_sim(mprob, Ks, Kn, ext, n_inst=R)
    b.set_state_all(arr, T, dt, step)
    b.run_async(12)
    out = {k: np.zeros(R * N) for k in names}
    T2, dt2, step2 = np.zeros(R), np.zeros(R), np.zeros(R, dtype=np.int64)
    b.get_state_all(out, T2, dt2, step2, wait=True)
    a.run(12)
    for r in range(R):
        st = a.state(r)
        for k in names:
            assert np.array_equal(out[k][r * N:(r + 1) * N], st[k])
        assert T2[r] == st["T"] and step2[r] == st["step"] == 42


def test_state_roundtrip_resumes_identically(qdfn_mod, oracle_mod):
    rec = mixed_rects()
    Ks, Kn, prob, ext, _ = _setup(oracle_mod, rec)
    a = _gpu_sim(prob, Ks, Kn, ext)
    a.run(80)
    st = a.state(0)
    a.run(40)
    b = _gpu_sim(prob, Ks, Kn, ext)
    b.set_state(0, st)
    b.run(40)
    sa, sb = a.state(0), b.state(0)
    assert sa["T"] == sb["T"] and np.array_equal(sa["D"], sb["D"])


def test_timeout_returns_an_error_and_context_stays_usable(qdfn_mod, oracle_mod):
    from qdfn import QdfnError
    rec = mixed_rects()
    Ks, Kn, prob, ext, _ = _setup(oracle_mod, rec)
    sim = _gpu_sim(prob, Ks, Kn, ext)
    with pytest.raises(QdfnError) as ei:
        sim.run(10 ** 9, timeout_s=0.05)
    assert ei.value.code == -14
    sim2 = _gpu_sim(prob, Ks, Kn, ext)
    sim2.run(5)
    assert sim2.state(0)["step"] == 5


def test_empty_control_set_is_reported_like_the_reference(qdfn_mod, oracle_mod):
    """All patches at V = 0 with zero acceleration: |V/Accel| is NaN everywhere
    and Julia's `minimum` over the empty filtered set throws; both sides stop."""
    from qdfn import QdfnError
    rec = mixed_rects()
    Ks, Kn, prob, ext, oprob = _setup(oracle_mod, rec)
    prob = dict(prob, V_i=np.zeros(rec.shape[0]))
    oprob = dict(oprob, V_i=np.zeros(rec.shape[0]))
    sim = _gpu_sim(prob, Ks, Kn, ext)
    with pytest.raises(QdfnError) as ei:
        sim.run(3)
    assert ei.value.code == -11
    o = oracle_mod.Simulation(oprob, ("dense", Ks, Kn))
    with pytest.raises(RuntimeError, match="empty"):
        o.run(3)
