"""Solver branches and arithmetic helpers that the other trajectory tests do
not reach, on the GPU against the FP64 oracle:

* InterpolateFromStressChange (scripts/Functions_Solvers.jl:465-540) with a
  3-sample ExternalStress_TimeArray starting at t > 0: the ramp from zero
  before the first sample (:497-507), the interior interpolation, and the hold
  after the last sample (:509-517), for both main (stress at TOld + Dt) and
  main_H (stress at TOld);
* the slip (Ruina) evolution law, EvolutionDR != 1 (:12);
* the reciprocal-based division of the friction solves against IEEE division
  on random operands and on hard cases (significands near 2, the edges of the
  fast range 2^-895 and 2^896, subnormal results, signed zeros)."""
import numpy as np
import pytest

from _systems import problem_for, small_network

pytestmark = pytest.mark.gpu
G, NU = 32e9, 0.25


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _run_pair(oracle_mod, prob, ext, Ks, Kn, nsteps, rstep=10):
    from qdfn import simulate
    sim = simulate.Simulation(prob, record_step=rstep, max_records=nsteps // rstep)
    sim.set_dense(Ks, Kn, "fp64")
    if ext is not None:
        sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    sim.run(nsteps, timeout_s=120)
    op = dict(prob)
    if ext is not None:
        op.update(ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
    o = oracle_mod.Simulation(op, ("dense", Ks, Kn))
    oh = o.run(nsteps, record_step=rstep, max_rec=nsteps // rstep)
    return sim, o, oh


@pytest.mark.parametrize("interp_at_told", [0, 1])
def test_external_stress_ramp_interior_and_hold(qdfn_mod, oracle_mod, interp_at_told):
    from qdfn import assemble
    rec = small_network(seed=2)["records"]
    N = rec.shape[0]
    Ks, Kn = assemble.assemble_rect(rec, rec, G, NU)
    prob = problem_for(rec, Ks, seed=4)
    prob["interp_at_told"] = interp_at_told
    rng = np.random.default_rng(7)
    # sample times from a run without forcing: steps ~80, ~200 and ~320 of
    # 400, so the forced run starts before the first and ends after the last
    dry = oracle_mod.Simulation(dict(prob), ("dense", Ks, Kn)).run(400, record_step=40, max_rec=10)["T"]
    t = np.array([dry[1], dry[4], dry[7]])
    # small changes (kPa), so that the forced run's time stepping stays close to the dry run's
    shear = np.vstack([rng.uniform(0.5e3, 1.5e3, N), rng.uniform(1.5e3, 2.5e3, N), rng.uniform(2.5e3, 3.0e3, N)])
    normal = np.vstack([rng.uniform(-2e2, 2e2, N) for _ in range(3)])
    pressure = np.vstack([rng.uniform(0, 1e2, N) for _ in range(3)])
    ext = dict(t=t, normal=normal.ravel(), shear=shear.ravel(), pressure=pressure.ravel())
    nsteps = 400
    sim, o, oh = _run_pair(oracle_mod, prob, ext, Ks, Kn, nsteps)
    h = sim.history(0)
    # the window covers all three regimes of the interpolation
    assert oh["T"][0] < t[0] and np.any((oh["T"] > t[0]) & (oh["T"] < t[-1])) and oh["T"][-1] > t[-1], oh["T"]
    assert sim.state(0)["step"] == o.step == nsteps
    assert _rel(h["T"], oh["T"]) < 1e-9
    assert _rel(h["D"], oh["D"]) < 1e-9
    assert _rel(h["sigma"], oh["sigma"]) < 1e-12
    sim.close()


def test_slip_law_trajectory(qdfn_mod, oracle_mod):
    from qdfn import assemble, synth
    rec = small_network(seed=6)["records"]
    Ks, Kn = assemble.assemble_rect(rec, rec, G, NU)
    prob = problem_for(rec, Ks, seed=8)
    prob["evolution_dr"] = 2
    ext = synth.external_ramp(rec.shape[0], 1e6, 1e11)
    nsteps = 300
    sim, o, oh = _run_pair(oracle_mod, prob, ext, Ks, Kn, nsteps)
    h = sim.history(0)
    st = sim.state(0)
    assert st["step"] == o.step == nsteps
    # to rounding over the first 100 steps; over all 300 (through the
    # nucleation of the first slip-law events, which amplifies rounding
    # differences) within 1e-4
    assert _rel(h["T"][:10], oh["T"][:10]) < 1e-9
    assert _rel(h["D"][:10], oh["D"][:10]) < 1e-9 and _rel(h["theta"][:10], oh["theta"][:10]) < 1e-9
    assert abs(st["T"] / o.T - 1) < 1e-4
    assert _rel(h["D"], oh["D"]) < 1e-4
    # the law is in effect: theta differs from the aging-law run of the same problem
    sim2, _, _ = _run_pair(oracle_mod, dict(prob, evolution_dr=1), ext, Ks, Kn, nsteps)
    assert _rel(sim2.history(0)["theta"], h["theta"]) > 1e-6
    sim.close()
    sim2.close()


def _hard_division_operands(rng, n):
    """Dividends and divisors that stress a reciprocal-based quotient."""
    def near_two(k):   # significands 2 - tiny (1.999...)
        return np.ldexp(2.0 - np.ldexp(rng.integers(1, 1 << 20, k).astype(np.float64), -52), 0)
    xs, ds = [], []
    k = n // 8
    e = rng.integers(-60, 60, k)
    xs.append(near_two(k) * np.exp2(e)); ds.append(near_two(k) * np.exp2(rng.integers(-60, 60, k)))
    xs.append(near_two(k)); ds.append(1.0 + np.ldexp(rng.integers(1, 1 << 20, k).astype(np.float64), -52))
    xs.append(rng.uniform(1, 2, k)); ds.append(near_two(k))
    # operands at the edges of the fast path's range and just outside it
    for lo, hi in ((-897, -893), (893, 898)):
        xs.append(rng.uniform(1, 2, k) * np.exp2(rng.integers(lo, hi, k)))
        ds.append(rng.uniform(1, 2, k) * np.exp2(rng.integers(-3, 3, k)))
        xs.append(rng.uniform(1, 2, k) * np.exp2(rng.integers(-3, 3, k)))
        ds.append(rng.uniform(1, 2, k) * np.exp2(rng.integers(lo, hi, k)))
    # quotients that underflow to subnormals or overflow
    xs.append(rng.uniform(1, 2, k) * 2.0 ** -1000); ds.append(rng.uniform(1, 2, k) * 2.0 ** 60)
    x = np.concatenate(xs)
    d = np.concatenate(ds)
    sign = rng.choice([-1.0, 1.0], (2, x.shape[0]))
    x, d = x * sign[0], d * sign[1]
    specials = np.array([0.0, -0.0, 1.0, -1.0, 3.0, np.inf, 5e-324, 1e300])
    xs2, ds2 = np.meshgrid(specials, specials[[0, 1, 2, 3, 4, 5, 6, 7]])
    return np.concatenate([x, xs2.ravel()]), np.concatenate([d, ds2.ravel()])


def test_reciprocal_division_matches_ieee(qdfn_mod):
    import torch
    from qdfn import _lib
    L = _lib.load()
    rng = np.random.default_rng(2024)
    xh, dh = _hard_division_operands(rng, 1 << 20)
    # plus random operands over the exponents the solves meet
    m = 1 << 22
    xr = rng.uniform(1, 2, m) * np.exp2(rng.integers(-80, 80, m)) * rng.choice([-1.0, 1.0], m)
    dr = rng.uniform(1, 2, m) * np.exp2(rng.integers(-80, 80, m)) * rng.choice([-1.0, 1.0], m)
    x = np.concatenate([xh, xr])
    d = np.concatenate([dh, dr])
    with np.errstate(all="ignore"):
        ref = x / d                                       # IEEE division, round to nearest
    xt = torch.tensor(x, device="cuda")
    dt = torch.tensor(d, device="cuda")
    qt = torch.empty_like(xt)
    _lib.check(L.qdfn_check_division(x.shape[0], xt.data_ptr(), dt.data_ptr(), qt.data_ptr(), None))
    torch.cuda.synchronize()
    q = qt.cpu().numpy()
    same = (q.view(np.int64) == ref.view(np.int64)) | (np.isnan(q) & np.isnan(ref))
    bad = np.nonzero(~same)[0]
    assert bad.size == 0, [(float(x[i]), float(d[i]), float(q[i]), float(ref[i])) for i in bad[:8]]
