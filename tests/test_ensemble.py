"""Batched ensembles of fault networks of uneven size in ONE persistent launch
(qdfn_ensemble_*): every member runs on its own share of the SMs with its own
adaptive steps; each instance is checked against its own oracle run."""
import numpy as np
import pytest

from _systems import problem_for

G, NU = 32e9, 0.25


def test_sm_shares_are_proportional_and_fit():
    from qdfn import _lib
    from qdfn.ensemble import sm_shares
    s = sm_shares([1.0, 1.0, 2.0, 4.0], 152)
    assert s.sum() == 152 and list(s) == [19, 19, 38, 76]
    s = sm_shares([1e6] + [1.0] * 20, 152)          # tiny members still get one SM each
    assert s.sum() == 152 and s.min() == 1 and s[0] == 152 - 20
    s = sm_shares([3.0, 1.0, 1.0], 4)                # longest time 1.5 (3/2), the others 1
    assert list(s) == [2, 1, 1]
    s = sm_shares([5.0, 2.0, 2.0, 1.0], 7)           # the smallest longest time on 7 blocks is 2.0
    assert s.sum() == 7 and max(c / b for c, b in zip([5.0, 2.0, 2.0, 1.0], s)) == 2.0
    with pytest.raises(_lib.QdfnError):
        sm_shares(np.ones(200), 152)                 # more members than SMs
    with pytest.raises(_lib.QdfnError):
        sm_shares([1.0, 0.0], 152)                   # costs must be positive


def test_state_record_layout_round_trips():
    """The ensemble state record (qdfn_ensemble_set/get_state_all's host
    buffer): member after member [6][n_inst][N] doubles, then T, dt and step
    [n_inst] as 8-byte words -- packed and unpacked on the host, no GPU."""
    import types
    from qdfn import ensemble, simulate
    rng = np.random.default_rng(0)
    sims = [types.SimpleNamespace(n_inst=R, N=N) for R, N in ((4, 7), (1, 3), (2, 5))]
    words = sum(6 * m.n_inst * m.N + 3 * m.n_inst for m in sims)
    ens = types.SimpleNamespace(members=sims, state_words=lambda: words)
    states = [[dict({k: rng.normal(size=m.N) for k in simulate.Simulation.STATE_FIELDS},
                    T=float(rng.uniform()), dt=float(rng.uniform()), step=int(rng.integers(0, 1 << 40)))
               for _ in range(m.n_inst)] for m in sims]
    buf = ensemble.Ensemble.pack_states(ens, states)
    assert buf.shape == (words,)
    # member 1 starts after member 0's 6*4*7 + 3*4 words; its V is first, its step last
    o1 = 6 * 4 * 7 + 12
    assert np.array_equal(buf[o1:o1 + 3], states[1][0]["V"])
    assert buf[o1 + 18 + 2:o1 + 18 + 3].view(np.int64)[0] == states[1][0]["step"]
    back = ensemble.Ensemble.unpack_states(ens, buf)
    for a, b in zip(back, states):
        for x, y in zip(a, b):
            assert x["T"] == y["T"] and x["dt"] == y["dt"] and x["step"] == y["step"]
            for k in simulate.Simulation.STATE_FIELDS:
                assert np.array_equal(x[k], y[k])


def _member(seed, R, n_faults=4, patch=400.0, length=(1200.0, 2400.0)):
    """One geometry with R friction draws: the member dict and what its oracle
    runs need."""
    from qdfn import assemble, synth
    rec = synth.fault_network(seed=seed, n_faults=n_faults, patch=patch, length=length)["records"]
    N = rec.shape[0]
    Ks, Kn = assemble.assemble_rect(rec, rec, G, NU)
    prob = problem_for(rec, Ks)
    ext = synth.external_ramp(N, 1e6, 1e11)
    draws = synth.friction_draws(dict(prob, N=N), R, seed=seed)
    mprob = dict(prob)
    for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
        mprob[k] = draws[k]
    for k in ("sigma0", "V_const", "mass"):
        mprob[k] = np.tile(prob[k], R)
    return dict(problem=mprob, n_inst=R, Ks=Ks, Kn=Kn, ext=ext), (prob, ext, draws, Ks, Kn, N, R)


def _oracle_run(oracle_mod, ref, r, nsteps):
    prob, ext, draws, Ks, Kn, N, R = ref
    op = dict(prob, ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
    for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
        op[k] = draws[k][r * N:(r + 1) * N]
    o = oracle_mod.Simulation(op, ("dense", Ks, Kn))
    o.run(nsteps)
    return o


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.gpu
def test_ensemble_members_follow_their_oracles(qdfn_mod, oracle_mod):
    """Three geometries (3, 4 and 4 friction draws), FP64 operator, one launch:
    every instance matches its own oracle run to 1e-9."""
    from qdfn import ensemble
    built = [_member(seed, R) for seed, R in ((1, 3), (2, 4), (4, 4))]
    ens = ensemble.Ensemble([m for m, _ in built], precision="fp64")
    assert sum(ens.blocks) <= 152 and min(ens.blocks) >= 1
    ens.run(80, timeout_s=120)
    for sim, (_, ref) in zip(ens.members, built):
        for r in range(ref[6]):
            o = _oracle_run(oracle_mod, ref, r, 80)
            st = sim.state(r)
            assert st["step"] == o.step == 80
            assert abs(st["T"] / o.T - 1) < 1e-9
            assert _rel(st["D"], o.state["D"]) < 1e-9
    ens.close()


@pytest.mark.gpu
def test_fp32_ensemble_members_within_1e6_of_the_fp64_oracle(qdfn_mod, oracle_mod):
    """Eight geometries x 4 friction draws with the operator stored in FP32
    (mixed precision), 200 steps in one launch, recorded every step: every
    instance against its FP64 oracle run over its interseismic horizon (until a
    patch accelerates past twice the starting slip rate; a nucleation's
    runaway amplifies any perturbation) -- relative slip error at matched
    simulated times within 1e-6."""
    from qdfn import ensemble
    from test_mixed_precision_contract import matched_time_err, pre_nucleation_records
    steps, rstep = 200, 1
    built = [_member(10 + k, 4, n_faults=3 + k % 3) for k in range(8)]
    for m, _ in built:
        m.update(record_step=rstep, max_records=steps // rstep)
    ens = ensemble.Ensemble([m for m, _ in built], precision="fp32")
    ens.run(steps, timeout_s=120)
    worst, horizons = 0.0, []
    for sim, (m, ref) in zip(ens.members, built):
        for r in range(4):
            prob, ext, draws, Ks, Kn, N, R = ref
            op = dict(prob, ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
            for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
                op[k] = draws[k][r * N:(r + 1) * N]
            oh = oracle_mod.Simulation(op, ("dense", Ks, Kn)).run(steps, record_step=rstep, max_rec=steps // rstep)
            gh = sim.history(r)
            assert sim.state(r)["step"] == steps and gh["T"].shape == oh["T"].shape
            n = pre_nucleation_records(oh, N, np.max(op["V_i"]))
            horizons.append(n * rstep)
            if n:
                worst = max(worst, matched_time_err(gh, oh, n))
    assert np.median(horizons) >= 30, horizons
    assert worst <= 1e-6, (worst, horizons)
    ens.close()


@pytest.mark.gpu
def test_sixteen_uneven_members_finish_and_rebalance(qdfn_mod, oracle_mod):
    """Sixteen members of 18 to ~1,000 patches (uneven), FP32 x 4 draws: a run,
    two autotuner rounds (the SMs re-divided by measured member time), and more
    runs all finish without a timeout; every instance takes exactly the steps
    asked for, and instance 0 of each member stays within 1e-6 of its oracle."""
    from qdfn import ensemble
    from test_mixed_precision_contract import matched_time_err, pre_nucleation_records
    specs = [(30 + k, 2 + (k * 5) % 11, 200.0 + 40.0 * (k % 5)) for k in range(16)]
    built = [_member(s, 4, n_faults=nf, patch=pt, length=(1000.0, 3000.0)) for s, nf, pt in specs]
    for m, _ in built:
        m.update(record_step=1, max_records=180)
    sizes = [ref[5] for _, ref in built]
    assert max(sizes) > 10 * min(sizes)
    ens = ensemble.Ensemble([m for m, _ in built], precision="fp32")
    b0 = ens.blocks.copy()
    hist = ens.autotune(120, rounds=2, timeout_s=120)
    assert all(h.sum() <= 152 and h.min() >= 1 for h in hist)
    ens.run(60, timeout_s=120)
    assert b0.sum() <= 152
    for sim, (_, ref) in zip(ens.members, built):
        for r in range(4):
            assert sim.state(r)["step"] == 180
        prob, ext, draws, Ks, Kn, N, R = ref
        op = dict(prob, ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
        for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
            op[k] = draws[k][:N]
        oh = oracle_mod.Simulation(op, ("dense", Ks, Kn)).run(180, record_step=1, max_rec=180)
        n = pre_nucleation_records(oh, N, np.max(op["V_i"]))
        if n:   # instance 0 over its interseismic horizon, across the re-divisions
            assert matched_time_err(sim.history(0), oh, n) <= 1e-6
    ens.close()


@pytest.mark.gpu
def test_ensemble_rejects_mixed_members_and_member_runs_in_flight(qdfn_mod):
    import torch
    from qdfn import _lib, ensemble
    m1, _ = _member(1, 4)
    m2, _ = _member(2, 1)
    with pytest.raises(_lib.QdfnError):   # instance-count classes 4 and 1 differ
        ensemble.Ensemble([m1, m2], precision="fp32")
    ens = ensemble.Ensemble([m1, _member(3, 4)[0]], precision="fp32")
    st = torch.cuda.Stream()
    ens.run_async(20, timeout_s=60, stream=st.cuda_stream)
    with pytest.raises(_lib.QdfnError):   # a member may not run on its own meanwhile
        ens.members[0].run(1)
    ens.sync()
    assert ens.members[0].state(0)["step"] == 20
    ens.members[0].run(1)                 # between ensemble runs it is an ordinary context
    assert ens.members[0].state(0)["step"] == 21
    with pytest.raises(_lib.QdfnError):
        ens.set_blocks([0, 1])
    ens.set_blocks([2, 3])
    assert 1 <= ens.blocks[0] <= 2 and 1 <= ens.blocks[1] <= 3   # (small members use fewer)
    ens.close()


@pytest.mark.gpu
def test_one_copy_state_transfer_matches_the_members(qdfn_mod):
    """qdfn_ensemble_{set,get}_state_all: the whole ensemble's state in one
    host buffer.  Setting a packed record puts every member's state in place
    (what each member's own calls read back, bit for bit); after a run, the
    record read back is every member's state; a run in flight on the stream is
    completed by the read; setting during a run is refused."""
    import torch
    from qdfn import _lib, ensemble
    built = [_member(seed, R, n_faults=3) for seed, R in ((5, 4), (6, 3), (7, 4))]
    ens = ensemble.Ensemble([m for m, _ in built], precision="fp32")
    ens.run(20, timeout_s=60)
    snap = [[sim.state(r) for r in range(sim.n_inst)] for sim in ens.members]
    ens.run(15, timeout_s=60)
    buf = torch.empty(ens.state_words(), dtype=torch.float64).pin_memory()
    assert ens.state_words() == sum(6 * sim.n_inst * sim.N + 3 * sim.n_inst for sim in ens.members)
    ens.pack_states(snap, out=buf)
    ens.set_state_all(buf)
    torch.cuda.synchronize()
    for sim, sts in zip(ens.members, snap):
        for r, st in enumerate(sts):
            got = sim.state(r)
            assert got["step"] == st["step"] == 20 and got["T"] == st["T"] and got["dt"] == st["dt"]
            for k in ensemble.simulate.Simulation.STATE_FIELDS:
                assert np.array_equal(got[k], st[k]), k
    st = torch.cuda.Stream()
    ens.run_async(15, timeout_s=60, stream=st.cuda_stream)
    with pytest.raises(_lib.QdfnError):
        ens.set_state_all(buf, stream=st.cuda_stream)
    ens.get_state_all(buf, stream=st.cuda_stream, wait=True)   # completes the run
    back = ens.unpack_states(buf)
    for sim, sts in zip(ens.members, back):
        for r, rec in enumerate(sts):
            own = sim.state(r)
            assert rec["step"] == own["step"] == 35 and rec["T"] == own["T"] and rec["dt"] == own["dt"]
            for k in ensemble.simulate.Simulation.STATE_FIELDS:
                assert np.array_equal(rec[k], own[k]), k
    # the same 15 steps from the restored state give the same record
    ens.pack_states(snap, out=buf)
    ens.set_state_all(buf)
    ens.run(15, timeout_s=60)
    again = [[sim.state(r) for r in range(sim.n_inst)] for sim in ens.members]
    for a, b in zip(again, back):
        for x, y in zip(a, b):
            assert x["T"] == y["T"] and np.array_equal(x["D"], y["D"])
    ens.close()
