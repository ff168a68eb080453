"""The committed C1 single-fault fixture (tests/golden/make_golden.py): the
oracle still reproduces it, and the GPU FP64 path follows it."""
import importlib.util
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _maker():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _fixture():
    return dict(np.load(os.path.join(GOLD, "c1_single_fault_oracle.npz")))


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_oracle_reproduces_the_c1_fixture(oracle_mod):
    fx = _fixture()
    out = _maker().run_oracle(oracle_mod)
    assert out["step"] == fx["step"] == 400 and out["frag_count"] == fx["frag_count"] > 0
    assert np.array_equal(out["Dt"] > 0, fx["Dt"] > 0)
    for k in ("T", "Dt", "D", "V", "theta", "T_state", "frag_t", "frag_moment"):
        assert _rel(out[k], fx[k]) < 1e-12, k


@pytest.mark.gpu
def test_gpu_fp64_follows_the_c1_fixture(qdfn_mod, oracle_mod):
    """GPU-assembled operator (FP64 Okada) and the FP64 step loop against the
    oracle: to 1e-9 until step 120 (before the first event nucleates), the time
    history to 1e-4 and the event onsets to 1e-9 over 400 steps."""
    from qdfn import assemble, events, simulate, synth
    fx = _fixture()
    sysd = synth.single_fault()
    rec = sysd["records"]
    Ks, Kn = assemble.assemble_rect(rec, rec, sysd["G"], sysd["nu"])
    prob = synth.problem_dict(sysd, np.diag(Ks))
    ext = synth.external_ramp(sysd["N"], sysd["stressing_rate"], 1e12)
    sim = simulate.Simulation(prob, record_step=2, max_records=200)
    sim.set_dense(Ks, Kn, "fp64")
    sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    sim.run(120, timeout_s=120)
    st = sim.state(0)
    assert abs(st["T"] / fx["T_state"] - 1) < 1e-9
    for k in ("D", "V", "theta"):
        assert _rel(st[k], fx[k]) < 1e-9, k
    sim.run(280, timeout_s=120)
    h = sim.history(0)
    assert sim.state(0)["step"] == fx["step"] and h["T"].shape == fx["T"].shape
    assert _rel(h["T"][:60], fx["T"][:60]) < 1e-9 and _rel(h["Dt"][:60], fx["Dt"][:60]) < 1e-9
    assert _rel(h["T"], fx["T"]) < 1e-4
    ft, _, fm, fn = events.event_fragments(h["T"], h["D"], rec[:, :3], events.patch_area_rect(rec[:, 3], rec[:, 4]),
                                           sysd["G"])
    assert fn == fx["frag_count"]
    assert _rel(ft, fx["frag_t"]) < 1e-9 and _rel(fm, fx["frag_moment"]) < 1e-3
