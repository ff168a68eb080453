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
    assert out["step"] == fx["step"] == 400
    assert np.array_equal(out["Dt"] > 0, fx["Dt"] > 0)
    for k in ("T", "Dt", "D", "V", "theta"):
        assert _rel(out[k], fx[k]) < 1e-12, k


@pytest.mark.gpu
def test_gpu_fp64_follows_the_c1_fixture(qdfn_mod, oracle_mod):
    """GPU-assembled operator (FP64 Okada) and the FP64 step loop against the
    oracle's 400 steps: same step sequence, time and state within 1e-9."""
    from qdfn import assemble, simulate, synth
    fx = _fixture()
    sysd = synth.single_fault()
    rec = sysd["records"]
    Ks, Kn = assemble.assemble_rect(rec, rec, sysd["G"], sysd["nu"])
    prob = synth.problem_dict(sysd, np.diag(Ks))
    ext = synth.external_ramp(sysd["N"], sysd["stressing_rate"], 1e12)
    sim = simulate.Simulation(prob, record_step=10, max_records=40)
    sim.set_dense(Ks, Kn, "fp64")
    sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    sim.run(400, timeout_s=120)
    st, h = sim.state(0), sim.history(0)
    assert st["step"] == fx["step"]
    assert _rel(h["T"], fx["T"]) < 1e-9 and _rel(h["Dt"], fx["Dt"]) < 1e-9
    for k in ("D", "V", "theta"):
        assert _rel(st[k], fx[k]) < 1e-9, k
