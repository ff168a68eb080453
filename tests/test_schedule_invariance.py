"""The overlapped operator/solve phase gives the same bits whatever its schedule.

The FP32 path's step is scheduled dynamically: the operator tiles go to
whichever SM asks next, a step streams the next step's first column chunks
during its own solve tail (QDFN_SPEC_COLS early column chunks, discarded when
the step retries), row blocks holding high-velocity patches go first
(QDFN_RB_ORDER=1) or all go in index order, and each patch is solved on a lane
pair (QDFN_PAIR_SOLVE=1, 16-row chunks) or on one lane (2: every lane, 32-row
chunks; 0: the even lanes alone).  None of this may change a result: every row's products are
summed over the same column chunks in the same order, and the lane-pair solver
performs the one-lane solver's arithmetic.  So runs that differ only in these
settings must agree bit for bit -- through a loaded network that reaches the
high-velocity solver and retried steps.  The per-context early-column setting
(qdfn_set_early_cols) is a schedule setting like the others.
"""
import os

import numpy as np
import pytest

from _systems import problem_for

pytestmark = pytest.mark.gpu
G, NU = 32e9, 0.25
FIELDS = ("V", "D", "theta", "friction", "accel", "sigma_old")


@pytest.fixture(scope="module")
def loaded_network(qdfn_mod):
    """1568 patches (12 faults of 200 m patches), loaded at 2e7 Pa/yr so that
    ruptures and retried steps come early.  With the grid capped at 16 blocks
    the FP32 tiling has 2 full-width row blocks of 16 column chunks: early
    tiles wait on solved row blocks of the same step."""
    from qdfn import assemble, synth
    rec = synth.fault_network(seed=3, n_faults=12, patch=200.0, length=(2000.0, 4000.0))["records"]
    Ks, Kn = assemble.assemble_rect(rec, rec, G, NU)
    prob = problem_for(rec, Ks, seed=4)
    ext = synth.external_ramp(rec.shape[0], 2e7, 1e11)
    return prob, Ks, Kn, ext


def _run(net, env, nsteps, chunk, precision, early=None):
    """States after every `chunk` steps, with `env` set while the context is
    configured (the schedule settings are read then); `early`: the context's
    early-column setting."""
    from qdfn import simulate
    prob, Ks, Kn, ext = net
    old = {k: os.environ.get(k) for k in env}
    try:
        os.environ.update({k: str(v) for k, v in env.items()})
        sim = simulate.Simulation(prob, n_inst=2)
        sim.set_dense(Ks, Kn, precision)
        sim.set_blocks(16)
        if early is not None:
            sim.set_early_cols(early)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    states = []
    for _ in range(nsteps // chunk):
        sim.run(chunk, timeout_s=120)
        states.append([sim.state(r) for r in range(2)])
    return states, sim.counters()


def _same(a, b):
    for sa, sb in zip(a, b):
        for r in range(2):
            assert sa[r]["step"] == sb[r]["step"]
            assert sa[r]["T"] == sb[r]["T"] and sa[r]["dt"] == sb[r]["dt"]
            for k in FIELDS:
                assert np.array_equal(sa[r][k], sb[r][k], equal_nan=True), k


@pytest.mark.parametrize("precision", ["fp32", "bf16x2"])
def test_early_tiles_and_lane_pairs_change_no_bit(qdfn_mod, loaded_network, precision):
    nsteps, chunk = 400, 100
    ref, cnt = _run(loaded_network, {"QDFN_SPEC_COLS": 0, "QDFN_PAIR_SOLVE": 0, "QDFN_RB_ORDER": 0},
                    nsteps, chunk, precision)
    # the horizon reaches retried steps (each discards the next step's early
    # tiles) and the high-velocity solver
    assert cnt["solve_passes"] > cnt["steps"] and cnt["highv_solves"] > 0, cnt
    for env in ({"QDFN_SPEC_COLS": 8, "QDFN_PAIR_SOLVE": 1, "QDFN_RB_ORDER": 1},     # the defaults
                {"QDFN_SPEC_COLS": 16, "QDFN_PAIR_SOLVE": 1, "QDFN_RB_ORDER": 1},    # every column chunk early
                {"QDFN_SPEC_COLS": 0, "QDFN_PAIR_SOLVE": 1, "QDFN_RB_ORDER": 0},
                {"QDFN_SPEC_COLS": 8, "QDFN_PAIR_SOLVE": 0, "QDFN_RB_ORDER": 1},
                {"QDFN_SPEC_COLS": 8, "QDFN_PAIR_SOLVE": 2, "QDFN_RB_ORDER": 1},     # one lane per patch, 32 rows
                {"QDFN_SPEC_COLS": 0, "QDFN_PAIR_SOLVE": 2, "QDFN_RB_ORDER": 0}):
        got, _ = _run(loaded_network, env, nsteps, chunk, precision)
        _same(ref, got)


def test_early_columns_per_context_change_no_bit(qdfn_mod, loaded_network):
    nsteps, chunk = 200, 100
    ref, _ = _run(loaded_network, {}, nsteps, chunk, "fp32")
    for cols in (0, 1, 64):
        got, _ = _run(loaded_network, {}, nsteps, chunk, "fp32", early=cols)
        _same(ref, got)

