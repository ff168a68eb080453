"""The reference's own input files through the pipeline: its default bulk input
(Input_BulkFaultGeometry.txt, a BP5QD-like strike-slip setup with loading
faults), the Ridgecrest example geometry and the NormalFaults.obj triangle mesh,
carried verbatim in tests/golden/reference_inputs.npz (written by
tests/golden/make_reference_inputs.py from the reference checkout).

CPU: the C-ABI parser and the Python restatement read the files alike
(ReadBulkInput / BulkToSegment / RotVerts_UnitVectors,
scripts/Functions_BuildInputFile.jl:82-377; ObjReader.jl:44-135), with the
patch counts the gridding rule gives.  GPU: FP64 stiffness assembly of all
three against the oracle, and the drop-in `main` on the BP5QD input against the
oracle's run of the same steps (RUN2 -> RUN3 flow: Functions_RSFDFN3DMain_D.jl
driven with the parameters QUAKEDFN_RunARG.jl:150-201 derives, ParameterAdj
left at its shipped identity)."""
import hashlib
import math
import os

import numpy as np
import pytest

from qdfn import geometry as G

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "reference_inputs.npz")


def _fixture():
    return np.load(FIX)


def _bulk_file(tmp_path, key):
    p = tmp_path / (key + ".txt")
    p.write_text(str(_fixture()[key + "_text"]))
    return str(p)


def test_fixture_texts_are_the_reference_files_verbatim():
    z = _fixture()
    for key in ("bp5qd", "ridgecrest"):
        assert hashlib.sha256(str(z[key + "_text"]).encode()).hexdigest() == str(z[key + "_sha256"])
    V, F = z["obj_vertices"], z["obj_faces"]
    assert V.shape == (604, 3) and F.shape == (1100, 3) and F.min() == 0 and F.max() == 603


@pytest.mark.parametrize("key,count,nload", [("bp5qd", 4005, 5), ("ridgecrest", 3404, 0)])
def test_reference_bulk_files_parse_alike(qdfn_mod, tmp_path, key, count, nload):
    path = _bulk_file(tmp_path, key)
    a = G.read_bulk_input(path)
    b = G.read_bulk_input_abi(path)
    assert a["RorT"] == b["RorT"] == "R"
    assert a["FaultCount"] == b["FaultCount"] == count
    assert a["LoadingFaultCount"] == b["LoadingFaultCount"] == nload
    # the gridding rule, counted straight from the bulk rows
    rows = [r.split() for r in str(_fixture()[key + "_text"]).splitlines()[3:] if r.strip()]
    assert sum(math.ceil(float(r[3]) / float(r[17])) * math.ceil(float(r[4]) / float(r[17])) for r in rows) == count
    sa, sb = a["Input_Segment"], b["Input_Segment"]
    assert np.array_equal(sa[:, 3:14], sb[:, 3:14]) and np.array_equal(sa[:, 15:], sb[:, 15:])
    assert np.max(np.abs(sa[:, 0:3] - sb[:, 0:3])) <= 1e-12 * np.max(np.abs(sa[:, 0:3]))
    assert np.allclose(sa[:, 14], sb[:, 14], rtol=1e-12, atol=0)
    assert np.all(sa[-nload:, 15] > 0) if nload else np.all(sa[:, 15] == 0)   # loading faults last
    assert np.all(sa[:count - nload, 15] == 0)


def test_obj_mesh_to_bulk_parses_alike(qdfn_mod, tmp_path):
    z = _fixture()
    header, bulk = G.obj_to_bulk(z["obj_vertices"], z["obj_faces"])
    path = str(tmp_path / "tri.txt")
    G.write_bulk_file(path, header, bulk)
    a = G.read_bulk_input(path)
    b = G.read_bulk_input_abi(path)
    assert a["RorT"] == b["RorT"] == "T" and a["FaultCount"] == b["FaultCount"] == 1100
    assert np.array_equal(a["Input_Segment"], b["Input_Segment"])
    seg = a["Input_Segment"]
    assert np.max(seg[:, [2, 5, 8]]) <= 0.0                 # half-space: every vertex at or below z = 0
    pa = G.rot_verts_unit_vectors(seg, seg[:, 9])
    pb = G.rot_verts_unit_vectors_abi(seg, seg[:, 9])
    for x, y in zip(pa, pb):
        assert np.max(np.abs(x - y)) <= 1e-12 * max(1.0, np.max(np.abs(x)))


def _rect_setup(tmp_path, key):
    d = G.read_bulk_input(_bulk_file(tmp_path, key))
    s = G.read_segment_input(d["Input_Segment"], d["RorT"])
    return d, s, G.rect_records(s)


def _cols(rec):
    return dict(cx=rec[:, 0], cy=rec[:, 1], cz=rec[:, 2], ls=rec[:, 3], ld=rec[:, 4], strike=rec[:, 5],
                dip=rec[:, 6], rake=rec[:, 7])


def _row_rel(A, B, S, N):
    scale = np.maximum(np.max(np.abs(S), axis=1, keepdims=True), np.max(np.abs(N), axis=1, keepdims=True))
    return float(np.max(np.abs(A - B) / scale))


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["bp5qd", "ridgecrest"])
def test_reference_geometries_assemble_like_the_oracle(qdfn_mod, oracle_mod, tmp_path, key):
    from qdfn import assemble
    d, s, rec = _rect_setup(tmp_path, key)
    Ks, Kn = assemble.assemble_rect(rec, rec, d["ShearModulus"], d["PoissonRatio"])
    Ko_s, Ko_n = oracle_mod.assemble_rect(_cols(rec), _cols(rec), d["ShearModulus"], d["PoissonRatio"])
    assert _row_rel(Ks, Ko_s, Ko_s, Ko_n) <= 1e-12
    assert _row_rel(Kn, Ko_n, Ko_s, Ko_n) <= 1e-12
    assert np.all(np.diag(Ks) < 0)


@pytest.mark.gpu
def test_reference_obj_mesh_assembles_like_the_oracle(qdfn_mod, oracle_mod, tmp_path):
    from qdfn import assemble
    z = _fixture()
    header, bulk = G.obj_to_bulk(z["obj_vertices"], z["obj_faces"])
    path = str(tmp_path / "tri.txt")
    G.write_bulk_file(path, header, bulk)
    d = G.read_bulk_input_abi(path)
    s = G.read_segment_input(d["Input_Segment"], "T")
    P1, P2, P3, un, _, _, us = G.rot_verts_unit_vectors_abi(d["Input_Segment"], s["FaultRakeAngle"])
    cen = s["FaultCenter"]
    Ks, Kn = assemble.assemble_tri(P1, P2, P3, s["FaultRakeAngle"], cen, un, us, d["ShearModulus"],
                                   d["PoissonRatio"])
    Ko_s, Ko_n = oracle_mod.assemble_tri(P1, P2, P3, s["FaultRakeAngle"], cen, un, us, d["ShearModulus"],
                                         d["PoissonRatio"])
    assert np.all(np.isfinite(Ks)) and np.all(np.isfinite(Kn))
    assert _row_rel(Ks, Ko_s, Ko_s, Ko_n) <= 1e-11
    assert _row_rel(Kn, Ko_n, Ko_s, Ko_n) <= 1e-11


@pytest.mark.gpu
def test_main_on_the_reference_bp5qd_input_tracks_the_oracle(qdfn_mod, oracle_mod, tmp_path):
    """The drop-in `main` (FP64) on the reference's default input for 300 steps
    -- a patch starts at 0.03 m/s, so the high-velocity solver runs from step 0
    -- against the oracle's run of the same problem: recorded times, slip and
    slip rate every 10 steps within 1e-9, and the saved file has the reference's
    keys and TotalRecord x N shapes."""
    from qdfn import assemble, simulate
    d, s, rec = _rect_setup(tmp_path, "bp5qd")
    N, Nl = d["FaultCount"], d["LoadingFaultCount"]
    Ks, Kn = assemble.assemble_rect(rec, rec, d["ShearModulus"], d["PoissonRatio"])
    mass = G.fault_mass(s["FaultLengthStrike"], s["FaultLengthDip"], d["RockDensity"])
    rdt = G.rupture_dt(mass, np.diag(Ks), 3.0)
    steps, rstep = 300, 10
    out = str(tmp_path / "Result.npz")
    hist = simulate.main(Ks, Kn, 0, d["ShearModulus"], N, Nl, mass, s["Fault_a"], s["Fault_b"], s["Fault_Dc"],
                         s["Fault_Theta_i"], s["Fault_V_i"], s["Fault_Friction_i"], s["Fault_NormalStress"],
                         s["Fault_V_Const"], steps, rstep, 1e-2, 5.0, rdt, 1e7, out, d["RockDensity"],
                         s["FaultCenter"], s["FaultLengthStrike"], s["FaultLengthDip"], s["FaultStrikeAngle"],
                         s["FaultDipAngle"], s["FaultRakeAngle"], 100, d["MinimumNS"], 0.0, 1,
                         external_stress=None)
    prob = dict(N=N, Nload=Nl, a=s["Fault_a"], b=s["Fault_b"], Dc=s["Fault_Dc"], theta_i=s["Fault_Theta_i"],
                V_i=s["Fault_V_i"], f_i=s["Fault_Friction_i"], sigma0=s["Fault_NormalStress"],
                V_const=s["Fault_V_Const"], mass=mass, G=d["ShearModulus"], rho=d["RockDensity"],
                sigma_min=d["MinimumNS"], switch_v=1e-2, dt_cut=5.0, rupture_dt=rdt, max_dt=1e7, alpha_evo=0.0,
                evolution_dr=1, interp_at_told=0)
    o = oracle_mod.Simulation(prob, ("dense", Ks, Kn))
    oh = o.run(steps, record_step=rstep, max_rec=steps // rstep)
    assert hist["T"].shape[0] == oh["T"].shape[0] == steps // rstep
    assert np.max(np.abs(hist["T"] / oh["T"] - 1)) <= 1e-9
    for k in ("D", "V"):
        assert np.max(np.abs(hist[k] - oh[k])) <= 1e-9 * np.max(np.abs(oh[k])), k
    assert np.max(s["Fault_V_i"][:N - Nl]) > 1e-2            # starts fast: the high-velocity solver runs
    z = np.load(out)
    total = int(round(steps / rstep))
    for k in ("History_V", "History_Disp", "History_Theta", "History_NormalStress"):
        assert z[k].shape == (total, N), k
    assert z["History_Time"].shape == (total, 1)
