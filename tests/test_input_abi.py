"""The input front end in the C ABI (qdfn_read_bulk_input, qdfn_bulk_to_segment,
qdfn_rot_verts_unit_vectors) gives what the Python restatement gives:
ReadBulkInput / LRtoRake / BulkToSegment / RotVerts_UnitVectors
(scripts/Functions_BuildInputFile.jl:82-377).  Host code only: runs without a
GPU.  Tolerances cover the last-ulp differences of 3x3 products (numpy may
fuse or reorder them)."""
import numpy as np
import pytest

from qdfn import geometry as G

TOL = 1e-12


def _write_bulk(path, rows, header=(1, 3.2e10, 0.25, 2670.0, 1.05, 0.6, 2.0e6)):
    lines = ["SwitchSS/RN\tShearMod\tPoissonRatio\tR_Density\tCrit_TooClose\tTooCloseNormal_Multiplier\tMinimum_NS",
             "\t".join(repr(float(x)) for x in header),
             "\t".join("c%d" % k for k in range(len(rows[0])))]
    lines += ["\t".join(repr(float(x)) for x in r) for r in rows]
    path.write_text("\n".join(lines) + "\n")


def _rect_rows(rng, n):
    rows = []
    for k in range(n):
        rows.append([rng.uniform(-5e3, 5e3), rng.uniform(-5e3, 5e3), rng.uniform(2e3, 7e3),
                     rng.uniform(1e3, 4e3), rng.uniform(5e2, 2e3), rng.uniform(0, 180), rng.uniform(45, 90),
                     float(rng.choice([-1.0, 1.0])), 0.01, 0.015, 1e-3, 1e6, 1e-9, 0.6, 1e7, 1.8e4,
                     float(rng.choice([0.0, 0.0, 0.0, 1e-9])), float(rng.choice([250.0, 400.0, 700.0]))])
    return rows


@pytest.mark.parametrize("switch", [1, 2])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_read_bulk_rectangles_matches_python(qdfn_mod, tmp_path, switch, seed):
    rng = np.random.default_rng(seed)
    p = tmp_path / "bulk.txt"
    _write_bulk(p, _rect_rows(rng, 6), header=(switch, 3.2e10, 0.25, 2670.0, 1.05, 0.6, 2.0e6))
    a = G.read_bulk_input(str(p))
    b = G.read_bulk_input_abi(str(p))
    for k in ("Switch_StrikeSlip_or_ReverseNormal", "ShearModulus", "PoissonRatio", "RockDensity", "DropCrit",
              "DropCritNormalStressMultiplier", "MinimumNS", "RorT", "LoadingFaultCount", "FaultCount"):
        assert a[k] == b[k], k
    sa, sb = a["Input_Segment"], b["Input_Segment"]
    assert sa.shape == sb.shape and sa.shape[1] == 19
    # the integer-valued and copied columns exactly, the centres to rounding
    assert np.array_equal(sa[:, 3:14], sb[:, 3:14]) and np.array_equal(sa[:, 15:], sb[:, 15:])
    scale = np.max(np.abs(sa[:, 0:3]))
    assert np.max(np.abs(sa[:, 0:3] - sb[:, 0:3])) <= TOL * scale
    assert np.allclose(sa[:, 14], sb[:, 14], rtol=TOL, atol=0)


def test_read_bulk_triangles_matches_python(qdfn_mod, tmp_path):
    rng = np.random.default_rng(7)
    rows = []
    for k in range(9):
        P = rng.uniform(-3e3, 3e3, (3, 3))
        P[:, 2] = -np.abs(P[:, 2]) - 100.0
        rows.append(list(P.ravel()) + [30.0 * (k % 4), 0.01, 0.015, 1e-3, 1e6, 1e-9, 0.6, 1e7, 1.8e4,
                                        float(k % 3 == 0) * 1e-9, 500.0])
    p = tmp_path / "tri.txt"
    _write_bulk(p, rows)
    a = G.read_bulk_input(str(p))
    b = G.read_bulk_input_abi(str(p))
    assert a["RorT"] == b["RorT"] == "T"
    assert a["LoadingFaultCount"] == b["LoadingFaultCount"] and a["FaultCount"] == b["FaultCount"] == 9
    assert np.array_equal(a["Input_Segment"], b["Input_Segment"])


def test_bulk_to_segment_matches_python(qdfn_mod):
    bulk = np.zeros((2, 18))
    bulk[0, :] = [100.0, 200.0, 5000.0, 4000.0, 2000.0, 30.0, 60.0, 0.0, 0.01, 0.015, 1e-3, 1e6, 1e-9, 0.6,
                  1e7, 2000.0, 0.0, 500.0]
    bulk[1, :] = [0.0, 0.0, 3000.0, 800.0, 600.0, 90.0, 90.0, 180.0, 0.01, 0.015, 1e-3, 1e6, 1e-9, 0.6,
                  1e7, 0.0, 1e-9, 1000.0]   # one patch: the centre is copied
    a, b = G.bulk_to_segment(bulk), G.bulk_to_segment_abi(bulk)
    assert a.shape == b.shape == (8 * 4 + 1, 19)
    assert np.max(np.abs(a - b)) <= TOL * np.max(np.abs(a))
    assert np.array_equal(a[-1], b[-1])


def test_rot_verts_unit_vectors_matches_python(qdfn_mod):
    rng = np.random.default_rng(11)
    n = 40
    seg = np.zeros((n, 10))
    seg[:, 0:9] = rng.uniform(-2e3, 2e3, (n, 9))
    seg[:, 9] = rng.uniform(-180, 180, n)
    seg[::5, 9] = 90.0   # exact right angles
    a = G.rot_verts_unit_vectors(seg, seg[:, 9])
    b = G.rot_verts_unit_vectors_abi(seg, seg[:, 9])
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)      # vertex swap decisions and copies
    for x, y in zip(a[3:], b[3:]):
        assert np.max(np.abs(x - y)) <= 1e-15


def test_malformed_bulk_files_are_rejected(qdfn_mod, tmp_path):
    from qdfn import _lib
    p = tmp_path / "bad.txt"
    p.write_text("h\n1 2 3\nh\n1 2 3 4 5\n")
    with pytest.raises(_lib.QdfnError):
        G.read_bulk_input_abi(str(p))
    rows = _rect_rows(np.random.default_rng(0), 2)
    q = tmp_path / "nan.txt"
    _write_bulk(q, rows)
    txt = q.read_text().replace(repr(float(rows[1][4])), "abc", 1)
    q.write_text(txt)
    with pytest.raises(_lib.QdfnError):
        G.read_bulk_input_abi(str(q))
    with pytest.raises(_lib.QdfnError):
        G.read_bulk_input_abi(str(tmp_path / "missing.txt"))
    bulk = np.zeros((1, 18))
    with pytest.raises(_lib.QdfnError):   # zero lengths: no finite gridding
        G.bulk_to_segment_abi(bulk)
