"""Host-side input parsing and discretisation (ReadBulkInput, BulkToSegment,
ReadSegmentInput, RotVerts_UnitVectors)."""
import os

import numpy as np
import pytest

from qdfn import geometry as G

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_sind_cosd_exact_at_right_angles():
    for d, s, c in [(0, 0, 1), (90, 1, 0), (180, 0, -1), (270, -1, 0), (-90, -1, 0), (450, 1, 0)]:
        assert G.sind(d) == s and G.cosd(d) == c
    for d in np.linspace(-720, 720, 97):
        assert abs(G.sind(d) - np.sin(np.radians(d))) < 1e-15
        assert abs(G.cosd(d) - np.cos(np.radians(d))) < 1e-15


def _write_bulk(path, rows, header=(1, 3.2e10, 0.25, 2670.0, 1.05, 0.6, 2.0e6)):
    lines = ["SwitchSS/RN\tShearMod\tPoissonRatio\tR_Density\tCrit_TooClose\tTooCloseNormal_Multiplier\tMinimum_NS",
             "\t".join(repr(float(x)) for x in header),
             "\t".join("c%d" % k for k in range(len(rows[0])))]
    lines += ["\t".join(repr(float(x)) for x in r) for r in rows]
    path.write_text("\n".join(lines) + "\n")


def test_bulk_file_is_gridded(tmp_path):
    # three vertical strike-slip bulk faults, 1 km MaxLeng
    rows = [[0.0, -20000.0, 8000.0, 12000.0, 12000.0, 90.0, 90.0, 1.0, 0.004, 0.03, 0.13, 1.3e8, 0.03, 0.6,
             2.5e7, 0.0, 0.0, 1000.0],
            [0.0, 6000.0, 8000.0, 40000.0, 12000.0, 90.0, 90.0, 1.0, 0.004, 0.03, 0.14, 1.4e8, 1e-9, 0.6,
             2.5e7, 0.0, 0.0, 1000.0],
            [0.0, 0.0, 1500.0, 52500.0, 1000.0, 90.0, 90.0, -1.0, 0.03, 0.03, 0.14, 1.4e8, 1e-9, 0.6,
             2.5e7, 0.0, 0.0, 1000.0]]
    p = tmp_path / "bulk.txt"
    _write_bulk(p, rows)
    d = G.read_bulk_input(str(p))
    assert d["RorT"] == "R"
    assert d["ShearModulus"] == 3.2e10 and d["PoissonRatio"] == 0.25 and d["MinimumNS"] == 2.0e6
    seg = d["Input_Segment"]
    assert d["FaultCount"] == seg.shape[0] == 12 * 12 + 40 * 12 + 53 * 1
    assert seg.shape[1] == 19 and d["LoadingFaultCount"] == 0
    # LR = +1 -> rake 180, -1 -> rake 0 (switch 1)
    assert set(np.unique(seg[:, 7])) == {0.0, 180.0}


def test_bulk_to_segment_preserves_area_and_centre():
    bulk = np.zeros((1, 18))
    bulk[0, :] = [100.0, 200.0, 5000.0, 4000.0, 2000.0, 30.0, 60.0, 0.0, 0.01, 0.015, 1e-3, 1e6, 1e-9, 0.6,
                  1e7, 2000.0, 0.0, 500.0]
    seg = G.bulk_to_segment(bulk)
    assert seg.shape == (8 * 4, 19)
    assert np.isclose(np.sum(seg[:, 3] * seg[:, 4]), 4000.0 * 2000.0)
    assert np.allclose(seg[:, 0:3].mean(axis=0), [100.0, 200.0, 5000.0], atol=1e-9)
    # normal stress = Sig0 + SigGrad * depth
    assert np.allclose(seg[:, 14], 1e7 + 2000.0 * seg[:, 2])
    # all patch centres lie on the fault plane
    n = np.array([G.cosd(30.0) * G.sind(60.0) * -1, G.sind(30.0) * G.sind(60.0) * -1, 0.0])
    rs = np.array([[G.cosd(30), -G.sind(30), 0], [G.sind(30), G.cosd(30), 0], [0, 0, 1]])
    rd = np.array([[1, 0, 0], [0, G.cosd(60), -G.sind(60)], [0, G.sind(60), G.cosd(60)]])
    normal = rs @ rd @ np.array([0, 0, 1.0])
    rel = (seg[:, 0:3] * np.array([1, 1, -1])) - np.array([100.0, 200.0, -5000.0])
    assert np.max(np.abs(rel @ normal)) < 1e-9


def test_lr_to_rake_modes():
    bulk = np.zeros((4, 18))
    bulk[:, 6] = [60, 60, 120, 120]
    bulk[:, 7] = [-1, 1, -1, 1]
    assert list(G.lr_to_rake(1, bulk)[:, 7]) == [0, 180, 0, 180]
    assert list(G.lr_to_rake(2, bulk)[:, 7]) == [90, 270, 270, 90]


def test_wrong_column_count_is_an_error(tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("h\n1 2 3 4 5 6 7\nh\n" + " ".join(["1"] * 17) + "\n")
    with pytest.raises(G.InputFormatError):
        G.read_bulk_input(str(p))


def test_loading_faults_are_moved_last(tmp_path):
    rows = []
    for k, vc in enumerate([1e-9, 0.0, 0.0]):
        rows.append([0.0, 5000.0 * k, 5000.0, 2000.0, 2000.0, 90, 90, 1, 0.01, 0.015, 1e-3, 1e6, 1e-9, 0.6,
                     1e7, 0.0, vc, 1000.0])
    p = tmp_path / "b.txt"
    p.write_text("h\n1 3.2e10 0.25 2670 1.05 0.6 1e6\nh\n" + "\n".join(" ".join(str(x) for x in r) for r in rows))
    d = G.read_bulk_input(str(p))
    seg = d["Input_Segment"]
    assert d["LoadingFaultCount"] == 4
    assert np.all(seg[-4:, 15] > 0) and np.all(seg[:-4, 15] == 0)


def test_triangle_vertices_are_flipped_to_positive_normal_y():
    seg = np.zeros((2, 20))
    seg[0, 0:9] = [0, 0, -1000, 1000, 0, -1000, 0, 0, -2000]       # normal along -y -> flipped
    seg[1, 0:9] = [0, 0, -1000, 0, 0, -2000, 1000, 0, -1000]        # normal along +y
    P1, P2, P3, un, us, ud, uslip = G.rot_verts_unit_vectors(seg, np.array([0.0, 90.0]))
    assert np.all(un[:, 1] > 0)
    assert np.allclose(np.linalg.norm(uslip, axis=1), 1.0)
    assert np.allclose(uslip[1], ud[1])
