"""Reservoir-cuboid coupling (the reference's CuboidCoupling module): input
files, the cuboid Green's functions and the forcing on fault patches.  Host
code: runs without a GPU."""
import math

import numpy as np
import pytest

from qdfn import cuboids as Cb
from qdfn import geometry as Gm


def _scalar_gf(p, centre, length, cm, G, pi):
    """One point, one cuboid, written out term by term (an independent
    restatement of the vectorised Green's function)."""
    V = Cb.cuboid_vertices(centre, length)
    S = [-1, 1, 1, -1, 1, -1, -1, 1]
    pd, ps = cm / (4 * pi), cm * G / (2 * pi)

    def f(x, y, z, R):
        return z * math.atan((x * y) / (z * R)) - x * math.log(abs(R + y)) - y * math.log(abs(R + x))
    d = [0.0, 0.0, 0.0]
    s = [0.0] * 6
    for j in range(8):
        xb, yb, zm = V[j, 0] - p[0], V[j, 1] - p[1], V[j, 2] - p[2]
        rm = math.sqrt(xb * xb + yb * yb + zm * zm)
        d[0] += pd * S[j] * f(yb, zm, xb, rm)
        d[1] += pd * S[j] * f(xb, zm, yb, rm)
        d[2] += -pd * S[j] * f(xb, yb, zm, rm)
        s[0] += ps * S[j] * math.atan((xb * rm) / (yb * zm))
        s[1] += ps * S[j] * math.atan((yb * rm) / (xb * zm))
        s[2] += ps * S[j] * math.atan((zm * rm) / (xb * yb))
        s[3] += -ps * S[j] * math.log(rm - zm)
        s[4] += ps * S[j] * math.log(rm + yb)
        s[5] += ps * S[j] * math.log(rm + xb)
    return np.array(d), np.array(s)


def test_vertices_in_module_order():
    V = Cb.cuboid_vertices([1.0, 2.0, 3.0], [2.0, 4.0, 6.0])
    assert V.tolist() == [[0, 0, 0], [2, 0, 0], [0, 4, 0], [2, 4, 0], [0, 0, 6], [2, 0, 6], [0, 4, 6], [2, 4, 6]]


def test_green_functions_match_a_scalar_restatement():
    rng = np.random.default_rng(2)
    centres = np.array([[0.0, 0.0, 3000.0], [2500.0, -800.0, 2500.0]])
    lengths = np.array([[4000.0, 2000.0, 200.0], [1000.0, 1000.0, 500.0]])
    pts = np.column_stack([rng.uniform(-6e3, 6e3, 15), rng.uniform(-6e3, 6e3, 15), rng.uniform(500, 6e3, 15)])
    disp, sig = Cb.green_functions(pts, centres, lengths, 1e-11, 3e10)
    for i in range(pts.shape[0]):
        for j in range(2):
            d, s = _scalar_gf(pts[i], centres[j], lengths[j], 1e-11, 3e10, Cb.REFERENCE_PI)
            assert np.allclose(disp[:, i, j], d, rtol=1e-10, atol=1e-22)
            assert np.allclose(sig[:, i, j], s, rtol=1e-10, atol=1e-12)


def test_stress_outside_a_dilating_cuboid_is_deviatoric_and_decays():
    """Outside a uniformly dilating inclusion in a full space the stress has
    no trace (inside it is 4 Cm G per unit pressure); far away it falls off as
    r^-3."""
    c, L = np.array([[0.0, 0.0, 5000.0]]), np.array([[1000.0, 800.0, 600.0]])
    dirs = np.array([[1.0, 0.3, 0.2], [0.2, -1.0, 0.5], [-0.4, 0.1, 1.0]])
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    for dv in dirs:
        pts = c[0] + np.outer([3e3, 6e3, 1.2e4], dv)
        _, s = Cb.green_functions(pts, c, L, 1e-11, 3e10, pi=math.pi)
        s = s[:, :, 0]
        trace, mag = s[0] + s[1] + s[2], np.max(np.abs(s[:3]), axis=0)
        assert np.all(np.abs(trace) <= 1e-8 * mag)
        ratio = np.max(np.abs(s), axis=0)
        assert ratio[0] / ratio[1] == pytest.approx(8.0, rel=0.15)   # (6/3)^3
        assert ratio[1] / ratio[2] == pytest.approx(8.0, rel=0.15)
    _, s = Cb.green_functions(np.array([[0.0, 0.0, 5000.0], [100.0, 50.0, 5100.0]]), c, L, 1e-11, 3e10, pi=math.pi)
    assert np.allclose(s[0] + s[1] + s[2], 4 * 1e-11 * 3e10, rtol=1e-12)


def test_input_files_and_forcing(tmp_path):
    (tmp_path / "cub.txt").write_text("Index, CenterX, CenterY, CenterZ, LengthX, LengthY, LengthZ\n"
                                      "1, 0, 0, 3000, 4000, 2000, 200\n2, 5000, 0, 3000, 1000, 1000, 200\n")
    (tmp_path / "pp.txt").write_text("time(sec), 0.0, 1.0e8, 2.0e8\ncuboid1, 0.0, -1.0e7, -2.0e7\n"
                                     "cuboid2, 0.0, 5.0e6, 1.0e7\n")
    (tmp_path / "tt.txt").write_text("time(sec), 0.0, 1.0e8, 2.0e8\ncuboid1, 0.0, 0.0, -10.0\ncuboid2, 0, 0, 0\n")
    cen, lens = Cb.read_cuboids(str(tmp_path / "cub.txt"))
    assert cen.tolist() == [[0, 0, 3000], [5000, 0, 3000]] and lens.tolist() == [[4000, 2000, 200], [1000, 1000, 200]]
    t, pp = Cb.read_history(str(tmp_path / "pp.txt"))
    _, tt = Cb.read_history(str(tmp_path / "tt.txt"))
    assert t.tolist() == [0.0, 1e8, 2e8] and pp.shape == (3, 2) and pp[2].tolist() == [-2e7, 1e7]
    # three patches: inside cuboid 1, inside cuboid 2, outside both
    fc = np.array([[100.0, 50.0, 3000.0], [5100.0, 0.0, 3050.0], [0.0, 3000.0, 3000.0]])
    G, nu = 3e10, 0.25
    out = Cb.fault_forcing(fc, np.array([0.0, 30.0, 90.0]), np.full(3, 90.0), np.array([0.0, 90.0, 180.0]),
                           G, nu, cen, lens, t, pp, tt)
    assert out["normal"].shape == out["shear"].shape == out["pressure"].shape == (3, 3)
    assert out["pressure"][:, 0].tolist() == pp[:, 0].tolist()
    assert out["pressure"][:, 1].tolist() == pp[:, 1].tolist()
    assert np.all(out["pressure"][:, 2] == 0)
    assert np.all(out["normal"][0] == 0) and np.all(out["shear"][0] == 0)   # no change at t = 0
    # linear in the histories: doubling them doubles the forcing
    out2 = Cb.fault_forcing(fc, np.array([0.0, 30.0, 90.0]), np.full(3, 90.0), np.array([0.0, 90.0, 180.0]),
                            G, nu, cen, lens, t, 2 * pp, 2 * tt)
    assert np.allclose(out2["normal"], 2 * out["normal"], rtol=1e-12, atol=1e-6)
    assert np.allclose(out2["shear"], 2 * out["shear"], rtol=1e-12, atol=1e-6)
    # the fault-frame rotation for a vertical east-striking patch (strike 90, dip 90)
    R = np.array([[1, 0, 0], [0, Gm.cosd(-90.0), -Gm.sind(-90.0)], [0, Gm.sind(-90.0), Gm.cosd(-90.0)]]) @ \
        np.array([[Gm.cosd(-90.0), -Gm.sind(-90.0), 0], [Gm.sind(-90.0), Gm.cosd(-90.0), 0], [0, 0, 1]])
    ps = out["poro_stress"][:, 2, 2]        # time 2, patch 2 (strike 90, dip 90, rake 180)
    eff = -np.array([[ps[0], ps[3], ps[4]], [ps[3], ps[1], ps[5]], [ps[4], ps[5], ps[2]]]) + out["pressure"][2, 2] * np.eye(3)
    sf = R @ eff @ R.T
    assert out["normal"][2, 2] == pytest.approx(-sf[2, 2], rel=1e-12, abs=1e-6)
    assert out["shear"][2, 2] == pytest.approx(Gm.cosd(180.0) * sf[0, 2] + Gm.sind(180.0) * sf[1, 2], rel=1e-12,
                                               abs=1e-6)


def test_triangle_projection_agrees_with_the_rotation():
    """For a patch given by its unit normal and slip vector the traction
    projection equals the strike/dip rotation of the rectangle path."""
    rng = np.random.default_rng(5)
    n = 6
    fc = np.column_stack([rng.uniform(-2e3, 2e3, n), rng.uniform(-2e3, 2e3, n), rng.uniform(2e3, 4e3, n)])
    strike, dip, rake = rng.uniform(0, 180, n), rng.uniform(30, 90, n), rng.uniform(-180, 180, n)
    cen, lens = np.array([[0.0, 0.0, 3000.0]]), np.array([[3000.0, 3000.0, 300.0]])
    t = np.array([0.0, 1e8])
    pp = np.array([[0.0], [-1e7]])
    a = Cb.fault_forcing(fc, strike, dip, rake, 3e10, 0.25, cen, lens, t, pp)
    nv, sv = np.zeros((n, 3)), np.zeros((n, 3))
    for i in range(n):
        Rs = np.array([[Gm.cosd(-strike[i]), -Gm.sind(-strike[i]), 0], [Gm.sind(-strike[i]), Gm.cosd(-strike[i]), 0],
                       [0, 0, 1]])
        Rd = np.array([[1, 0, 0], [0, Gm.cosd(-dip[i]), -Gm.sind(-dip[i])], [0, Gm.sind(-dip[i]), Gm.cosd(-dip[i])]])
        Rm = Rd @ Rs
        nv[i] = Rm[2]
        sv[i] = Gm.cosd(rake[i]) * Rm[0] + Gm.sind(rake[i]) * Rm[1]
    b = Cb.fault_forcing(fc, None, None, None, 3e10, 0.25, cen, lens, t, pp, normals=nv, slips=sv)
    assert np.allclose(a["normal"], b["normal"], rtol=1e-10, atol=1e-4)
    assert np.allclose(a["shear"], b["shear"], rtol=1e-10, atol=1e-4)
    assert np.array_equal(a["pressure"], b["pressure"])
