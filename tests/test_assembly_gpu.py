"""Stiffness assembly on the GPU vs the FP64 oracle: every entry within 1e-12 of
the row's stress scale, max over the row of max(|K_shear|, |K_normal|).  (The
normal matrix alone is no scale: on coplanar strike-slip patches its exact
value is 0 and the computed entries are rounding noise of ~1e-9 Pa/m.)

Triangles are held to 1e-11: the triangular-dislocation formulas sum three
large angular-dislocation terms into a small result, and a one-ulp change of
the acos/sin/cos/tan results alone moves entries by up to 3e-10 of the row
scale (measured with the oracle).  CUDA's and glibc's transcendentals differ by
an ulp or two, which sets the floor of GPU/CPU agreement near 2e-12."""
import numpy as np
import pytest

from _systems import bumpy_triangles, cols, mixed_rects, small_network

pytestmark = pytest.mark.gpu
TOL = 1e-12
TOL_TRI = 1e-11
G, NU = 32e9, 0.25


def rowrel(A, B, S=None, N=None):
    """max |A - B| / row scale; the scale is max(|S|, |N|) over the row (the
    oracle's shear and normal matrices), or max|B| when they are not given."""
    if S is None:
        scale = np.max(np.abs(B), axis=1, keepdims=True)
    else:
        scale = np.maximum(np.max(np.abs(S), axis=1, keepdims=True), np.max(np.abs(N), axis=1, keepdims=True))
    return float(np.max(np.abs(A - B) / scale))


def test_rect_assembly_matches_oracle(qdfn_mod, oracle_mod):
    from qdfn import assemble
    rec = mixed_rects()
    Ks, Kn = assemble.assemble_rect(rec, rec, G, NU)
    Ko_s, Ko_n = oracle_mod.assemble_rect(cols(rec), cols(rec), G, NU)
    assert not np.isnan(Ks).any()
    assert rowrel(Ks, Ko_s, Ko_s, Ko_n) < TOL
    assert rowrel(Kn, Ko_n, Ko_s, Ko_n) < TOL


def test_rect_network_assembly_matches_oracle(qdfn_mod, oracle_mod):
    from qdfn import assemble
    sysd = small_network()
    rec = sysd["records"]
    Ks, Kn = assemble.assemble_rect(rec, rec, G, NU)
    Ko_s, Ko_n = oracle_mod.assemble_rect(cols(rec), cols(rec), G, NU)
    assert rowrel(Ks, Ko_s, Ko_s, Ko_n) < TOL and rowrel(Kn, Ko_n, Ko_s, Ko_n) < TOL
    assert np.all(np.diag(Ks) < 0)


def test_rect_rectangular_blocks_and_layouts(qdfn_mod, oracle_mod):
    from qdfn import assemble
    rec = mixed_rects()
    src, recv = rec[:17], rec[5:60]
    Ks_r, Kn_r = assemble.assemble_rect(src, recv, G, NU, layout="row")
    Ks_c, Kn_c = assemble.assemble_rect(src, recv, G, NU, layout="col")
    assert Ks_r.shape == (recv.shape[0], src.shape[0])
    assert np.array_equal(Ks_r, Ks_c) and np.array_equal(Kn_r, Kn_c)
    Ko_s, _ = oracle_mod.assemble_rect(cols(src), cols(recv), G, NU)
    assert rowrel(Ks_r, Ko_s) < TOL


def test_rect_empty_input(qdfn_mod):
    from qdfn import assemble
    Ks, Kn = assemble.assemble_rect(np.zeros((0, 8)), np.zeros((0, 8)), G, NU)
    assert Ks.shape == (0, 0)


def test_tri_assembly_matches_oracle(qdfn_mod, oracle_mod):
    from qdfn import assemble, geometry
    seg = bumpy_triangles()
    P1, P2, P3, un, _, _, us = geometry.rot_verts_unit_vectors(seg, seg[:, 9])
    cen = (P1 + P2 + P3) / 3
    Ks, Kn = assemble.assemble_tri(P1, P2, P3, seg[:, 9], cen, un, us, G, NU)
    Ko_s, Ko_n = oracle_mod.assemble_tri(P1, P2, P3, seg[:, 9], cen, un, us, G, NU)
    assert not np.isnan(Ks).any()
    assert rowrel(Ks, Ko_s, Ko_s, Ko_n) < TOL_TRI and rowrel(Kn, Ko_n, Ko_s, Ko_n) < TOL_TRI
    assert np.all(np.diag(Ks) < 0)


def test_tri_edge_receivers_give_nan_like_the_reference(qdfn_mod, oracle_mod):
    from qdfn import assemble
    P1 = np.array([[-1000.0, 0.0, -2000.0]]); P2 = np.array([[1000.0, 0.0, -2000.0]])
    P3 = np.array([[0.0, 0.0, -1000.0]])
    cen = np.array([[0.0, 0.0, -2000.0], [0.0, 300.0, -1500.0]])   # on an edge / off the plane
    n = np.array([[0.0, 1.0, 0.0], [0.0, 1.0, 0.0]]); s = np.array([[1.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    Ks, Kn = assemble.assemble_tri(P1, P2, P3, np.zeros(1), cen, n, s, G, NU)
    Ko, _ = oracle_mod.assemble_tri(P1, P2, P3, np.zeros(1), cen, n, s, G, NU)
    assert np.isnan(Ks[0, 0]) and np.isnan(Ko[0, 0])
    assert abs(Ks[1, 0] - Ko[1, 0]) < TOL_TRI * abs(Ko[1, 0])


def test_tri_rejects_vertices_above_surface(qdfn_mod):
    from qdfn import QdfnError, assemble
    P = np.array([[0.0, 0.0, 10.0]])
    with pytest.raises(QdfnError):
        assemble.assemble_tri(P, P, P, np.zeros(1), np.array([[0.0, 0.0, -5.0]]), np.eye(3)[:1],
                              np.eye(3)[:1], G, NU)


def test_rectangle_equals_two_triangles_on_gpu(qdfn_mod):
    """Okada and TDstressHS kernels agree on the same planar patch."""
    from qdfn import assemble, geometry, synth
    rec = synth.grid_fault(0.0, 0.0, 2500.0, 2000.0, 1000.0, 0.0, 60.0, 30.0, 1000.0)   # 2 patches
    Ks_r, Kn_r = assemble.assemble_rect(rec, rec, G, NU)
    # each rectangle split in two triangles; receivers = rectangle centres
    tri = []
    for r in rec:
        cx, cy, cz, L, W, st, dp, rk = r
        cd, sd = np.cos(np.radians(dp)), np.sin(np.radians(dp))
        c = lambda xs, ws: np.array([cx + xs * L / 2, cy + ws * W / 2 * cd, -cz + ws * W / 2 * sd])
        A, B, C, D = c(-1, -1), c(1, -1), c(1, 1), c(-1, 1)
        tri += [(A, B, C), (A, C, D)]
    seg = np.zeros((len(tri), 20))
    for t, (a, b, c) in enumerate(tri):
        seg[t, 0:3], seg[t, 3:6], seg[t, 6:9], seg[t, 9] = a, b, c, rec[0, 7]
    P1, P2, P3, un, _, _, us = geometry.rot_verts_unit_vectors(seg, seg[:, 9])
    cen = np.column_stack([rec[:, 0], rec[:, 1], -rec[:, 2]])
    nrm = np.repeat(un[::2], 1, axis=0)
    sl = np.repeat(us[::2], 1, axis=0)
    Ks_t, Kn_t = assemble.assemble_tri(P1, P2, P3, seg[:, 9], cen, nrm, sl, G, NU)
    Ks_t2 = Ks_t[:, 0::2] + Ks_t[:, 1::2]
    Kn_t2 = Kn_t[:, 0::2] + Kn_t[:, 1::2]
    # a rectangle's own centre lies on the diagonal shared by its two triangles
    # (an edge point: NaN, as in the reference), so compare the cross terms
    off = ~np.eye(rec.shape[0], dtype=bool)
    assert np.all(np.isnan(np.diag(Ks_t2)))
    # triangle slip convention (Ss = -cos(rake)) vs Okada's: compare magnitudes
    scale = np.max(np.abs(Ks_r))
    assert np.max(np.abs(np.abs(Ks_t2[off]) - np.abs(Ks_r[off]))) < 1e-9 * scale
    assert np.max(np.abs(np.abs(Kn_t2[off]) - np.abs(Kn_r[off]))) < 1e-9 * scale
