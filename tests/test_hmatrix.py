"""H-matrix operator: block structure (CPU) and the device operator and
simulation against the oracle's H path and against the dense operator (GPU)."""
import numpy as np
import pytest

from _systems import cols, mixed_rects, problem_for, small_network

G, NU = 32e9, 0.25


def test_cluster_tree_is_a_permutation_with_contiguous_nodes():
    from qdfn.hmatrix import ClusterTree
    pts = np.random.default_rng(0).uniform(-1000, 1000, (700, 3))
    t = ClusterTree(pts, leaf=32)
    assert sorted(t.perm.tolist()) == list(range(700))
    for k, ch in enumerate(t.children):
        if ch:
            a, b = ch
            assert t.starts[a] == t.starts[k] and t.ends[a] == t.starts[b] and t.ends[b] == t.ends[k]
        else:
            assert t.ends[k] - t.starts[k] <= 32


def test_block_partition_covers_the_matrix_once():
    from qdfn.hmatrix import ClusterTree, block_partition
    pts = np.random.default_rng(1).uniform(-5000, 5000, (500, 3))
    t = ClusterTree(pts, leaf=24)
    cover = np.zeros((500, 500), dtype=int)
    nadm = 0
    for s, r, adm in block_partition(t, eta=2.0):
        cover[t.starts[r]:t.ends[r], t.starts[s]:t.ends[s]] += 1
        nadm += adm
        if adm:
            assert max(t.diam(s), t.diam(r)) <= 2.0 * t.dist(s, r)
    assert np.all(cover == 1)
    assert nadm > 0


def test_touching_boxes_and_repeated_centres_are_never_admissible():
    """Blocks whose boxes touch (distance 0) stay dense even when both boxes
    are points: a single element, and clusters of identical centres."""
    from qdfn.hmatrix import ClusterTree, block_partition, host_partition
    perm, spans = host_partition(np.array([[1.0, 2.0, 3.0]]), leaf=8)
    assert spans == [(0, 1, 0, 1, False)]
    pts = np.repeat(np.array([[0.0, 0.0, 0.0], [5000.0, 0.0, 0.0]]), 20, axis=0)
    t = ClusterTree(pts, leaf=4)
    for s, r, adm in block_partition(t, eta=2.0):
        if adm:
            assert t.dist(s, r) > 0
        else:
            assert t.ends[s] - t.starts[s] <= 4 and t.ends[r] - t.starts[r] <= 4
    # the two clusters, 5 km apart and each a point, are low-rank to each other
    assert any(adm for _, _, adm in block_partition(t, eta=2.0))


@pytest.mark.gpu
def test_hmatrix_operator_matches_dense_and_oracle(qdfn_mod, oracle_mod):
    from qdfn import assemble, hmatrix, simulate, synth
    sysd = small_network(seed=5, n_faults=6, patch=250.0)
    rec = sysd["records"]
    H, perm = hmatrix.build_rect(rec, G, NU, leaf=32, eta=2.0, tol=1e-8)
    recp = rec[perm]
    N = rec.shape[0]
    assert H.stored_entries() < 2 * N * N
    Ks, Kn = assemble.assemble_rect(recp, recp, G, NU)
    Hs, Hn = H.to_dense(N)
    assert np.linalg.norm(Hs - Ks) < 1e-7 * np.linalg.norm(Ks)
    assert np.linalg.norm(Hn - Kn) < 1e-7 * np.linalg.norm(Ks)
    prob = problem_for(recp, Ks)
    prob["interp_at_told"] = 1
    sim = simulate.Simulation(prob)
    hmatrix.set_hmatrix(sim, H, "fp64")
    D = np.random.default_rng(2).uniform(0, 1, N)
    tld, knd = sim.apply(D)
    blocks = dict(range=H.ranges, sD=H.dense_s, sU=H.U_s, sVt=H.Vt_s, nD=H.dense_n, nU=H.U_n, nVt=H.Vt_n)
    o = oracle_mod.Simulation(dict(prob), ("hmat", blocks))
    otld, oknd = o.apply(D)
    rel = lambda a, b: np.max(np.abs(a - b)) / np.max(np.abs(b))
    assert rel(tld[0], otld) < 1e-12 and rel(knd[0], oknd) < 1e-12
    assert np.allclose(sim.kself(), o.kself(), rtol=0, atol=0)
    # against the dense operator: main_H divides after the product, main before
    od = oracle_mod.Simulation(dict(prob), ("dense", Ks, Kn))
    dt, dk = od.apply(D)
    assert rel(tld[0], dt) < 1e-6 and rel(knd[0], dk) < 1e-6


@pytest.mark.gpu
def test_hmatrix_trajectory_matches_oracle(qdfn_mod, oracle_mod):
    from qdfn import hmatrix, simulate, synth
    sysd = small_network(seed=5, n_faults=6, patch=250.0)
    rec = sysd["records"]
    H, perm = hmatrix.build_rect(rec, G, NU, leaf=32, eta=2.0, tol=1e-8)
    recp = rec[perm]
    Hs, _ = H.to_dense(rec.shape[0])
    prob = problem_for(recp, Hs)
    prob["interp_at_told"] = 1
    ext = synth.external_ramp(rec.shape[0], 1e6, 1e11)
    for prec, tol in (("fp64", 1e-9), ("fp32", 1e-4)):
        sim = simulate.Simulation(prob)
        hmatrix.set_hmatrix(sim, H, prec)
        sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
        sim.run(200, timeout_s=120)
        blocks = dict(range=H.ranges, sD=H.dense_s, sU=H.U_s, sVt=H.Vt_s, nD=H.dense_n, nU=H.U_n, nVt=H.Vt_n)
        o = oracle_mod.Simulation(dict(prob, ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"],
                                       ext_p=ext["pressure"]), ("hmat", blocks))
        o.run(200)
        st = sim.state(0)
        assert st["step"] == 200
        assert abs(st["T"] / o.T - 1) < tol
        assert np.max(np.abs(st["D"] - o.state["D"])) / np.max(np.abs(o.state["D"])) < tol


def _tri_system(nx=32, ny=20, seed=1):
    from qdfn import geometry
    from _systems import bumpy_triangles
    seg = bumpy_triangles(nx=nx, ny=ny, seed=seed)
    P1, P2, P3, un, _, _, us = geometry.rot_verts_unit_vectors(seg, seg[:, 9])
    cen = (P1 + P2 + P3) / 3
    return P1, P2, P3, seg[:, 9].copy(), cen, un, us


@pytest.mark.gpu
def test_triangle_hmatrix_aca_on_demand_matches_dense_and_oracle(qdfn_mod, oracle_mod):
    """A curved triangulated fault (1,280 TDstressHS elements, leaf 32, eta 2):
    ACA forms its rows and columns from the triangle kernel on index ranges (no
    admissible block assembled whole); the compressed operator equals the dense
    triangle operator to the ACA tolerance, and the device H product (warp tasks)
    equals the oracle's H product of the same blocks to 1e-12, in FP64 and
    with FP32 block storage to its rounding."""
    from qdfn import assemble, hmatrix, simulate
    P1, P2, P3, rake, cen, un, us = _tri_system()
    N = P1.shape[0]
    H, perm = hmatrix.build_tri(P1, P2, P3, rake, cen, un, us, G, NU, leaf=32, eta=2.0, tol=1e-8)
    assert any(U is not None for U in H.U_s) and H.stored_entries() < 2 * N * N
    Ks, Kn = assemble.assemble_tri(P1[perm], P2[perm], P3[perm], rake[perm], cen[perm], un[perm], us[perm], G, NU)
    Hs, Hn = H.to_dense(N)
    assert np.linalg.norm(Hs - Ks) <= 1e-6 * np.linalg.norm(Ks)
    assert np.linalg.norm(Hn - Kn) <= 1e-6 * np.linalg.norm(Kn)
    recp = np.column_stack([cen[perm], np.full((N, 2), 80.0), np.zeros((N, 3))])
    prob = problem_for(recp, Hs, seed=2)
    prob["interp_at_told"] = 1
    blocks = dict(range=H.ranges, sD=H.dense_s, sU=H.U_s, sVt=H.Vt_s, nD=H.dense_n, nU=H.U_n, nVt=H.Vt_n)
    o = oracle_mod.Simulation(dict(prob), ("hmat", blocks))
    D = np.random.default_rng(4).uniform(0, 1, N)
    otld, oknd = o.apply(D)
    rel = lambda a, b: np.max(np.abs(a - b)) / np.max(np.abs(b))
    for prec, tol in (("fp64", 1e-12), ("fp32", 2e-6)):
        sim = simulate.Simulation(prob)
        hmatrix.set_hmatrix(sim, H, prec)
        tld, knd = sim.apply(D)
        assert rel(tld[0], otld) < tol and rel(knd[0], oknd) < tol, prec
        sim.close()
