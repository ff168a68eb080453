"""The H-matrix structure built on the device (qdfn_hstruct_*: k-d cluster
tree of median splits, block partition) against a host restatement of the
same rules -- the permutation and the block list must be equal, element for
element -- plus the partition's invariants and an operator compressed on it.

The rules restated here: level by level, every node of more than `leaf`
elements orders its elements by the centre coordinate along the longest axis
of its box (the lower axis on ties; equal coordinates by element index) and
splits its range into halves (first half = floor(n / 2)); boxes are the
min/max of a node's centres; a (receiver, source) node pair is
low-rank when dist > 0 and max(diam) <= eta * dist (diam = box diagonal, dist
= box-to-box distance, each sqrt((x*x + y*y) + z*z)), dense when both are
leaves, else split (a leaf stands in for its children).  These replace the
reference's k-means tree (scripts/Functions_Hmatrix.jl:1-212), which is
randomly initialised and not reproducible."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
G, NU = 32e9, 0.25


def _host_structure(c, leaf, eta):
    N = c.shape[0]
    start, end, child, level = [0], [N], [], [0]
    v = 0
    while v < len(start):   # the tree's shape: level order, halving
        n = end[v] - start[v]
        if n > leaf:
            h = n // 2
            child.append((len(start), len(start) + 1))
            start += [start[v], start[v] + h]
            end += [start[v] + h, end[v]]
            level += [level[v] + 1, level[v] + 1]
        else:
            child.append(None)
        v += 1
    order = np.arange(N)
    lo, hi = [None] * len(start), [None] * len(start)
    for lv in range(max(level) + 1):   # boxes, then each splitting node sorted along its longest axis
        for v in (k for k in range(len(start)) if level[k] == lv):
            pts = c[order[start[v]:end[v]]]
            lo[v], hi[v] = pts.min(axis=0), pts.max(axis=0)
            if child[v] is not None:
                ax = int(np.argmax(hi[v] - lo[v]))
                seg = order[start[v]:end[v]]
                order[start[v]:end[v]] = seg[np.lexsort((seg, pts[:, ax] + 0.0))]
    perm = order
    norm = lambda x: float(np.sqrt((x[0] * x[0] + x[1] * x[1]) + x[2] * x[2]))
    blocks = []
    stack = [(0, 0)]
    while stack:
        t, s = stack.pop()
        dt, ds = norm(hi[t] - lo[t]), norm(hi[s] - lo[s])
        gap = np.maximum(0.0, np.maximum(lo[t] - hi[s], lo[s] - hi[t]))
        dist = norm(gap)
        adm = dist > 0 and max(dt, ds) <= eta * dist
        if adm or (child[t] is None and child[s] is None):
            blocks.append((start[s], end[s], start[t], end[t], bool(adm)))
            continue
        for a in (child[t] or (t,)):
            for b in (child[s] or (s,)):
                stack.append((a, b))
    return perm, sorted(blocks, key=lambda b: (b[2], b[0]))


def _check(c, leaf, eta):
    from qdfn import hmatrix
    perm, spans = hmatrix.device_partition(c, leaf, eta)
    hperm, hspans = _host_structure(c, leaf, eta)
    assert np.array_equal(perm, hperm)
    assert spans == hspans
    N = c.shape[0]
    cover = np.zeros((N, N), dtype=np.int32) if N <= 4096 else None
    for (s0, s1, r0, r1, adm) in spans:
        assert 0 <= s0 < s1 <= N and 0 <= r0 < r1 <= N
        if not adm:
            assert s1 - s0 <= leaf and r1 - r0 <= leaf   # dense: both nodes are leaves
        if s0 == r0 and s1 == r1:
            assert not adm   # a diagonal block is always dense (it holds K_Self)
        if cover is not None:
            cover[r0:r1, s0:s1] += 1
    if cover is not None:
        assert (cover == 1).all()   # every (receiver, source) entry in exactly one block
    return perm, spans


def test_rectangle_network_structure_matches_the_host_rules(qdfn_mod):
    from qdfn import synth
    rec = synth.fault_network(seed=3, n_faults=12, patch=200.0, length=(2000.0, 4000.0))["records"]
    c = rec[:, :3] * np.array([1.0, 1.0, -1.0])
    for leaf, eta in ((32, 2.0), (16, 1.0), (64, 3.0)):
        _, spans = _check(c, leaf, eta)
        assert any(sp[4] for sp in spans)   # there are low-rank blocks


def test_triangle_mesh_structure_matches_the_host_rules(qdfn_mod):
    from qdfn import geometry, synth
    net = synth.curved_fault_network(seed=1, n_faults=3, length=3000.0, width=2000.0, edge=160.0)
    seg = net["seg"]
    P1, P2, P3, *_ = geometry.rot_verts_unit_vectors_abi(seg, seg[:, 9])
    _check((P1 + P2 + P3) / 3, 64, 2.0)


def test_degenerate_inputs(qdfn_mod):
    from qdfn import _lib, hmatrix
    _check(np.array([[1.0, 2.0, -3.0]]), 64, 2.0)                          # one element: one dense block
    _check(np.tile([[5.0, 5.0, -5.0]], (100, 1)), 8, 2.0)                  # identical centres: never admissible
    _check(np.column_stack([np.arange(64.0), np.zeros(64), np.zeros(64)]), 64, 2.0)   # N = leaf, one axis
    with pytest.raises(_lib.QdfnError):
        hmatrix.device_partition(np.array([[0.0, 0.0, np.nan]]), 64, 2.0)
    with pytest.raises(_lib.QdfnError):
        hmatrix.device_partition(np.zeros((4, 3)), 0, 2.0)


def test_operator_on_the_device_structure(qdfn_mod):
    """build_rect on the device structure: the compressed operator matches the
    dense one (permuted) to the ACA tolerance."""
    from qdfn import assemble, hmatrix, synth
    rec = synth.fault_network(seed=5, n_faults=6, patch=250.0)["records"]
    H, perm = hmatrix.build_rect(rec, G, NU, leaf=32, eta=2.0, tol=1e-8, tree="device")
    Ks, Kn = assemble.assemble_rect(rec, rec, G, NU)
    Hs, Hn = H.to_dense(rec.shape[0])
    for A, B in ((Hs, Ks[np.ix_(perm, perm)]), (Hn, Kn[np.ix_(perm, perm)])):
        assert np.linalg.norm(A - B) <= 1e-6 * np.linalg.norm(B)
    assert sum(U is not None for U in H.U_s) > 0
