"""H-matrix elastic operator: cluster tree, block structure, compression.

The reference builds its tree by recursive k-means bisection
(scripts/Functions_Hmatrix.jl:1-158, `GroupAndSort_AllLevel`), declares a block
admissible when centre distance / max diameter > 1 (:163-212, `BuildHierarchy`)
and compresses admissible blocks with `LowRankApprox.pqrfact` of the full
dense block (scripts/Functions_BuildInputFile.jl:705-712, 784-791).  Its
k-means is randomly initialised, so its trees are not reproducible; here the
tree is a deterministic principal-axis median bisection down to `leaf`
patches, admissibility is the standard bounding-box rule
max(diam) <= eta * dist, and admissible blocks are compressed by adaptive
cross approximation with partial pivoting (ACA) followed by QR/SVD
recompression, to a relative Frobenius tolerance.  Blocks are formed on the GPU
by the assembly kernels; the block list is handed to qdfn_set_hmatrix in the
reference's ElementRange_SR form (source range, receiver range).
"""
import ctypes as C

import numpy as np

from . import _lib


MAX_RANK = 128   # the device's rank limit of a low-rank block (larger: stored dense)


class ClusterTree:
    """Binary tree over patch centres; `perm` orders patches so every node is a
    contiguous index range [start, end)."""

    def __init__(self, points, leaf=64):
        pts = np.asarray(points, dtype=np.float64)
        n = pts.shape[0]
        self.leaf = leaf
        self.starts, self.ends, self.children, self.lo, self.hi = [], [], [], [], []
        perm = np.arange(n)

        def build(idx, start):
            node = len(self.starts)
            self.starts.append(start)
            self.ends.append(start + len(idx))
            self.children.append(())
            p = pts[idx]
            self.lo.append(p.min(axis=0))
            self.hi.append(p.max(axis=0))
            if len(idx) <= leaf:
                perm[start:start + len(idx)] = idx
                return node
            c = p - p.mean(axis=0)
            # principal axis of the centres (deterministic sign)
            w, v = np.linalg.eigh(c.T @ c)
            ax = v[:, -1]
            ax = ax if ax[np.argmax(np.abs(ax))] > 0 else -ax
            proj = c @ ax
            order = np.argsort(proj, kind="stable")
            half = len(idx) // 2
            a = build(idx[order[:half]], start)
            b = build(idx[order[half:]], start + half)
            self.children[node] = (a, b)
            return node

        build(np.arange(n), 0)
        self.perm = perm
        self.lo = np.array(self.lo)
        self.hi = np.array(self.hi)

    def diam(self, k):
        return float(np.linalg.norm(self.hi[k] - self.lo[k]))

    def dist(self, a, b):
        gap = np.maximum(0.0, np.maximum(self.lo[a] - self.hi[b], self.lo[b] - self.hi[a]))
        return float(np.linalg.norm(gap))


def block_partition(tree, eta=2.0):
    """(src_node, recv_node, admissible) leaves of the block tree."""
    out = []

    def rec(t, s):
        d = tree.dist(t, s)
        if d > 0 and max(tree.diam(t), tree.diam(s)) <= eta * d:   # touching boxes: never admissible
            out.append((s, t, True))
            return
        ct, cs = tree.children[t], tree.children[s]
        if not ct and not cs:
            out.append((s, t, False))
            return
        for a in (ct or (t,)):
            for b in (cs or (s,)):
                rec(a, b)

    rec(0, 0)
    return out


def device_partition(centres, leaf=64, eta=2.0):
    """The cluster tree and block partition built on the GPU
    (qdfn_hstruct_build: k-d tree of median splits along each node's longest
    box axis, admissibility dist > 0 and max(diam) <= eta * dist).  Returns (perm, spans)
    with spans a list of (s0, s1, r0, r1, admissible), half-open ranges of
    positions in the order perm."""
    L = _lib.load()
    c = np.ascontiguousarray(np.asarray(centres, dtype=np.float64).reshape(-1, 3))
    N = c.shape[0]
    h = C.c_void_p()
    _lib.check(L.qdfn_hstruct_build(C.byref(h), N, C.c_void_p(c.ctypes.data), int(leaf), float(eta)))
    try:
        nb = C.c_int64()
        _lib.check(L.qdfn_hstruct_sizes(h, C.byref(nb), None))
        perm = np.zeros(N, dtype=np.int64)
        ranges = np.zeros((nb.value, 4), dtype=np.int64)
        adm = np.zeros(nb.value, dtype=np.int32)
        _lib.check(L.qdfn_hstruct_get(h, C.c_void_p(perm.ctypes.data), C.c_void_p(ranges.ctypes.data),
                                      C.c_void_p(adm.ctypes.data)))
    finally:
        L.qdfn_hstruct_destroy(h)
    spans = [(int(a), int(b) + 1, int(c_), int(d) + 1, bool(m)) for (a, b, c_, d), m in zip(ranges, adm)]
    return perm, spans


def host_partition(centres, leaf=64, eta=2.0):
    """The same (perm, spans) from the host principal-axis tree (ClusterTree)
    and block_partition."""
    tree = ClusterTree(np.asarray(centres), leaf=leaf)
    spans = [(tree.starts[s], tree.ends[s], tree.starts[t], tree.ends[t], adm)
             for (s, t, adm) in block_partition(tree, eta)]
    return tree.perm, spans


def partition(centres, leaf, eta, tree):
    if tree == "device":
        return device_partition(centres, leaf, eta)
    if tree == "pca":
        return host_partition(centres, leaf, eta)
    raise ValueError("tree must be 'device' or 'pca'")


def aca(block, tol, max_rank=None):
    """ACA with partial pivoting on a dense torch block (m x n), then QR/SVD
    recompression; returns (U (m x k), Vt (k x n)) with
    ||block - U Vt||_F <= tol ||block||_F (estimated the ACA way)."""
    m, n = block.shape
    return aca_fn(lambda i: block[i].clone(), lambda j: block[:, j].clone(), m, n, tol, max_rank,
                  device=block.device, dtype=block.dtype)


def aca_fn(row_fn, col_fn, m, n, tol, max_rank=None, device=None, dtype=None):
    """ACA with partial pivoting (Bebendorf's rule) on a block known only through
    row_fn(i) -> row i (length n) and col_fn(j) -> column j (length m), torch
    tensors; then QR/SVD recompression.  Entries are formed on demand -- a rank-k
    block costs about k (m + n) evaluations instead of m n."""
    import torch
    max_rank = max_rank or min(m, n)
    Us, Vs = [], []
    used_rows = torch.zeros(m, dtype=torch.bool, device=device)
    i = 0
    frob2 = 0.0
    for _ in range(max_rank):
        row = row_fn(i)
        for u, v in zip(Us, Vs):
            row -= u[i] * v
        used_rows[i] = True
        j = int(torch.argmax(torch.abs(row)))
        piv = row[j]
        if abs(float(piv)) == 0.0:
            cand = torch.nonzero(~used_rows).flatten()
            if len(cand) == 0:
                break
            i = int(cand[0])
            continue
        v = row / piv
        col = col_fn(j)
        for u, vv in zip(Us, Vs):
            col -= vv[j] * u
        u = col
        nu2 = float(u @ u) * float(v @ v)
        cross = 0.0
        for uu, vv in zip(Us, Vs):
            cross += float(uu @ u) * float(vv @ v)
        frob2 += nu2 + 2 * cross
        Us.append(u)
        Vs.append(v)
        if nu2 <= (tol ** 2) * max(frob2, 1e-300):
            break
        cand = torch.abs(u).masked_fill(used_rows, -1.0)
        i = int(torch.argmax(cand))
        if cand[i] < 0:
            break
    if not Us:
        return (torch.zeros((m, 0), dtype=dtype, device=device),
                torch.zeros((0, n), dtype=dtype, device=device))
    U = torch.stack(Us, dim=1)
    V = torch.stack(Vs, dim=0)
    # recompression: U = Qu Ru, V^T = Qv Rv -> SVD of Ru Rv^T
    Qu, Ru = torch.linalg.qr(U)
    Qv, Rv = torch.linalg.qr(V.T)
    W, S, Zt = torch.linalg.svd(Ru @ Rv.T)
    tot = float(torch.sum(S ** 2))
    tail = torch.flip(torch.cumsum(torch.flip(S ** 2, [0]), 0), [0])
    keep = int(torch.sum(tail > (tol ** 2) * tot))
    keep = max(keep, 1)
    U2 = Qu @ (W[:, :keep] * S[:keep])
    Vt2 = (Zt[:keep] @ Qv.T)
    return U2, Vt2


class HMatrix:
    """Blocks of one operator pair (shear, normal) over a ClusterTree ordering."""

    def __init__(self, ranges, dense_s, U_s, Vt_s, dense_n, U_n, Vt_n, perm):
        self.ranges = ranges          # nb x 4: src_begin, src_end, recv_begin, recv_end (0-based, inclusive)
        self.dense_s, self.U_s, self.Vt_s = dense_s, U_s, Vt_s
        self.dense_n, self.U_n, self.Vt_n = dense_n, U_n, Vt_n
        self.perm = perm

    @property
    def nblocks(self):
        return self.ranges.shape[0]

    def stored_entries(self):
        tot = 0
        for b in range(self.nblocks):
            for D, U, Vt in ((self.dense_s[b], self.U_s[b], self.Vt_s[b]), (self.dense_n[b], self.U_n[b],
                                                                             self.Vt_n[b])):
                tot += D.size if D is not None else U.size + Vt.size
        return tot

    def to_dense(self, N):
        Ks, Kn = np.zeros((N, N)), np.zeros((N, N))
        for b, (s0, s1, r0, r1) in enumerate(self.ranges):
            for K, D, U, Vt in ((Ks, self.dense_s[b], self.U_s[b], self.Vt_s[b]),
                                (Kn, self.dense_n[b], self.U_n[b], self.Vt_n[b])):
                K[r0:r1 + 1, s0:s1 + 1] = D if D is not None else U @ Vt
        return Ks, Kn


def build_rect(records, shear_modulus, poisson, leaf=64, eta=2.0, tol=1e-6, device="cuda", tree="pca"):
    """Build the H-matrix of a rectangular-patch system (records n x 8).
    tree: "pca" (host principal-axis bisection) or "device" (qdfn_hstruct_build).
    Returns (HMatrix, perm): block ranges index the permuted ordering
    records[perm]."""
    import torch
    from . import assemble
    perm, spans = partition(np.asarray(records)[:, :3] * np.array([1.0, 1.0, -1.0]), leaf, eta, tree)
    rec = torch.tensor(np.ascontiguousarray(np.asarray(records)[perm]), dtype=torch.float64, device=device)
    ranges, ds, us, vs, dn, un, vn = [], [], [], [], [], [], []
    for (s0, s1, r0, r1, adm) in spans:
        ns, nr = s1 - s0, r1 - r0
        Ks = torch.empty((ns, nr), dtype=torch.float64, device=device)
        Kn = torch.empty((ns, nr), dtype=torch.float64, device=device)
        assemble.assemble_rect_dev(rec[s0:s1], rec[r0:r1], shear_modulus, poisson, Ks, Kn, layout="col")
        Bs, Bn = Ks.T, Kn.T      # recv x src
        ranges.append((s0, s1 - 1, r0, r1 - 1))
        if adm:
            for B, Ul, Vl, Dl in ((Bs, us, vs, ds), (Bn, un, vn, dn)):
                U, Vt = aca(B.contiguous(), tol)
                if U.shape[1] * (nr + ns) < nr * ns:
                    Ul.append(U.cpu().numpy()); Vl.append(Vt.cpu().numpy()); Dl.append(None)
                else:
                    Ul.append(None); Vl.append(None); Dl.append(B.cpu().numpy())
        else:
            for B, Ul, Vl, Dl in ((Bs, us, vs, ds), (Bn, un, vn, dn)):
                Ul.append(None); Vl.append(None); Dl.append(B.contiguous().cpu().numpy())
    return HMatrix(np.array(ranges, dtype=np.int64), ds, us, vs, dn, un, vn, perm), perm


def build_tri(P1, P2, P3, rake, centre, nhat, shat, shear_modulus, poisson, leaf=64, eta=2.0, tol=1e-6,
              device="cuda", chunk=1 << 24, tree="pca"):
    """Build the H-matrix of a triangular-patch system (TDstressHS kernels,
    StiffnessMatrix_ByParts_Calculation_Tri, scripts/Functions_BuildInputFile.jl:551-594,
    in the block structure HmatBuild_T builds at :643-723).  Entries are
    formed on the GPU from index lists (qdfn_assemble_tri_pairs_dev): the
    near-field blocks whole, in batches of `chunk` entries, and the admissible
    blocks only where batched ACA asks for them (one row and one column per
    block and iteration, every block in the same launches) -- no admissible
    block is ever formed whole.  tree: "pca" (host principal-axis bisection)
    or "device" (qdfn_hstruct_build).  Returns (HMatrix, perm): block ranges
    index the permuted ordering (every per-patch array [perm])."""
    import torch
    from . import assemble
    perm, pspans = partition(np.asarray(centre), leaf, eta, tree)
    dv = lambda a: torch.tensor(np.ascontiguousarray(np.asarray(a)[perm]), dtype=torch.float64,
                                device=device)
    p1, p2, p3, rk, cen, nh, sh = (dv(a) for a in (P1, P2, P3, rake, centre, nhat, shat))

    def evaluate(ridx, sidx):
        outs, outn = [], []
        for k in range(0, int(ridx.shape[0]), chunk):
            a, b = assemble.assemble_tri_pairs_dev(ridx[k:k + chunk].contiguous(), sidx[k:k + chunk].contiguous(),
                                                   p1, p2, p3, rk, cen, nh, sh, shear_modulus, poisson)
            outs.append(a)
            outn.append(b)
        if not outs:
            z = torch.zeros(0, dtype=torch.float64, device=device)
            return z, z
        return torch.cat(outs), torch.cat(outn)

    def dense_blocks(bl):
        """(recv x src) host arrays of both matrices for blocks (s0, s1, r0, r1)."""
        res = []
        for k0 in range(0, len(bl), 256):
            part = bl[k0:k0 + 256]
            rr, ss = [], []
            for (s0, s1, r0, r1) in part:
                r = torch.arange(r0, r1, device=device)
                c = torch.arange(s0, s1, device=device)
                rr.append(r.repeat_interleave(s1 - s0))
                ss.append(c.repeat(r1 - r0))
            Ks, Kn = evaluate(torch.cat(rr), torch.cat(ss))
            Ks, Kn = Ks.cpu().numpy(), Kn.cpu().numpy()
            off = 0
            for (s0, s1, r0, r1) in part:
                n = (s1 - s0) * (r1 - r0)
                res.append((Ks[off:off + n].reshape(r1 - r0, s1 - s0), Kn[off:off + n].reshape(r1 - r0, s1 - s0)))
                off += n
        return res

    spans = [sp[:4] for sp in pspans]
    near = [k for k, sp in enumerate(pspans) if not sp[4]]
    far = [k for k, sp in enumerate(pspans) if sp[4]]
    nb = len(pspans)
    ds, us, vs, dn, un, vn = ([None] * nb for _ in range(6))
    for k, (Bs, Bn) in zip(near, dense_blocks([spans[k] for k in near])):
        ds[k], dn[k] = Bs, Bn
    if far:
        nr = [spans[k][3] - spans[k][2] for k in far]
        ns = [spans[k][1] - spans[k][0] for k in far]
        (fs, fn), ro, co = aca_batched(nr, ns, [spans[k][2] for k in far], [spans[k][0] for k in far], evaluate,
                                       tol)
        redo = []
        for j, k in enumerate(far):
            for (U, V, rank), Ul, Vl, side in ((fs, us, vs, 0), (fn, un, vn, 1)):
                rk_b = int(rank[j])
                if rk_b < MAX_RANK and rk_b * (nr[j] + ns[j]) < nr[j] * ns[j]:
                    Ul[k] = np.ascontiguousarray(U[ro[j]:ro[j] + nr[j], :rk_b])
                    Vl[k] = np.ascontiguousarray(V[:rk_b, co[j]:co[j] + ns[j]])
                else:
                    redo.append((k, side))
        if redo:   # not worth compressing (or not converged at the rank limit): stored dense
            for (k, side), (Bs, Bn) in zip(redo, dense_blocks([spans[k] for k, _ in redo])):
                if side == 0:
                    ds[k] = Bs
                else:
                    dn[k] = Bn
    ranges = np.array([(s0, s1 - 1, r0, r1 - 1) for (s0, s1, r0, r1) in spans], dtype=np.int64)
    return HMatrix(ranges, ds, us, vs, dn, un, vn, perm), perm


def _seg_argmax(vals, seg, nseg):
    """Per segment: the largest value and the first flat index holding it
    (vals float64 CUDA tensor, seg its segment ids)."""
    import torch
    m = torch.full((nseg,), -float("inf"), dtype=vals.dtype, device=vals.device)
    m = m.scatter_reduce(0, seg, vals, reduce="amax", include_self=True)
    n = vals.shape[0]
    idx = torch.arange(n, device=vals.device)
    cand = torch.where(vals == m[seg], idx, torch.full_like(idx, n))
    first = torch.full((nseg,), n, dtype=idx.dtype, device=vals.device)
    first = first.scatter_reduce(0, seg, cand, reduce="amin", include_self=True)
    return m, first


def _seg_sum(vals, seg, nseg):
    import torch
    return torch.zeros(nseg, dtype=vals.dtype, device=vals.device).index_add_(0, seg, vals)


def aca_batched(nr, ns, r0, s0, evaluate, tol, max_rank=MAX_RANK):
    """ACA with partial pivoting on many blocks at once, both matrices of the
    pair (shear, normal) with their own pivots: every iteration asks
    `evaluate(recv, src) -> (Ks, Kn)` (CUDA index tensors, global indices) for
    one row of each active block and side, then one column -- two gathered
    kernel launches per iteration for all blocks together.  Returns, per
    side, the host arrays U (sum nr x rank_max), V (rank_max x sum ns) and the
    per-block ranks; block b's factors are U[ro_b:ro_b+nr_b, :rank_b] and
    V[:rank_b, co_b:co_b+ns_b] (ro, co the exclusive prefix sums of nr, ns)."""
    import torch
    dev = "cuda"
    B = len(nr)
    nr_t = torch.tensor(nr, dtype=torch.int64, device=dev)
    ns_t = torch.tensor(ns, dtype=torch.int64, device=dev)
    r0_t = torch.tensor(r0, dtype=torch.int64, device=dev)
    s0_t = torch.tensor(s0, dtype=torch.int64, device=dev)
    ro = torch.cumsum(nr_t, 0) - nr_t
    co = torch.cumsum(ns_t, 0) - ns_t
    Tr, Tc = int(nr_t.sum()), int(ns_t.sum())
    rblk = torch.repeat_interleave(torch.arange(B, device=dev), nr_t)
    cblk = torch.repeat_interleave(torch.arange(B, device=dev), ns_t)
    rloc = torch.arange(Tr, device=dev) - ro[rblk]
    cloc = torch.arange(Tc, device=dev) - co[cblk]
    out = []
    sides = [dict(active=torch.ones(B, dtype=torch.bool, device=dev), piv=torch.zeros(B, dtype=torch.int64, device=dev),
                  used=torch.zeros(Tr, dtype=torch.bool, device=dev), frob2=torch.zeros(B, dtype=torch.float64,
                                                                                        device=dev),
                  rank=torch.zeros(B, dtype=torch.int64, device=dev), U=[], V=[]) for _ in range(2)]
    for it in range(max_rank):
        if not any(bool(sd["active"].any()) for sd in sides):
            break
        # rows: the pivot row of every active block, for both sides in one launch
        rr, ss, parts = [], [], []
        for sd in sides:
            m = sd["active"][cblk]
            ic = torch.nonzero(m).flatten()
            b = cblk[ic]
            rr.append(r0_t[b] + sd["piv"][b])
            ss.append(s0_t[b] + cloc[ic])
            parts.append(ic)
        Ks, Kn = evaluate(torch.cat(rr), torch.cat(ss))
        off = 0
        cols = []
        for side, sd in enumerate(sides):
            ic = parts[side]
            vals = (Ks if side == 0 else Kn)[off:off + ic.shape[0]]
            off += ic.shape[0]
            R = torch.zeros(Tc, dtype=torch.float64, device=dev)
            R[ic] = vals
            for Ul, Vl in zip(sd["U"], sd["V"]):
                R -= Ul[ro + sd["piv"]][cblk] * Vl
            act_c = sd["active"][cblk]
            absR = torch.where(act_c, R.abs(), torch.full_like(R, -1.0))
            mx, jf = _seg_argmax(absR, cblk, B)
            jf = torch.clamp(jf, max=Tc - 1)
            piv = R[jf]
            ok = sd["active"] & (mx > 0)
            sd["active"] = ok
            sd["jf"] = jf
            sd["v"] = torch.where(ok[cblk], R / torch.where(ok, piv, torch.ones_like(piv))[cblk], torch.zeros_like(R))
            m = ok[rblk]
            ir = torch.nonzero(m).flatten()
            b = rblk[ir]
            cols.append((ir, r0_t[b] + rloc[ir], s0_t[b] + (jf[b] - co[b])))
        Ks, Kn = evaluate(torch.cat([c[1] for c in cols]), torch.cat([c[2] for c in cols]))
        off = 0
        for side, sd in enumerate(sides):
            ir = cols[side][0]
            vals = (Ks if side == 0 else Kn)[off:off + ir.shape[0]]
            off += ir.shape[0]
            u = torch.zeros(Tr, dtype=torch.float64, device=dev)
            u[ir] = vals
            jf = sd["jf"]
            for Ul, Vl in zip(sd["U"], sd["V"]):
                u -= Vl[jf][rblk] * Ul
            act_r = sd["active"][rblk]
            u = torch.where(act_r, u, torch.zeros_like(u))
            v = sd["v"]
            nu2 = _seg_sum(u * u, rblk, B) * _seg_sum(v * v, cblk, B)
            cross = torch.zeros(B, dtype=torch.float64, device=dev)
            for Ul, Vl in zip(sd["U"], sd["V"]):
                cross += _seg_sum(u * Ul, rblk, B) * _seg_sum(v * Vl, cblk, B)
            sd["frob2"] = sd["frob2"] + torch.where(sd["active"], nu2 + 2 * cross, torch.zeros_like(nu2))
            sd["U"].append(u)
            sd["V"].append(v)
            sd["rank"] += sd["active"].to(torch.int64)
            conv = nu2 <= (tol ** 2) * torch.clamp(sd["frob2"], min=1e-300)
            # next pivot row: the largest |u| among the rows not used yet
            sd["used"] = sd["used"] | torch.zeros_like(sd["used"]).index_fill_(0, ro + sd["piv"], True) & \
                sd["active"][rblk]
            cand = torch.where(sd["used"] | ~act_r, torch.full_like(u, -1.0), u.abs())
            mx, nxt = _seg_argmax(cand, rblk, B)
            sd["piv"] = torch.where(mx >= 0, torch.clamp(nxt, max=Tr - 1) - ro, sd["piv"])
            sd["active"] = sd["active"] & ~conv & (mx >= 0)
    for sd in sides:
        k = len(sd["U"])
        U = torch.stack(sd["U"], 1).cpu().numpy() if k else np.zeros((Tr, 0))
        V = torch.stack(sd["V"], 0).cpu().numpy() if k else np.zeros((0, Tc))
        out.append((U, V, sd["rank"].cpu().numpy()))
    return out, ro.cpu().numpy(), co.cpu().numpy()


def set_hmatrix(sim, H, precision="fp64"):
    """Hand an HMatrix to a Simulation (qdfn_set_hmatrix)."""
    L = _lib.load()
    nb = H.nblocks
    prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    keep = []

    def arr(a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        return a.ctypes.data_as(C.POINTER(C.c_double))

    def plist(lst):
        p = (C.POINTER(C.c_double) * nb)()
        for b, a in enumerate(lst):
            p[b] = arr(a) if a is not None else C.POINTER(C.c_double)()
        return p

    rng = np.ascontiguousarray(H.ranges, dtype=np.int64)
    rank_s = np.array([-1 if H.dense_s[b] is not None else H.U_s[b].shape[1] for b in range(nb)], dtype=np.int64)
    rank_n = np.array([-1 if H.dense_n[b] is not None else H.U_n[b].shape[1] for b in range(nb)], dtype=np.int64)
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))
    _lib.check(L.qdfn_set_hmatrix(sim._h, nb, ip(rng), ip(rank_s), plist(H.U_s), plist(H.Vt_s), plist(H.dense_s),
                                  ip(rank_n), plist(H.U_n), plist(H.Vt_n), plist(H.dense_n), prec))
    sim._keep["hmat"] = (keep, rng, rank_s, rank_n)


def set_hmatrix_from_reference(sim, ElementRange_SR, ShearStiffness_H, NormalStiffness_H, zero_normal=False,
                               precision="fp64"):
    """Blocks in the reference's form: ElementRange_SR (B x 4, 1-based,
    inclusive: source range, receiver range) and per block either a dense
    (recv x src) matrix or a (U, Vt) pair (e.g. a PartialQR converted to
    U = Q, Vt = R P^T)."""
    rng = np.asarray(ElementRange_SR, dtype=np.int64) - 1
    nb = rng.shape[0]
    ds, us, vs, dn, un, vn = [], [], [], [], [], []
    for b in range(nb):
        for blk, Dl, Ul, Vl in ((ShearStiffness_H[b], ds, us, vs), (NormalStiffness_H[b], dn, un, vn)):
            if zero_normal and Dl is dn:
                nr, ns = rng[b, 3] - rng[b, 2] + 1, rng[b, 1] - rng[b, 0] + 1
                Dl.append(np.zeros((nr, ns))); Ul.append(None); Vl.append(None)
            elif isinstance(blk, (tuple, list)):
                Ul.append(np.asarray(blk[0])); Vl.append(np.asarray(blk[1])); Dl.append(None)
            else:
                Dl.append(np.asarray(blk)); Ul.append(None); Vl.append(None)
    H = HMatrix(rng, ds, us, vs, dn, un, vn, None)
    set_hmatrix(sim, H, precision)
    return H
