// H-matrix structure built on the device: the cluster tree over the element
// centres and the block partition, standing in for the reference's k-means
// tree and block hierarchy (GroupAndSort_AllLevel and BuildHierarchy,
// scripts/Functions_Hmatrix.jl:1-212), whose random initialisation makes its
// trees irreproducible.
//
//  1. Tree: level by level, every node of more than `leaf` elements orders
//     its elements by their centre's coordinate along the longest axis of the
//     node's box (ties: the lower axis; equal coordinates: the lower element
//     index) and splits its range in two halves (the first floor(n / 2)): a
//     k-d tree of median splits.  All nodes of a level are ordered by ONE
//     bitonic sort of (node start, coordinate key, element) over the whole
//     order (one launch per merge stage); elements of nodes that do not split
//     keep their places (their key is their position).
//  2. Boxes: the exact min/max of each node's centres, one warp per node.
//  3. Partition: a frontier of (receiver node, source node) pairs, one thread
//     each per launch: admissible when dist > 0 and max(diam) <= eta * dist
//     (box diagonal, box-to-box distance) -> low-rank block; both leaves -> dense block;
//     otherwise the pair's children pairs go to the next frontier (a leaf
//     stands in for its own children).  The blocks are then ordered by
//     (receiver start, source start) so the result does not depend on the
//     order in which threads appended them.
//
// Every floating-point step is a single IEEE operation compiled without
// contraction, so a host restatement of the same rules reproduces the
// permutation and the partition exactly (tests/test_hstruct.py).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "qdfn_internal.h"

struct qdfn_hstruct {
    int64_t N = 0;
    std::vector<int64_t> perm;                 // [N] element at each position of the order
    std::vector<int64_t> ranges;               // [nb][4] s0, s1, r0, r1 (inclusive)
    std::vector<int32_t> adm;                  // [nb] 1 low-rank, 0 dense
    std::vector<int64_t> nstart, nend;         // tree nodes (level order)
};

namespace qdfn {
namespace {

__device__ __forceinline__ unsigned long long ord_key_d(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return b ^ ((unsigned long long)((long long)b >> 63) | 0x8000000000000000ull);
}

// boxes of the nodes of one level: one warp per node, exact min/max of its
// centres; the split axis (longest extent, the lower axis on ties) is written
// at the node's start position for splitting nodes, -1 for the others
__global__ void k_level_boxes(int n, const int* __restrict__ nodes, const long long* __restrict__ nstart,
                              const long long* __restrict__ nend, const long long* __restrict__ order,
                              const double* __restrict__ c, int leaf, double* lo, double* hi, int* axis_at) {
    const int w = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (w >= n) return;
    const int node = nodes[w];
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (long long p = nstart[node] + lane; p < nend[node]; p += 32) {
        const long long e = order[p];
        for (int a = 0; a < 3; ++a) {
            mn[a] = fmin(mn[a], c[e * 3 + a]);
            mx[a] = fmax(mx[a], c[e * 3 + a]);
        }
    }
    for (int a = 0; a < 3; ++a)
        for (int o = 16; o > 0; o >>= 1) {
            mn[a] = fmin(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = fmax(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
    if (lane == 0) {
        for (int a = 0; a < 3; ++a) {
            lo[node * 3 + a] = mn[a];
            hi[node * 3 + a] = mx[a];
        }
        int ax = 0;
        if (mx[1] - mn[1] > mx[ax] - mn[ax]) ax = 1;
        if (mx[2] - mn[2] > mx[ax] - mn[ax]) ax = 2;
        axis_at[nstart[node]] = (nend[node] - nstart[node] > leaf) ? ax : -1;
    }
}

// sort keys of one level: (start of the position's node, coordinate key or
// the position itself, element)
__global__ void k_level_keys(int64_t N, int64_t npad, const long long* __restrict__ seg,
                             const int* __restrict__ axis_at, const long long* __restrict__ order,
                             const double* __restrict__ c, long long* k1, unsigned long long* k2, long long* idx) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npad) return;
    if (p >= N) {   // padding sorts last
        k1[p] = 0x7fffffffffffffffll;
        k2[p] = ~0ull;
        idx[p] = 0x7fffffffffffffffll;
        return;
    }
    const long long s = seg[p], e = order[p];
    const int ax = axis_at[s];
    k1[p] = s;
    k2[p] = ax >= 0 ? ord_key_d(c[e * 3 + ax] + 0.0) : (unsigned long long)p;   // (+0.0: -0 and 0 compare equal)
    idx[p] = e;
}

// one compare-exchange stage of the bitonic network over (k1, k2, idx)
__global__ void k_bitonic3(int64_t npad, long long* k1, unsigned long long* k2, long long* idx, int64_t j,
                           int64_t k) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    const int64_t l = i ^ j;
    if (l <= i) return;
    const bool up = (i & k) == 0;
    const long long a1 = k1[i], b1 = k1[l];
    const unsigned long long a2 = k2[i], b2 = k2[l];
    const long long a3 = idx[i], b3 = idx[l];
    const bool greater = a1 != b1 ? a1 > b1 : (a2 != b2 ? a2 > b2 : a3 > b3);
    if (greater == up) {
        k1[i] = b1; k1[l] = a1;
        k2[i] = b2; k2[l] = a2;
        idx[i] = b3; idx[l] = a3;
    }
}

// the children's segments of the splitting nodes of a level: one warp per node
__global__ void k_level_split(int n, const int* __restrict__ nodes, const long long* __restrict__ nstart,
                              const long long* __restrict__ nend, int leaf, long long* seg) {
    const int w = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (w >= n) return;
    const int node = nodes[w];
    const long long s = nstart[node], e = nend[node];
    if (e - s <= leaf) return;
    const long long h = s + (e - s) / 2;
    for (long long p = s + lane; p < e; p += 32) seg[p] = p < h ? s : h;
}

__device__ __forceinline__ double norm3(double x, double y, double z) { return sqrt((x * x + y * y) + z * z); }

// one frontier round of the partition: pair (t receiver node, s source node)
__global__ void k_partition(int n, const int2* __restrict__ fin, const double* __restrict__ lo,
                            const double* __restrict__ hi, const int2* __restrict__ child, double eta, int2* fout,
                            unsigned* nout, unsigned cap_out, int4* blocks, unsigned* nblk, unsigned cap_blk) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int t = fin[k].x, s = fin[k].y;
    const double dt = norm3(hi[t * 3] - lo[t * 3], hi[t * 3 + 1] - lo[t * 3 + 1], hi[t * 3 + 2] - lo[t * 3 + 2]);
    const double ds = norm3(hi[s * 3] - lo[s * 3], hi[s * 3 + 1] - lo[s * 3 + 1], hi[s * 3 + 2] - lo[s * 3 + 2]);
    double g[3];
    for (int a = 0; a < 3; ++a) g[a] = fmax(0.0, fmax(lo[t * 3 + a] - hi[s * 3 + a], lo[s * 3 + a] - hi[t * 3 + a]));
    const double dist = norm3(g[0], g[1], g[2]);
    const int2 ct = child[t], cs = child[s];
    const bool lt = ct.x < 0, ls = cs.x < 0;
    const bool adm = dist > 0.0 && fmax(dt, ds) <= eta * dist;   // boxes that touch are never admissible
    if (adm || (lt && ls)) {
        const unsigned b = atomicAdd(nblk, 1u);
        if (b < cap_blk) blocks[b] = make_int4(s, t, adm ? 1 : 0, 0);
        return;
    }
    const int ta[2] = {lt ? t : ct.x, lt ? t : ct.y}, sa[2] = {ls ? s : cs.x, ls ? s : cs.y};
    const int nt = lt ? 1 : 2, ns = ls ? 1 : 2;
    const unsigned o = atomicAdd(nout, (unsigned)(nt * ns));
    for (int a = 0; a < nt; ++a)
        for (int b = 0; b < ns; ++b) {
            const unsigned p = o + (unsigned)(a * ns + b);
            if (p < cap_out) fout[p] = make_int2(ta[a], sa[b]);
        }
}

template <class T>
struct DBuf {
    T* p = nullptr;
    ~DBuf() { if (p) cudaFree(p); }
    int alloc(size_t n) {
        if (p) cudaFree(p);
        p = nullptr;
        return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) == cudaSuccess ? QDFN_OK
                                                                                    : fail(QDFN_ERR_NOMEM, "cudaMalloc failed");
    }
};

}  // namespace
}  // namespace qdfn

using namespace qdfn;

extern "C" int qdfn_hstruct_build(qdfn_hstruct** out, int64_t N, const double* centres, int leaf, double eta) {
    if (!out || !centres) return fail(QDFN_ERR_INVALID, "null argument");
    *out = nullptr;
    if (N < 1 || N > (int64_t)1 << 30) return fail(QDFN_ERR_INVALID, "N must be in 1..2^30");
    if (leaf < 1) return fail(QDFN_ERR_INVALID, "leaf must be >= 1");
    if (!(eta > 0) || !std::isfinite(eta)) return fail(QDFN_ERR_INVALID, "eta must be positive");
    if (N / leaf > ((int64_t)1 << 27)) return fail(QDFN_ERR_INVALID, "too many tree nodes (raise leaf)");
    for (int64_t i = 0; i < 3 * N; ++i)
        if (!std::isfinite(centres[i])) return fail(QDFN_ERR_INVALID, "centres must be finite");
    // the tree's shape depends on N and leaf only: level order, halving
    std::vector<long long> nstart{0}, nend{N};
    std::vector<int2> child;
    std::vector<int> level{0};
    for (size_t v = 0; v < nstart.size(); ++v) {
        const long long n = nend[v] - nstart[v];
        if (n > leaf) {
            const long long half = n / 2;
            const int a = (int)nstart.size();
            nstart.push_back(nstart[v]); nend.push_back(nstart[v] + half); level.push_back(level[v] + 1);
            nstart.push_back(nstart[v] + half); nend.push_back(nend[v]); level.push_back(level[v] + 1);
            child.push_back(make_int2(a, a + 1));
        } else {
            child.push_back(make_int2(-1, -1));
        }
    }
    if (nstart.size() >= (size_t)1 << 30) return fail(QDFN_ERR_INVALID, "too many tree nodes (raise leaf)");
    const int nn = (int)nstart.size();
    int64_t npad = 1;
    while (npad < N) npad <<= 1;
    int maxlev = 0;
    for (int v = 0; v < nn; ++v) maxlev = std::max(maxlev, level[v]);
    DBuf<double> dc, dlo, dhi;
    DBuf<unsigned long long> dk2;
    DBuf<long long> dk1, didx, dorder, dseg, dns, dne;
    DBuf<int> daxis, dnodes;
    DBuf<int2> dchild;
    int rc;
    if ((rc = dc.alloc(3 * N)) || (rc = dk1.alloc(npad)) || (rc = dk2.alloc(npad)) || (rc = didx.alloc(npad)) ||
        (rc = dorder.alloc(N)) || (rc = dseg.alloc(N)) || (rc = daxis.alloc(N)) || (rc = dnodes.alloc(nn)) ||
        (rc = dlo.alloc(3 * (size_t)nn)) || (rc = dhi.alloc(3 * (size_t)nn)) || (rc = dns.alloc(nn)) ||
        (rc = dne.alloc(nn)) || (rc = dchild.alloc(nn)))
        return rc;
    QDFN_CUDA(cudaMemcpy(dc.p, centres, 3 * N * sizeof(double), cudaMemcpyHostToDevice));
    {
        std::vector<long long> iota(N);
        for (int64_t i = 0; i < N; ++i) iota[i] = i;
        QDFN_CUDA(cudaMemcpy(dorder.p, iota.data(), N * sizeof(long long), cudaMemcpyHostToDevice));
    }
    QDFN_CUDA(cudaMemset(dseg.p, 0, N * sizeof(long long)));
    QDFN_CUDA(cudaMemcpy(dns.p, nstart.data(), nn * sizeof(long long), cudaMemcpyHostToDevice));
    QDFN_CUDA(cudaMemcpy(dne.p, nend.data(), nn * sizeof(long long), cudaMemcpyHostToDevice));
    QDFN_CUDA(cudaMemcpy(dchild.p, child.data(), nn * sizeof(int2), cudaMemcpyHostToDevice));
    // level by level: the boxes, then one sort orders every splitting node
    // along its axis, then the children's segments
    for (int l = 0; l <= maxlev; ++l) {
        std::vector<int> lv;
        bool splits = false;
        for (int v = 0; v < nn; ++v)
            if (level[v] == l) {
                lv.push_back(v);
                splits = splits || child[v].x >= 0;
            }
        QDFN_CUDA(cudaMemcpy(dnodes.p, lv.data(), lv.size() * sizeof(int), cudaMemcpyHostToDevice));
        const unsigned wb = (unsigned)((lv.size() * 32 + 255) / 256);
        k_level_boxes<<<wb, 256>>>((int)lv.size(), dnodes.p, dns.p, dne.p, dorder.p, dc.p, leaf, dlo.p, dhi.p,
                                    daxis.p);
        QDFN_CUDA(cudaGetLastError());
        if (!splits) continue;
        k_level_keys<<<(unsigned)((npad + 255) / 256), 256>>>(N, npad, dseg.p, daxis.p, dorder.p, dc.p, dk1.p,
                                                              dk2.p, didx.p);
        QDFN_CUDA(cudaGetLastError());
        for (int64_t k = 2; k <= npad; k <<= 1)
            for (int64_t j = k >> 1; j > 0; j >>= 1)
                k_bitonic3<<<(unsigned)((npad + 255) / 256), 256>>>(npad, dk1.p, dk2.p, didx.p, j, k);
        QDFN_CUDA(cudaGetLastError());
        QDFN_CUDA(cudaMemcpy(dorder.p, didx.p, N * sizeof(long long), cudaMemcpyDeviceToDevice));
        k_level_split<<<wb, 256>>>((int)lv.size(), dnodes.p, dns.p, dne.p, leaf, dseg.p);
        QDFN_CUDA(cudaGetLastError());
    }
    // partition by frontier rounds; buffers grow and the round is redone when a count overflows
    std::vector<int4> blocks;
    {
        // small first buffers, doubled on demand (a round that overflows is
        // redone): every partition of more than 1024 blocks or frontier pairs
        // goes through the growth path, so the tests exercise it
        unsigned cap_f = 1024u, cap_b = 1024u;
        DBuf<int2> fa, fb;
        DBuf<int4> db;
        DBuf<unsigned> dcnt;   // [0] next frontier, [1] blocks
        if ((rc = fa.alloc(cap_f)) || (rc = fb.alloc(cap_f)) || (rc = db.alloc(cap_b)) || (rc = dcnt.alloc(2))) return rc;
        const int2 root = make_int2(0, 0);
        QDFN_CUDA(cudaMemcpy(fa.p, &root, sizeof(root), cudaMemcpyHostToDevice));
        unsigned n = 1, nblk = 0;
        QDFN_CUDA(cudaMemset(dcnt.p, 0, 2 * sizeof(unsigned)));
        while (n > 0) {
            unsigned cnt[2];
            for (;;) {
                const unsigned start[2] = {0u, nblk};
                QDFN_CUDA(cudaMemcpy(dcnt.p, start, sizeof(start), cudaMemcpyHostToDevice));
                k_partition<<<(n + 255) / 256, 256>>>((int)n, fa.p, dlo.p, dhi.p, dchild.p, eta, fb.p, dcnt.p, cap_f,
                                                      db.p, dcnt.p + 1, cap_b);
                QDFN_CUDA(cudaGetLastError());
                QDFN_CUDA(cudaMemcpy(cnt, dcnt.p, sizeof(cnt), cudaMemcpyDeviceToHost));
                if (cnt[0] <= cap_f && cnt[1] <= cap_b) break;
                if (cnt[1] > cap_b) {   // keep the blocks so far, then a larger buffer
                    std::vector<int4> keep(nblk);
                    if (nblk) QDFN_CUDA(cudaMemcpy(keep.data(), db.p, nblk * sizeof(int4), cudaMemcpyDeviceToHost));
                    cap_b = std::max(cap_b * 2, cnt[1]);
                    if ((rc = db.alloc(cap_b))) return rc;
                    if (nblk) QDFN_CUDA(cudaMemcpy(db.p, keep.data(), nblk * sizeof(int4), cudaMemcpyHostToDevice));
                }
                if (cnt[0] > cap_f) {   // the frontier in fa is intact: grow fb (and fa for later rounds)
                    std::vector<int2> keep(n);
                    QDFN_CUDA(cudaMemcpy(keep.data(), fa.p, n * sizeof(int2), cudaMemcpyDeviceToHost));
                    cap_f = std::max(cap_f * 2, cnt[0]);
                    if ((rc = fa.alloc(cap_f)) || (rc = fb.alloc(cap_f))) return rc;
                    QDFN_CUDA(cudaMemcpy(fa.p, keep.data(), n * sizeof(int2), cudaMemcpyHostToDevice));
                }
            }
            nblk = cnt[1];
            n = cnt[0];
            std::swap(fa.p, fb.p);
        }
        blocks.resize(nblk);
        if (nblk) QDFN_CUDA(cudaMemcpy(blocks.data(), db.p, nblk * sizeof(int4), cudaMemcpyDeviceToHost));
    }
    auto* h = new qdfn_hstruct();
    h->N = N;
    h->perm.resize(N);
    {
        std::vector<long long> order(N);
        QDFN_CUDA(cudaMemcpy(order.data(), dorder.p, N * sizeof(long long), cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < N; ++i) h->perm[i] = order[i];
    }
    // a fixed block order: by receiver start, then source start
    std::sort(blocks.begin(), blocks.end(), [&](const int4& a, const int4& b) {
        return nstart[a.y] != nstart[b.y] ? nstart[a.y] < nstart[b.y] : nstart[a.x] < nstart[b.x];
    });
    h->ranges.reserve(4 * blocks.size());
    for (const int4& b : blocks) {
        h->ranges.push_back(nstart[b.x]);
        h->ranges.push_back(nend[b.x] - 1);
        h->ranges.push_back(nstart[b.y]);
        h->ranges.push_back(nend[b.y] - 1);
        h->adm.push_back(b.z);
    }
    h->nstart.assign(nstart.begin(), nstart.end());
    h->nend.assign(nend.begin(), nend.end());
    *out = h;
    return QDFN_OK;
}

extern "C" int qdfn_hstruct_sizes(const qdfn_hstruct* h, int64_t* n_blocks, int64_t* n_nodes) {
    if (!h) return fail(QDFN_ERR_INVALID, "null structure");
    if (n_blocks) *n_blocks = (int64_t)h->adm.size();
    if (n_nodes) *n_nodes = (int64_t)h->nstart.size();
    return QDFN_OK;
}

extern "C" int qdfn_hstruct_get(const qdfn_hstruct* h, int64_t* perm, int64_t* ranges, int32_t* admissible) {
    if (!h) return fail(QDFN_ERR_INVALID, "null structure");
    if (perm) std::copy(h->perm.begin(), h->perm.end(), perm);
    if (ranges) std::copy(h->ranges.begin(), h->ranges.end(), ranges);
    if (admissible) std::copy(h->adm.begin(), h->adm.end(), admissible);
    return QDFN_OK;
}

extern "C" int qdfn_hstruct_destroy(qdfn_hstruct* h) {
    delete h;
    return QDFN_OK;
}
