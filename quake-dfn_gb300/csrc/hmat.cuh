// H-matrix elastic operator on the device (the block loop of
// HmatSolver_Pararllel, scripts/Functions_Hmatrix.jl:631-646).
//
// Block b maps source range [s0, s0+ns) to receiver range [r0, r0+nr).  Each of
// the shear and normal matrices has its own block list (same ranges, own
// ranks).  Storage, all in one buffer of the operator's element type:
//   dense  D^T, ns x nr   (entry (row i, col j) at j*nr + i: lanes on
//                          consecutive receiver rows read consecutive words)
//   low-rank  Vt, k x ns row-major, and U^T, k x nr
// The product runs in two passes inside the persistent kernel, as WARP tasks
// handed out in a fixed order over every warp of the grid (tree leaves hold at
// most `leaf` patches, so near-field blocks are small and a block per CTA
// would leave most threads idle); pass B starts with the dense blocks, which
// need nothing from pass A, and waits on a completion count of pass A (not on
// a grid barrier) before its low-rank blocks:
//   A: t_b[kk] = Vt_b[kk,:] x[src]    one task per (low-rank block, group of
//                                     rank rows): lanes stride the rows,
//                                     coalesced, warp sums
//   B: partial(b, i) = (D_b x[src])_i or (U_b t_b)_i
//                                     one task per (block, 64-row slice): a
//                                     lane per row (two rows), the x or t
//                                     values held by the lanes and broadcast
//                                     by shuffles, coalesced loads of D^T / U^T
// and every receiver row then sums its partials (row_sums_block: four threads
// per row and matrix, each over every fourth partial in block order, combined
// in a fixed order, so results are reproducible run to run).  Tasks are listed
// largest first and dealt out to the warps in snake order, which spreads the
// long ones.
#pragma once
#include "qdfn_internal.h"

namespace qdfn {
namespace hmat {

struct Blk {   // 72 bytes
    int64_t s0, ns, r0, nr;
    int64_t off_a;   // dense: D^T offset; low-rank: Vt offset
    int64_t off_b;   // low-rank: U^T offset
    int64_t toff;    // low-rank: t offset (in units of k entries, times R)
    int64_t slot;    // first partial slot (one per receiver row of the block)
    int32_t rank;    // < 0: dense
    int32_t pad;
};

struct Ops {
    const Blk* blk;          // [2][nb]: shear blocks then normal blocks
    int64_t nb;
    const void* store;       // element storage
    const int64_t* lr_list;  // pass-A tasks: (blk index << 8) | first rank row of the group
    int64_t n_lr;
    const int64_t* tile_list;   // pass-B tasks: (blk index << 20) | 64-row slice; dense blocks' first
    int64_t n_tiles;
    int64_t n_tiles_dense;      // the first n_tiles_dense tasks are dense blocks' (need no pass A)
    unsigned long long* a_done; // pass-A tasks completed since the launch began (monotone)
    double* t;               // low-rank intermediates
    double* part;            // [slots][R]
    const int64_t* rowptr;   // [2][N+1] CSR over receiver rows (shear, normal)
    const int64_t* rowslot;  // slot indices
};

static_assert(sizeof(Blk) == 72 && alignof(Blk) == 8, "Blk is read as nine 8-byte words");

constexpr int kSliceRows = 64;     // pass-B rows per warp task (two per lane)
constexpr int kChunk = 1024;       // (shared-memory sizing of the H launches)
constexpr int kMaxRank = 128;

__device__ __forceinline__ int64_t warp_id_global() {
    return (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
}
__device__ __forceinline__ int64_t warps_global() { return (int64_t)gridDim.x * (blockDim.x >> 5); }
// Task k of warp w among W warps: the lists are sorted largest first and dealt
// out in snake order (rounds alternate direction), so that no warp takes the
// largest task of every round
__device__ __forceinline__ int64_t snake_task(int64_t k, int64_t w, int64_t W) {
    return k * W + ((k & 1) ? W - 1 - w : w);
}

// rank rows per pass-A task: each lane keeps (hi, lo) sums for every row and
// instance in registers
template <int R>
__host__ __device__ constexpr int rows_a() { return R <= 2 ? 8 : 4; }

// A task's block descriptor, loaded once per task: nine independent 8-byte
// loads (every lane the same words; the array's 72-byte stride keeps only
// 8-byte alignment)
__device__ __forceinline__ Blk load_blk(const Blk* p) {
    const long long* w = reinterpret_cast<const long long*>(p);
    Blk b;
    b.s0 = __ldg(w); b.ns = __ldg(w + 1); b.r0 = __ldg(w + 2); b.nr = __ldg(w + 3);
    b.off_a = __ldg(w + 4); b.off_b = __ldg(w + 5); b.toff = __ldg(w + 6); b.slot = __ldg(w + 7);
    const int2 rk = __ldg(reinterpret_cast<const int2*>(w + 8));
    b.rank = rk.x;
    b.pad = rk.y;
    return b;
}

// Warp sums of G values per lane (G = 4 or 8; R instances each) kept as FP32
// (hi, lo) pairs (FP64 storage: hi alone).  The first log2(G) butterfly levels
// halve the values a lane holds -- at offset o a lane keeps the half its lane
// bit o selects and adds its partner's copy of that half -- so that lane L
// ends with the sum of value L / (32 / G) over its 32 / G-lane group; the last
// levels are plain butterflies.  Each combine is an error-free FP32 two-sum
// (hi) with the low parts added, so the warp reduction costs a few FP32
// operations per value instead of a chain of FP64 additions (the FP64 pipe is
// the GPU's narrowest).  Returns the FP64 sums in out (valid on the lanes
// L % (32 / G) == 0); fixed order, so results are reproducible.
template <class T, int G, int R>
__device__ __forceinline__ void warp_sums(T (&hi)[G][R], T (&lo)[G][R], int lane, double (&out)[R]) {
    static_assert(G == 4 || G == 8, "rank rows per task");
    auto combine = [](T& ah, T& al, T bh, T bl) {
        if constexpr (sizeof(T) == 4) {
            const T s = ah + bh, bp = s - ah;
            const T e = (ah - (s - bp)) + (bh - bp);
            al = al + bl + e;
            ah = s;
        } else {
            ah = ah + bh;
        }
    };
#pragma unroll
    for (int n = G, o = 16; n > 1; n >>= 1, o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int k = 0; k < n / 2; ++k)
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const T kh = up ? hi[k + n / 2][r] : hi[k][r], sh = up ? hi[k][r] : hi[k + n / 2][r];
                const T kl = up ? lo[k + n / 2][r] : lo[k][r], sl = up ? lo[k][r] : lo[k + n / 2][r];
                const T oh = __shfl_xor_sync(0xffffffffu, sh, o);
                T ol = 0;
                if constexpr (sizeof(T) == 4) ol = __shfl_xor_sync(0xffffffffu, sl, o);
                hi[k][r] = kh;
                lo[k][r] = kl;
                combine(hi[k][r], lo[k][r], oh, ol);
            }
    }
#pragma unroll
    for (int o = 16 / G; o > 0; o >>= 1)
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const T oh = __shfl_xor_sync(0xffffffffu, hi[0][r], o);
            T ol = 0;
            if constexpr (sizeof(T) == 4) ol = __shfl_xor_sync(0xffffffffu, lo[0][r], o);
            combine(hi[0][r], lo[0][r], oh, ol);
        }
#pragma unroll
    for (int r = 0; r < R; ++r) out[r] = sizeof(T) == 4 ? (double)hi[0][r] + (double)lo[0][r] : (double)hi[0][r];
}

// The fields of a block descriptor that pass A reads (five words).
struct BlkA {
    int64_t s0, ns, off_a, toff;
    int rank;
};
__device__ __forceinline__ BlkA load_blk_a(const Blk* p) {
    const long long* w = reinterpret_cast<const long long*>(p);
    BlkA b;
    b.s0 = __ldg(w); b.ns = __ldg(w + 1); b.off_a = __ldg(w + 4); b.toff = __ldg(w + 6);
    b.rank = __ldg(reinterpret_cast<const int*>(w + 8));
    return b;
}

// pass A: t_b = Vt_b x[src], one task per (low-rank block, group of up to
// rows_a rank rows): the lanes stride the block's source range, each load of
// x serving every row of the group, and each round issues the group's rows x 4
// column loads before any of them is used (HBM latency is hidden by the loads
// in flight, not by occupancy: one 16-warp CTA per SM)
template <class T, int R>
__device__ void pass_a(const Ops& h, const double* __restrict__ D, int64_t N, T*, double*) {
    constexpr int G = rows_a<R>();
    // 32-column rounds per batch (G x kUA loads per lane in flight), within the
    // persistent kernel's 128 registers
    constexpr int kUA = (sizeof(T) == 4 && R == 1) ? 4 : 2;
    const int lane = threadIdx.x & 31;
    const T* st = reinterpret_cast<const T*>(h.store);
    const int64_t W = warps_global(), w = warp_id_global();
    // the block descriptor of the next task is loaded while this one runs, and
    // the task code of the one after it: a small task then costs one round trip
    // (its data), not three (code, descriptor, data)
    int64_t k = 0, q = snake_task(0, w, W);
    const int64_t q1 = snake_task(1, w, W);
    int64_t code = q < h.n_lr ? __ldg(h.lr_list + q) : 0;
    int64_t code_n = q1 < h.n_lr ? __ldg(h.lr_list + q1) : 0;
    BlkA b = load_blk_a(h.blk + (code >> 8));
    unsigned long long done = 0;
    while (q < h.n_lr) {
        const int64_t qn = snake_task(++k, w, W), qnn = snake_task(k + 1, w, W);
        const int64_t code_nn = qnn < h.n_lr ? __ldg(h.lr_list + qnn) : 0;
        const BlkA bn = load_blk_a(h.blk + (code_n >> 8));
        const int kk0 = (int)(code & 255);
        const int nrow = min(G, b.rank - kk0);
        const T* row0 = st + b.off_a + (int64_t)kk0 * b.ns;
        const double* xs = D + b.s0;
        // each lane's products summed in T -- FP32 storage as an error-free
        // (hi, lo) pair on the FP32 pipe -- then the warp's sums (warp_sums)
        T hi[G][R], lo[G][R];
#pragma unroll
        for (int g = 0; g < G; ++g)
#pragma unroll
            for (int r = 0; r < R; ++r) { hi[g][r] = 0; lo[g][r] = 0; }
        for (int64_t j0 = 0; j0 < b.ns; j0 += 32 * kUA) {
            T v[kUA][G], xv[kUA][R];
#pragma unroll
            for (int u = 0; u < kUA; ++u) {
                const int64_t j = j0 + u * 32 + lane;
                const bool ok = j < b.ns;
#pragma unroll
                for (int g = 0; g < G; ++g) v[u][g] = (ok && g < nrow) ? __ldg(row0 + (int64_t)g * b.ns + j) : (T)0;
#pragma unroll
                for (int r = 0; r < R; ++r) xv[u][r] = ok ? (T)__ldcg(xs + (int64_t)r * N + j) : (T)0;
            }
#pragma unroll
            for (int u = 0; u < kUA; ++u)
#pragma unroll
                for (int g = 0; g < G; ++g)
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const T pr = v[u][g] * xv[u][r];
                        if constexpr (sizeof(T) == 4) {
                            const T sum = hi[g][r] + pr, bp = sum - hi[g][r];
                            lo[g][r] += (hi[g][r] - (sum - bp)) + (pr - bp);
                            hi[g][r] = sum;
                        } else {
                            hi[g][r] += pr;
                        }
                    }
        }
        double tot[R];
        warp_sums<T, G, R>(hi, lo, lane, tot);
        constexpr int kSpan = 32 / G;   // lanes per row after the halving levels
        const int g = lane / kSpan;
        if (lane % kSpan == 0 && g < nrow) {
#pragma unroll
            for (int r = 0; r < R; ++r) h.t[(b.toff + kk0 + g) * R + r] = tot[r];
        }
        q = qn;
        code = code_n;
        code_n = code_nn;
        b = bn;
        ++done;
    }
    // publish this warp's tasks: every lane fences its own t stores first
    __threadfence();
    __syncwarp();
    if (lane == 0 && done > 0 && h.a_done) atomicAdd(h.a_done, done);
}

__device__ __forceinline__ unsigned long long ld_acquire_ull(const unsigned long long* ptr) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(ptr) : "memory");
    return v;
}

// pass B: per receiver-row partials of every block, 64-row slices per warp
// (a lane per two rows).  The inner values (x of the block's sources, or t)
// are held by the lanes and broadcast by shuffles; the matrix columns are
// loaded sixteen at a time before they are used.  Tasks [lo, hi) of the list.
template <class T, int R>
__device__ void pass_b_range(const Ops& h, const double* __restrict__ D, int64_t N, int64_t lo, int64_t hi) {
    constexpr int U = sizeof(T) == 4 ? 16 : 8;   // columns loaded per batch: 2 x U loads per lane in flight
    const int lane = threadIdx.x & 31;
    const T* st = reinterpret_cast<const T*>(h.store);
    const int64_t W = warps_global(), w = warp_id_global();
    const int64_t n = hi - lo;
    int64_t k = 0, q = snake_task(0, w, W);
    int64_t code = q < n ? __ldg(h.tile_list + lo + q) : 0;
    while (q < n) {
        const Blk b = load_blk(h.blk + (code >> 20));
        const int64_t i0 = (code & ((1 << 20) - 1)) * kSliceRows;
        const int64_t qn = snake_task(++k, w, W);
        const int64_t code_n = qn < n ? __ldg(h.tile_list + lo + qn) : 0;
        const int64_t ia = i0 + lane, ib = i0 + 32 + lane;
        const bool va = ia < b.nr, vb = ib < b.nr;
        T sa[R], sb[R];
#pragma unroll
        for (int r = 0; r < R; ++r) { sa[r] = 0; sb[r] = 0; }
        const int64_t K = b.rank < 0 ? b.ns : b.rank;   // the inner dimension
        const T* base = st + (b.rank < 0 ? b.off_a : b.off_b);
        for (int64_t j0 = 0; j0 < K; j0 += 32) {
            T xv[R];
            const int64_t jl = j0 + lane;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                double v = 0.0;
                if (jl < K)
                    v = b.rank < 0 ? __ldcg(D + (int64_t)r * N + b.s0 + jl) : __ldcg(h.t + (b.toff + jl) * R + r);
                xv[r] = (T)v;
            }
            const int L = (int)min((int64_t)32, K - j0);
            for (int jb = 0; jb < L; jb += U) {
                T ma[U], mb[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const bool ok = jb + u < L;
                    const T* col = base + (j0 + jb + u) * b.nr;
                    ma[u] = (ok && va) ? __ldg(col + ia) : (T)0;
                    mb[u] = (ok && vb) ? __ldg(col + ib) : (T)0;
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const T x = __shfl_sync(0xffffffffu, xv[r], (jb + u) & 31);
                        sa[r] = fma(ma[u], x, sa[r]);
                        sb[r] = fma(mb[u], x, sb[r]);
                    }
                }
            }
        }
        if (va)
#pragma unroll
            for (int r = 0; r < R; ++r) h.part[(b.slot + ia) * R + r] = (double)sa[r];
        if (vb)
#pragma unroll
            for (int r = 0; r < R; ++r) h.part[(b.slot + ib) * R + r] = (double)sb[r];
        q = qn;
        code = code_n;
    }
}

// Pass B of a step: the dense blocks' tasks first (they need no pass-A
// result, so they fill the time while the last pass-A tasks finish), then a
// bounded wait until a_done reaches a_target (every pass-A task of this step
// has published its t), then the low-rank blocks' tasks.  a_target = 0: no
// wait (pass A ran in an earlier launch).  Returns false if the wait gave up
// (limit_ns, or another block's error in *gerr).
template <class T, int R>
__device__ bool pass_b(const Ops& h, const double* __restrict__ D, int64_t N, unsigned long long a_target,
                       uint64_t limit_ns, const int* gerr) {
    pass_b_range<T, R>(h, D, N, 0, h.n_tiles_dense);
    if (h.n_tiles <= h.n_tiles_dense) return true;
    int ok = 1;
    if (a_target > 0 && (threadIdx.x & 31) == 0 && ld_acquire_ull(h.a_done) < a_target) {
        uint64_t t0;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
        while (ld_acquire_ull(h.a_done) < a_target) {
            uint64_t t;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
            if (t - t0 > limit_ns || *(volatile const int*)gerr != 0) { ok = 0; break; }
            __nanosleep(128);
        }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok) return false;
    pass_b_range<T, R>(h, D, N, h.n_tiles_dense, h.n_tiles);
    return true;
}

// The products of a block's solve items q0..q1-1 (q = r N + i) for a step's
// first solve pass, by the whole block before its solves: four threads per
// (item, matrix), each summing every fourth partial of the row in block
// order, combined as (p0 + p1) + (p2 + p3) -- a fixed order, so results are
// reproducible; the solves then read tld and knd.  Every thread of the block
// runs the same rounds (the shuffles need whole warps).
template <int R>
__device__ void row_sums_block(const Ops& h, int64_t N, const double* __restrict__ kself, double* __restrict__ tld,
                               double* __restrict__ knd, int64_t q0, int64_t q1) {
    const int64_t work = (q1 - q0) * 8;
    for (int64_t base = 0; base < work; base += blockDim.x) {
        const int64_t t = base + threadIdx.x;
        const bool valid = t < work;
        const int sub = (int)(t & 3), side = (int)((t >> 2) & 1);
        double acc = 0.0;
        int64_t q = 0, i = 0;
        if (valid) {
            q = q0 + (t >> 3);
            const int r = (int)(q / N);
            i = q - (int64_t)r * N;
            const int64_t* rp = h.rowptr + side * (N + 1);
            const int64_t e = __ldg(rp + i + 1);
            int64_t k = __ldg(rp + i) + sub;
            for (; k + 12 < e; k += 16) {   // four of this thread's partials at a time, loaded before added
                int64_t sl[4];
                double v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) sl[u] = __ldg(h.rowslot + k + 4 * u);
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = __ldcg(h.part + sl[u] * R + r);
#pragma unroll
                for (int u = 0; u < 4; ++u) acc += v[u];
            }
            for (; k < e; k += 4) acc += __ldcg(h.part + __ldg(h.rowslot + k) * R + r);
        }
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
        if (valid && sub == 0) {
            if (side == 0) tld[q] = (-acc) / -kself[i];   // main_H :241-248: H_load (0 - D) ./ -K_Self
            else knd[q] = acc;                           // H_n D
        }
    }
}

}  // namespace hmat
}  // namespace qdfn
