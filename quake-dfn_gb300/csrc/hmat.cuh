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
// would leave most threads idle):
//   A: t_b[kk] = Vt_b[kk,:] x[src]    one task per (low-rank block, rank row):
//                                     lanes stride the row, coalesced, warp sum
//   B: partial(b, i) = (D_b x[src])_i or (U_b t_b)_i
//                                     one task per (block, 64-row slice): a
//                                     lane per row (two rows), the x or t
//                                     values held by the lanes and broadcast
//                                     by shuffles, coalesced loads of D^T / U^T
// and every receiver row then sums its partials in block order (a fixed
// order, so results are reproducible run to run).  Tasks are listed largest
// first, so the static round-robin spreads the long ones over the warps.
#pragma once
#include "qdfn_internal.h"

namespace qdfn {
namespace hmat {

struct Blk {
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
    const int64_t* lr_list;  // pass-A tasks: (blk index << 8) | rank row
    int64_t n_lr;
    const int64_t* tile_list;   // pass-B tasks: (blk index << 20) | 64-row slice
    int64_t n_tiles;
    double* t;               // low-rank intermediates
    double* part;            // [slots][R]
    const int64_t* rowptr;   // [2][N+1] CSR over receiver rows (shear, normal)
    const int64_t* rowslot;  // slot indices
};

constexpr int kSliceRows = 64;     // pass-B rows per warp task (two per lane)
constexpr int kChunk = 1024;       // (shared-memory sizing of the H launches)
constexpr int kMaxRank = 128;

__device__ __forceinline__ int64_t warp_id_global() {
    return (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
}
__device__ __forceinline__ int64_t warps_global() { return (int64_t)gridDim.x * (blockDim.x >> 5); }

// pass A: t_b = Vt_b x[src]
template <class T, int R>
__device__ void pass_a(const Ops& h, const double* __restrict__ D, int64_t N, T*, double*) {
    const int lane = threadIdx.x & 31;
    const T* st = reinterpret_cast<const T*>(h.store);
    for (int64_t q = warp_id_global(); q < h.n_lr; q += warps_global()) {
        const int64_t code = h.lr_list[q];
        const Blk b = h.blk[code >> 8];
        const int kk = (int)(code & 255);
        const T* row = st + b.off_a + (int64_t)kk * b.ns;
        // each lane's products summed in T -- FP32 storage as an error-free
        // (hi, lo) pair on the FP32 pipe -- then the warp's sum in FP64
        T hi[R], lo[R];
#pragma unroll
        for (int r = 0; r < R; ++r) { hi[r] = 0; lo[r] = 0; }
        for (int64_t j = lane; j < b.ns; j += 32) {
            const T v = __ldg(row + j);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const T p = v * (T)__ldcg(D + (int64_t)r * N + b.s0 + j);
                if constexpr (sizeof(T) == 4) {
                    const T sum = hi[r] + p, bp = sum - hi[r];
                    lo[r] += (hi[r] - (sum - bp)) + (p - bp);
                    hi[r] = sum;
                } else {
                    hi[r] += p;
                }
            }
        }
        double s[R];
#pragma unroll
        for (int r = 0; r < R; ++r) s[r] = (double)hi[r] + (double)lo[r];
#pragma unroll
        for (int r = 0; r < R; ++r) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s[r] += __shfl_xor_sync(0xffffffffu, s[r], o);
        }
        if (lane < R) {
            double v = s[0];
#pragma unroll
            for (int r = 1; r < R; ++r)
                if (lane == r) v = s[r];
            h.t[(b.toff + kk) * R + lane] = v;
        }
    }
}

// pass B: per receiver-row partials of every block, 64-row slices per warp
template <class T, int R>
__device__ void pass_b(const Ops& h, const double* __restrict__ D, int64_t N, T*) {
    const int lane = threadIdx.x & 31;
    const T* st = reinterpret_cast<const T*>(h.store);
    for (int64_t q = warp_id_global(); q < h.n_tiles; q += warps_global()) {
        const int64_t code = h.tile_list[q];
        const Blk b = h.blk[code >> 20];
        const int64_t i0 = (code & ((1 << 20) - 1)) * kSliceRows;
        const int64_t ia = i0 + lane, ib = i0 + 32 + lane;
        const bool va = ia < b.nr, vb = ib < b.nr;
        T sa[R], sb[R];
#pragma unroll
        for (int r = 0; r < R; ++r) { sa[r] = 0; sb[r] = 0; }
        const int64_t K = b.rank < 0 ? b.ns : b.rank;   // the inner dimension
        const T* base = st + (b.rank < 0 ? b.off_a : b.off_b);
        for (int64_t j0 = 0; j0 < K; j0 += 32) {
            // the lanes hold 32 inner values (x of the block's sources, or t)
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
            for (int jj = 0; jj < L; ++jj) {
                const T* col = base + (j0 + jj) * b.nr;
                const T ma = va ? __ldg(col + ia) : (T)0;
                const T mb = vb ? __ldg(col + ib) : (T)0;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const T x = __shfl_sync(0xffffffffu, xv[r], jj);
                    sa[r] = fma(ma, x, sa[r]);
                    sb[r] = fma(mb, x, sb[r]);
                }
            }
        }
        if (va)
#pragma unroll
            for (int r = 0; r < R; ++r) h.part[(b.slot + ia) * R + r] = (double)sa[r];
        if (vb)
#pragma unroll
            for (int r = 0; r < R; ++r) h.part[(b.slot + ib) * R + r] = (double)sb[r];
    }
}

// sum of the partials of receiver row i (side 0 shear, 1 normal), block order
template <int R>
__device__ __forceinline__ double row_sum(const Ops& h, int side, int64_t N, int64_t i, int r) {
    const int64_t* rp = h.rowptr + side * (N + 1);
    double s = 0.0;
    for (int64_t q = rp[i]; q < rp[i + 1]; ++q) s += __ldcg(h.part + h.rowslot[q] * R + r);
    return s;
}

}  // namespace hmat
}  // namespace qdfn
