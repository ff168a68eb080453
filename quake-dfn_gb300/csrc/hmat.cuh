// H-matrix elastic operator on the device (the block loop of
// HmatSolver_Pararllel, scripts/Functions_Hmatrix.jl:631-646).
//
// Block b maps source range [s0, s0+ns) to receiver range [r0, r0+nr).  Each of
// the shear and normal matrices has its own block list (same ranges, own
// ranks).  Storage, all in one buffer of the operator's element type:
//   dense  D^T, ns x nr   (entry (row i, col j) at j*nr + i: threads on
//                          consecutive receiver rows read consecutive words)
//   low-rank  Vt, k x ns row-major, and U^T, k x nr
// The product runs in two passes inside the persistent kernel:
//   A: t_b = Vt_b x[src]       one CTA per low-rank block, x staged in shared memory
//   B: partial(b, i) = (D_b x[src])_i or (U_b t_b)_i   one CTA per 256-row tile
// and every receiver row then sums its partials in block order (a fixed
// order, so results are reproducible run to run).
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
    const int64_t* lr_list;  // indices (into blk) of low-rank blocks, shear and normal
    int64_t n_lr;
    const int64_t* tile_list;   // pass-B tasks: (blk index << 20) | tile
    int64_t n_tiles;
    double* t;               // low-rank intermediates
    double* part;            // [slots][R]
    const int64_t* rowptr;   // [2][N+1] CSR over receiver rows (shear, normal)
    const int64_t* rowslot;  // slot indices
};

constexpr int kTileRows = 512;     // one receiver row per thread of a 512-thread block
constexpr int kChunk = 1024;
constexpr int kMaxRank = 128;

// pass A: t_b = Vt_b x[src]
template <class T, int R>
__device__ void pass_a(const Ops& h, const double* __restrict__ D, int64_t N, T* xs, double* acc) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const T* st = reinterpret_cast<const T*>(h.store);
    for (int64_t q = blockIdx.x; q < h.n_lr; q += gridDim.x) {
        const Blk b = h.blk[h.lr_list[q]];
        const int k = b.rank;
        for (int i = threadIdx.x; i < k * R; i += blockDim.x) acc[i] = 0.0;
        for (int64_t c0 = 0; c0 < b.ns; c0 += kChunk) {
            const int64_t L = min((int64_t)kChunk, b.ns - c0);
            __syncthreads();
            for (int64_t e = threadIdx.x; e < L * R; e += blockDim.x) {
                const int r = (int)(e / L);
                const int64_t j = e - (int64_t)r * L;
                xs[r * kChunk + j] = (T)__ldcg(D + (int64_t)r * N + b.s0 + c0 + j);
            }
            __syncthreads();
            for (int kk = wid; kk < k; kk += nw) {
                const T* row = st + b.off_a + (int64_t)kk * b.ns + c0;
                double s[R];
#pragma unroll
                for (int r = 0; r < R; ++r) s[r] = 0.0;
                for (int64_t j = lane; j < L; j += 32) {
                    const T v = __ldg(row + j);
#pragma unroll
                    for (int r = 0; r < R; ++r) s[r] += (double)(v * xs[r * kChunk + j]);
                }
#pragma unroll
                for (int r = 0; r < R; ++r) {
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) s[r] += __shfl_xor_sync(0xffffffffu, s[r], o);
                    if (lane == 0) acc[kk * R + r] += s[r];
                }
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < k * R; i += blockDim.x) h.t[b.toff * R + i] = acc[i];
        __syncthreads();
    }
}

// pass B: per receiver-row partials of every block
template <class T, int R>
__device__ void pass_b(const Ops& h, const double* __restrict__ D, int64_t N, T* xs) {
    const T* st = reinterpret_cast<const T*>(h.store);
    for (int64_t q = blockIdx.x; q < h.n_tiles; q += gridDim.x) {
        const int64_t code = h.tile_list[q];
        const Blk b = h.blk[code >> 20];
        const int64_t i0 = (code & ((1 << 20) - 1)) * kTileRows;
        const int64_t i = i0 + threadIdx.x;
        double out[R];
#pragma unroll
        for (int r = 0; r < R; ++r) out[r] = 0.0;
        if (b.rank < 0) {
            for (int64_t c0 = 0; c0 < b.ns; c0 += kChunk) {
                const int64_t L = min((int64_t)kChunk, b.ns - c0);
                __syncthreads();
                for (int64_t e = threadIdx.x; e < L * R; e += blockDim.x) {
                    const int r = (int)(e / L);
                    const int64_t j = e - (int64_t)r * L;
                    xs[r * kChunk + j] = (T)__ldcg(D + (int64_t)r * N + b.s0 + c0 + j);
                }
                __syncthreads();
                if (i < b.nr) {
                    const T* col = st + b.off_a + c0 * b.nr + i;
                    T s[R];
#pragma unroll
                    for (int r = 0; r < R; ++r) s[r] = 0;
                    for (int64_t j = 0; j < L; ++j) {
                        const T v = __ldg(col + j * b.nr);
#pragma unroll
                        for (int r = 0; r < R; ++r) s[r] = fma(v, xs[r * kChunk + j], s[r]);
                    }
#pragma unroll
                    for (int r = 0; r < R; ++r) out[r] += (double)s[r];
                }
            }
        } else {
            const int k = b.rank;
            __syncthreads();
            for (int e = threadIdx.x; e < k * R; e += blockDim.x)
                xs[e] = (T)__ldcg(h.t + b.toff * R + e);
            __syncthreads();
            if (i < b.nr) {
                const T* col = st + b.off_b + i;
                T s[R];
#pragma unroll
                for (int r = 0; r < R; ++r) s[r] = 0;
                for (int kk = 0; kk < k; ++kk) {
                    const T v = __ldg(col + (int64_t)kk * b.nr);
#pragma unroll
                    for (int r = 0; r < R; ++r) s[r] = fma(v, xs[kk * R + r], s[r]);
                }
#pragma unroll
                for (int r = 0; r < R; ++r) out[r] = (double)s[r];
            }
        }
        if (i < b.nr)
#pragma unroll
            for (int r = 0; r < R; ++r) h.part[(b.slot + i) * R + r] = out[r];
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
