// Device code of the persistent earthquake-cycle kernel (see sim.cu for the
// step structure), shared by the single-context launch (sim.cu) and the
// ensemble launch (ensemble.cu).
#pragma once
#include <cooperative_groups.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "qdfn_internal.h"
#include "hmat.cuh"
#include "sim_device.cuh"

namespace qdfn {
namespace {

constexpr int kSimThreads = 512;
// per-step counter sets in rotation: step s uses set s, streams the next
// step's early tiles into set s+1 and resets set s+2 (mod kSets), whose last
// reader -- step s-2's early-tile producers, which may run into the start of
// step s-1 -- has passed a grid barrier since
constexpr int kSets = 4;
constexpr int kGranule = 8;                 // operator bytes per thread and source column
constexpr int kMaxInst = 4;
constexpr int kRedSlots = 16;               // doubles per (CTA, instance) partial
constexpr int64_t kRetryCap = 10000;        // retries of one step before giving up
constexpr int kCounters = 18;               // qdfn_get_counters slots

// ---------------------------------------------------------------------------
// matrix element formats: each thread owns VEC consecutive receiver rows, one
// kGranule-byte granule per source column (sload decodes it from shared memory).
struct FmtF64 {
    static constexpr int VEC = 1;
    using X = double;  // staged x type
    __device__ __forceinline__ static void sload(const unsigned char* p, double v[1]) {
        v[0] = *reinterpret_cast<const double*>(p);
    }
};
struct FmtF32 {
    static constexpr int VEC = 2;
    using X = float;
    __device__ __forceinline__ static void sload(const unsigned char* p, float v[2]) {
        const float2 q = *reinterpret_cast<const float2*>(p);
        v[0] = q.x; v[1] = q.y;
    }
};
struct FmtBF16x2 {  // each 32-bit word: hi bf16 in the upper half, lo bf16 in the lower half
    static constexpr int VEC = 2;
    using X = float;
    __device__ __forceinline__ static void sload(const unsigned char* p, float v[2]) {
        const uint2 q = *reinterpret_cast<const uint2*>(p);
        v[0] = __uint_as_float(q.x & 0xFFFF0000u) + __uint_as_float(q.x << 16);
        v[1] = __uint_as_float(q.y & 0xFFFF0000u) + __uint_as_float(q.y << 16);
    }
};

}  // namespace

// Launch parameters of the persistent kernel (one context, or one member of
// an ensemble launch).
struct SimParams {
    int64_t N, Nload, ld;
    int R;
    int nblk;                        // thread blocks that run this context (its grid barrier's size)
    int evolution_dr, interp_at_told, hmat;
    double eta, sigma_min, switch_v, dt_cut, rupture_dt, max_dt, alpha_evo;
    int64_t record_step, max_records;
    // per [R][N] constants
    const double *a, *b, *Dc, *F0, *tau0, *sigma0, *Vconst, *mass, *omega;
    const double *ra, *rDc;          // 1/a and 1/Dc, correctly rounded (fixed for a run)
    const double* kself;             // [N]
    const unsigned char* unstable;   // [R][N]
    const int* has_unstable;         // [R]
    // external stress
    int64_t n_ext;
    const double *ext_t, *ext_n, *ext_s, *ext_p;
    // dense operator, source-major: entry (recv i, src j) at j*ld + i
    const void* E;
    const void* Kn;
    void* xd;                        // dense: D in the operator's x type, [patch][instance], padded;
                                     // two copies xd_stride elements apart (current / next step)
    int64_t xbuf;                    // dense: elements of one of the two shared-memory x buffers
    int64_t xd_stride, rb_stride;    // element strides of the two x copies and row-block counter sets
    hmat::Ops h;                     // H-matrix operator (hmat != 0)
    int nchunk;                      // column chunks of the matvec per row block
    int64_t chunk_len;
    // the row blocks from rb_small0 on (streamed last) use nchunk2 chunks of
    // chunk_len2 columns: smaller tiles at the end of the stream even out the
    // blocks' finishing times and shrink the last row blocks' solve tail
    int nchunk2;
    int64_t chunk_len2, rb_small0;
    // state [R][N]
    // state, two buffers swapped per accepted step: (V, D, theta, fric, accel,
    // sig_old, sw) and (Vn, Dn, thn, fn, accel_n, sn, sw_n); the host sees the
    // first set (the kernel copies back at its end when needed)
    double *V, *D, *theta, *fric, *accel, *sig_old;
    double *Vn, *Dn, *thn, *fn, *sn, *accel_n, *dtall, *tld, *knd;
    int *instab, *flag, *sw, *sw_n;
    double *part_s, *part_n;         // [2][max(nchunk, nchunk2)][R][N], by step parity
    int64_t part_stride;             // elements of one of the two partial buffers
    // scalars [R]
    double *T, *dt;
    int64_t *step, *nrec;
    int* status;                     // [R]
    // history [R][max_records][N] and [R][max_records]
    double *hT, *hDt, *hV, *hD, *hth, *hs;
    // barrier + reductions
    unsigned *bar_count, *bar_gen;
    double* red;                     // [2][nblocks][R][kRedSlots]
    // per-step counters, kSets sets used by steps in turn (mod kSets): [kSets],
    // and rb_done / rb_solved / rb_hot [kSets][rb_stride]
    unsigned long long* tile_ctr;    // dynamic tile counter of the dense operator
    unsigned long long* spec_ctr;    // tiles of the step streamed ahead during the step before
    unsigned* rb_solved;             // dense: solved row chunks per row block
    unsigned* rb_hot;                // dense: row block holds a patch on the high-velocity solver next step
    unsigned* rb_done;               // dense: tile arrivals per row block (one per operator warp and tile)
    unsigned long long* solve_ctr;   // dense: row chunks handed to the solver warps
    int* gerr;
    uint64_t budget_ns;             // wall-time budget of this launch
    unsigned long long* prof;       // cumulative counters (qdfn_get_counters)
    int64_t n_rb;                    // dense: operator row blocks
    int hold_cap;                    // dense: row chunks a block may hold at once in the overlapped phase
    int pair_solve;                  // overlapped phase: 1 one lane pair per patch, 16-row chunks; 2 one
                                     // lane per patch, 32-row chunks; 0 the even lanes alone, 16-row chunks
    int rb_ordered;                  // FP32/BF16 dense: row blocks with high-velocity patches first
    int c_spec;                      // dense: column chunks of the next step streamed during a step's tail
    int spec_stop;                   // no early-tile claims once this many blocks reached the step's barrier
    // ensemble "fill" mode (null: off): a member that has taken its nsteps
    // steps adds one to *fill_ctr and keeps stepping until fill_need members
    // have, so that no SM idles while the slowest member finishes
    unsigned* fill_ctr;
    unsigned fill_need;
    // adjoint recording (null: off): the solver each patch's accepted pass
    // used, [R][N] (0 low velocity, 1 high velocity, 2 loading fault)
    unsigned char* sw_used;
    // FP32/BF16 dense operator: the x copy of D holds D - dref (dref = slip of
    // patch 0 at the start of the step before, per instance, [2][R] by step
    // parity), and the products add dref x the stored matrices' row sums
    // (FP64, [N]; null for FP64 storage) -- the rounding of x to FP32 then
    // scales with the slip's spread over the patches, not with the slip
    double* dref;
    const double *rowsum_e, *rowsum_n;
    unsigned long long* tmax;        // [kSets][4] per-step max over blocks of (operator end, solver end,
                                     // chunk ready->solved, last row block complete), ns
};

namespace {

// bounded grid barrier; returns false on timeout, or as soon as another block
// has raised the error flag (all CTAs then return)
__device__ bool grid_barrier(const SimParams& p, uint64_t deadline_ns) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = p.bar_gen;
        const unsigned my_gen = *gen;
        __threadfence();
        const unsigned prev = atomicAdd(p.bar_count, 1u);
        int ok = 1;
        if (prev == (unsigned)p.nblk - 1) {
            atomicExch(p.bar_count, 0u);
            __threadfence();
            atomicAdd((unsigned*)p.bar_gen, 1u);
        } else {
            while (*gen == my_gen) {
                if (globaltimer_ns() > deadline_ns + 2000000000ull || *(volatile int*)p.gerr != 0) {
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (!ok) atomicExch(p.gerr, QDFN_ERR_TIMEOUT);
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Order-preserving map of doubles to unsigned 64-bit keys (sign bit flipped
// for x >= 0, all bits inverted for x < 0): min/max of keys is min/max of the
// values, on the integer pipe.  The FP64 pipe of this part is ~64x narrower
// than FP32, and these reductions run twice per step.  The reduced fields
// never hold NaN (a NaN velocity is carried by its own flag field), so the
// result equals fmin/fmax; the order of +0/-0 is -0 < +0.
__device__ __forceinline__ unsigned long long ord_key(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return b ^ ((unsigned long long)((long long)b >> 63) | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_val(unsigned long long k) {
    const unsigned long long b = (k & 0x8000000000000000ull) ? (k ^ 0x8000000000000000ull) : ~k;
    return __longlong_as_double((long long)b);
}
__device__ __forceinline__ unsigned long long key_op(int op, unsigned long long a, unsigned long long b) {
    return op == 0 ? (a > b ? a : b) : (a < b ? a : b);
}

// block-wide reduction of R*K doubles with op (0 = max, 1 = min)
template <int K>
__device__ void block_reduce(double (&v)[kMaxInst][K], const int (&ops)[K], int R) {
    __shared__ unsigned long long s_buf[kSimThreads / 32][kMaxInst][K];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int k = 0; k < K; ++k) {
            unsigned long long x = ord_key(v[r][k]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x = key_op(ops[k], x, __shfl_xor_sync(0xffffffffu, x, o));
            if (lane == 0) s_buf[wid][r][k] = x;
        }
    __syncthreads();
    // across warps: one thread per (instance, field), then thread 0 gathers
    __shared__ unsigned long long s_out[kMaxInst][K];
    if (threadIdx.x < R * K) {
        const int r = threadIdx.x / K, k = threadIdx.x % K;
        unsigned long long x = s_buf[0][r][k];
        for (int w = 1; w < kSimThreads / 32; ++w) x = key_op(ops[k], x, s_buf[w][r][k]);
        s_out[r][k] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int k = 0; k < K; ++k) v[r][k] = ord_val(s_out[r][k]);
    __syncthreads();
}

// Reduce K fields of every CTA's partial for instance r (slot layout of
// SimParams::red) across the grid: one warp, lanes stride over the CTAs, then
// a shuffle tree.  Every lane returns the result.  min/max only: exact, so the
// result does not depend on the order.
template <int K>
__device__ __forceinline__ void grid_fields(const double* slots_base, int nblk, int R, int r,
                                            const int (&ops)[K], double (&out)[K]) {
    const int lane = threadIdx.x & 31;
    unsigned long long acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = ord_key(ops[k] == 0 ? -INFINITY : INFINITY);
#pragma unroll 2
    for (int b = lane; b < nblk; b += 32) {   // (two blocks' slots in flight per lane)
        const double* s = slots_base + ((int64_t)b * R + r) * kRedSlots;
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] = key_op(ops[k], acc[k], ord_key(__ldcg(s + k)));
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] = key_op(ops[k], acc[k], __shfl_xor_sync(0xffffffffu, acc[k], o));
        out[k] = ord_val(acc[k]);
    }
}

// ---------------------------------------------------------------------------
// P2: dense elastic operator.
//
// Storage is tile-contiguous: receivers in row blocks of kSimThreads*VEC (one
// 8-byte granule per thread and source column, 4 KB per column), and within a
// row block the source columns back to back (see k_convert).  A tile is (row
// block, chunk of source columns); tiles are handed out by a global counter.
// Both matrices stream through a kStages-deep ring of 64 KB shared-memory
// stages, each filled by one 32 KB TMA bulk copy per matrix
// (cp.async.bulk ... mbarrier::complete_tx) issued by one thread, so the bytes
// in flight do not depend on the register-limited warp count of the
// persistent kernel.  x = D (all R instances) is staged per tile.  FP32/BF16
// products are summed in FP32 over 32 columns and folded error-free into
// (hi, lo) FP32 pairs; FP64 storage accumulates in FP64.
constexpr int kOpWarps = 8;                                     // operator role: warps [0, kOpWarps)
constexpr int kOpThreads = kOpWarps * 32;
constexpr int kProducerWarp = kSimThreads / 32 - 1;             // lane 0 fills the stage ring
constexpr int kStages = 3;
// FP32/BF16 steps that stream ahead: the solver warps [kOpWarps, kProducerWarp)
// run the step's first reduction pass and its grid barrier on their own
// (named barrier 1) while the operator warps and the producer finish the early
// tiles; everyone meets afterwards
constexpr int kSolverWarps = kProducerWarp - kOpWarps;
constexpr int kSolverThreads = kSolverWarps * 32;
__device__ __forceinline__ void solver_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kSolverThreads) : "memory"); }
// early-tile counter: closed (no further claims) once the step's solves are in
constexpr unsigned long long kSpecClosed = 1ull << 62;

// The same barrier for the solver warps of each block alone (named barrier 1;
// thread kOpThreads arrives for the block).  Every solver thread gets the same
// result.  The last block to arrive closes the early-tile counter `close`
// before it releases the others, so the number of early tiles is final for
// every block that leaves the barrier.
__device__ bool grid_barrier_solvers(const SimParams& p, uint64_t deadline_ns, unsigned long long* close) {
    __shared__ int s_ok;
    solver_sync();
    if (threadIdx.x == kOpThreads) {
        volatile unsigned* gen = p.bar_gen;
        const unsigned my_gen = *gen;
        __threadfence();
        const unsigned prev = atomicAdd(p.bar_count, 1u);
        int ok = 1;
        if (prev == (unsigned)p.nblk - 1) {
            atomicOr(close, kSpecClosed);
            atomicExch(p.bar_count, 0u);
            __threadfence();
            atomicAdd((unsigned*)p.bar_gen, 1u);
        } else {
            while (*gen == my_gen) {
                if (globaltimer_ns() > deadline_ns + 2000000000ull || *(volatile int*)p.gerr != 0) {
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (!ok) atomicExch(p.gerr, QDFN_ERR_TIMEOUT);
        s_ok = ok;
    }
    solver_sync();
    return s_ok != 0;
}

constexpr int kColsPerStage = 16;
constexpr int kFoldStages = 32 / kColsPerStage;                 // FP32 sums span 32 columns
constexpr int kSegBytes = kOpThreads * kGranule;                // one column of a row block, 2 KB
constexpr int kStageBytes = 2 * kColsPerStage * kSegBytes;      // E and Kn, 64 KB
constexpr int kPipeBytes = kStages * kStageBytes;               // 192 KB
constexpr int kMbarBytes = 128;
constexpr uint64_t kWaitLimitNs = 2000000000ull;                // 2 s per stage wait

__device__ __forceinline__ uint32_t smem_u32(const void* ptr) {
    return (uint32_t)__cvta_generic_to_shared(ptr);
}
__device__ __forceinline__ void mbar_init(uint64_t* m, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* m, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes)
                 : "memory");
}
// L2 policy for data read once per step (the operator stream): evict first,
// so that what the step re-reads (chunk partials, state) stays in L2
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* m,
                                         uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], "
        "%4;" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(m)), "l"(pol)
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* m, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(m)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait on a stage; false when the limit passes
__device__ __forceinline__ bool mbar_wait(uint64_t* m, uint32_t parity, uint64_t limit_ns) {
    if (mbar_try_wait(m, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait(m, parity))
        if (globaltimer_ns() - t0 > limit_ns) return false;
    return true;
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// orders this thread's generic-proxy global writes (the x copy of D) with
// later bulk-copy (async-proxy) reads of them
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* ptr) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(ptr) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* ptr) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ptr) : "memory");
    return v;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* m) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(m)) : "memory");
}

// Descriptor of the stage held by a ring slot.  The producer writes it before
// the arrival that completes the slot's "full" barrier (release), consumers
// read it after waiting on that barrier (acquire).
struct StageDesc {
    long long tile;   // operator tile, or -1: no tiles left (end marker)
    int q, nst;       // stage index within the tile, stages of the tile
    int seq;          // tile sequence number in this CTA (selects the x buffer)
    int next;         // 1: a tile of the next step (streamed ahead)
};
static_assert(6 * 8 + kStages * sizeof(StageDesc) <= kMbarBytes, "mbarriers + stage descriptors");

// Pipeline state of one CTA: stage memory, the "full" mbarriers (completed by
// the bulk copies' byte count), the "empty" mbarriers (one arrival per operator
// warp once it has read the stage), the stage descriptors, and the running
// stage counts.  `consumed` is identical in every operator thread; the
// producer fields are used by thread 0 alone.  The ring keeps running across
// tiles (the producer walks into the next tile as soon as a slot frees up) and
// across steps.
struct Pipe {
    unsigned char* stages;
    uint64_t* full;
    uint64_t* empty;
    StageDesc* desc;
    uint32_t consumed;
    // producer (thread 0)
    uint32_t filled;
    long long ftile;         // tile being filled; -2 none yet, -1 no tiles left
    int fq, fnst, fseq;      // its next stage, its stage count, its sequence number
    int fphase, fnext;       // 0 this step's tiles, 1 the next step's, 2 done; the tile's step
    uint32_t last_stage[2];  // last stage of the latest tile using each x buffer
};
constexpr uint32_t kNoStage = 0xffffffffu;

__device__ __forceinline__ void pipe_init(Pipe& pp, unsigned char* smem) {
    pp.stages = smem;
    pp.full = reinterpret_cast<uint64_t*>(smem + kPipeBytes);
    pp.empty = pp.full + kStages;
    pp.desc = reinterpret_cast<StageDesc*>(pp.full + 2 * kStages);
    pp.consumed = 0;
    pp.filled = 0;
    pp.ftile = -2;
    pp.fq = pp.fnst = 0;
    pp.fseq = -1;
    pp.fphase = 0;
    pp.fnext = 0;
    pp.last_stage[0] = pp.last_stage[1] = kNoStage;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(pp.full + s, 1);
            mbar_init(pp.empty + s, kOpWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
}

// error-free accumulation of an FP32 partial sum into an unevaluated pair
// hi + lo (Knuth's TwoSum: the rounding error of hi + p is recovered exactly
// and gathered in lo).  Six FP32 additions replace two FP64 ones: on this part
// the FP64 pipe is ~64x narrower than FP32, and the fold runs once per 32
// source columns for every row and instance.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float p) {
    const float s = hi + p;
    const float bp = s - hi;
    const float err = (hi - (s - bp)) + (p - bp);
    hi = s;
    lo += err;
}

// the R staged x values of one source column (stored contiguously, 16-byte
// aligned when R * sizeof(X) is a multiple of 16)
template <class X, int R>
__device__ __forceinline__ void xload(const X* p, X x[R]) {
    if constexpr (R * sizeof(X) % 16 == 0) {
#pragma unroll
        for (int k = 0; k < (int)(R * sizeof(X) / 16); ++k) {
            const uint4 q = reinterpret_cast<const uint4*>(p)[k];
            memcpy(reinterpret_cast<unsigned char*>(x) + 16 * k, &q, 16);
        }
    } else if constexpr (R * sizeof(X) == 8) {
        const uint2 q = *reinterpret_cast<const uint2*>(p);
        memcpy(x, &q, 8);
    } else {
#pragma unroll
        for (int r = 0; r < R; ++r) x[r] = p[r];
    }
}

// Sum of the column-chunk partials of row (instance r, receiver i), in chunk
// order (deterministic).  FP64 storage: the partials are doubles, summed in
// FP64.  FP32/BF16 storage (kPairs): each partial is the tile's (hi, lo) FP32
// pair; the hi parts are gathered error-free with TwoSum and the lo parts
// added, all on the FP32 pipe, and the pair becomes a double once per row.
// Loads are issued in batches (16 chunks per matrix, 8 when one lane sums
// both; past the last chunk a batch re-reads it and skips the sum), so every
// batch costs one memory round trip.
__device__ __forceinline__ int chunks_of_rb(const SimParams& p, int64_t rb) {
    return rb >= p.rb_small0 ? p.nchunk2 : p.nchunk;
}

// Rows of one solve chunk of the overlapped phase: 16 on lane pairs, 32 with
// one lane per patch.
__device__ __forceinline__ int solve_rows(const SimParams& p) { return p.pair_solve == 2 ? 32 : 16; }

// The state and constants of one solve chunk (rows i0..i0+rows-1 of instance
// r, rows 16 or 32) toward L1, issued by the claiming warp before it waits for
// the chunk's row block: 17 arrays, the 128-byte lines that the run can span
// (its first, middle and last element), one or two prefetches per lane.  The
// chunk's loads in solve_item then find their lines close instead of forming
// a chain of round trips behind the partial sums.  Hints only; the addresses
// stay inside the arrays (the last row is clamped to N - 1).
__device__ __forceinline__ void prefetch_chunk(const SimParams& p, int par, int r, int64_t i0, int rows) {
    const int lane = threadIdx.x & 31;
    const int64_t N = p.N;
    const int64_t ie = min(i0 + rows - 1, N - 1);
    const int64_t im = min(i0 + rows / 2, N - 1);
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const int slot = lane + 32 * t;
        const int a = slot / 3, l = slot % 3;
        if (a >= 17) continue;
        const int64_t e = l == 0 ? i0 : (l == 1 ? im : ie);   // first, middle or last element of the run
        const int64_t q = (int64_t)r * N + e;
        const void* ptr;
        switch (a) {
            case 0: ptr = (par ? p.Vn : p.V) + q; break;
            case 1: ptr = (par ? p.Dn : p.D) + q; break;
            case 2: ptr = (par ? p.fn : p.fric) + q; break;
            case 3: ptr = (par ? p.thn : p.theta) + q; break;
            case 4: ptr = (par ? p.sn : p.sig_old) + q; break;
            case 5: ptr = p.F0 + q; break;
            case 6: ptr = p.a + q; break;
            case 7: ptr = p.b + q; break;
            case 8: ptr = p.Dc + q; break;
            case 9: ptr = p.omega + q; break;
            case 10: ptr = p.rDc + q; break;
            case 11: ptr = p.ra + q; break;
            case 12: ptr = p.mass + q; break;
            case 13: ptr = p.sigma0 + q; break;
            case 14: ptr = p.tau0 + q; break;
            case 15: ptr = p.kself + e; break;
            default: ptr = (par ? p.sw_n : p.sw) + q; break;
        }
        asm volatile("prefetch.global.L1 [%0];" ::"l"(ptr));
    }
}

// One matrix's half of sum_partials (side 0 shear, 1 normal), for a lane pair
// that splits the two sums between its lanes; same order and arithmetic.
template <bool kPairs>
__device__ __forceinline__ double sum_partials_side(const SimParams& p, int r, int64_t i, int side, int ppar) {
    const int64_t cs = (int64_t)p.R * p.N;
    const int64_t base = (int64_t)ppar * p.part_stride + (int64_t)r * p.N + i;
    const int nch = chunks_of_rb(p, i / p.ld);
    const double* part = side == 0 ? p.part_s : p.part_n;
    if constexpr (kPairs) {
        const float2* ps = reinterpret_cast<const float2*>(part) + base;
        float h = 0.f, l = 0.f;
        for (int c = 0; c < nch; c += 16) {
            float2 t[16];
#pragma unroll
            for (int k = 0; k < 16; ++k) t[k] = __ldcg(ps + min(c + k, nch - 1) * cs);
#pragma unroll
            for (int k = 0; k < 16; ++k)
                if (c + k < nch) { two_sum_acc(h, l, t[k].x); l += t[k].y; }
        }
        return (double)h + (double)l;
    } else {
        const double* ps = part + base;
        double a = 0;
        for (int c = 0; c < nch; c += 16) {
            double t[16];
#pragma unroll
            for (int k = 0; k < 16; ++k) t[k] = __ldcg(ps + min(c + k, nch - 1) * cs);
#pragma unroll
            for (int k = 0; k < 16; ++k)
                if (c + k < nch) a += t[k];
        }
        return a;
    }
}

template <bool kPairs>
__device__ __forceinline__ void sum_partials(const SimParams& p, int r, int64_t i, double& ss, double& sn,
                                             int ppar = 0) {
    const int64_t cs = (int64_t)p.R * p.N;
    const int64_t base = (int64_t)ppar * p.part_stride + (int64_t)r * p.N + i;
    const int nch = chunks_of_rb(p, i / p.ld);
    if constexpr (kPairs) {
        const float2* ps = reinterpret_cast<const float2*>(p.part_s) + base;
        const float2* pn = reinterpret_cast<const float2*>(p.part_n) + base;
        float hs = 0.f, ls = 0.f, hn = 0.f, ln = 0.f;
        for (int c = 0; c < nch; c += 8) {
            float2 ts[8], tn[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int cc = min(c + k, nch - 1);   // (past the end: a repeat, not summed)
                ts[k] = __ldcg(ps + cc * cs);
                tn[k] = __ldcg(pn + cc * cs);
            }
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (c + k < nch) {
                    two_sum_acc(hs, ls, ts[k].x); ls += ts[k].y;
                    two_sum_acc(hn, ln, tn[k].x); ln += tn[k].y;
                }
        }
        ss = (double)hs + (double)ls;
        sn = (double)hn + (double)ln;
    } else {
        const double* ps = p.part_s + base;
        const double* pn = p.part_n + base;
        double as = 0, an = 0;
        for (int c = 0; c < nch; c += 8) {
            double ts[8], tn[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int cc = min(c + k, nch - 1);   // (past the end: a repeat, not summed)
                ts[k] = __ldcg(ps + cc * cs);
                tn[k] = __ldcg(pn + cc * cs);
            }
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (c + k < nch) { as += ts[k]; an += tn[k]; }
        }
        ss = as;
        sn = an;
    }
}

// Operator tile geometry: tile index -> (row block, column chunk, first
// column, column count, stage count).  Row-block-major; the row blocks from
// rb_small0 on use the half-width chunks.
struct TileGeo {   // 32-bit: N < 2^31
    int rb, c, j0, L, nst;
};
__device__ __forceinline__ TileGeo tile_geo(const SimParams& p, int64_t nrb, int64_t tile) {
    const int64_t nrb_big = min(p.rb_small0, nrb);
    const int64_t T1 = nrb_big * p.nchunk;
    TileGeo g;
    int64_t clen;
    if (tile < T1) { g.rb = (int)(tile / p.nchunk); g.c = (int)(tile % p.nchunk); clen = p.chunk_len; }
    else { g.rb = (int)(nrb_big + (tile - T1) / p.nchunk2); g.c = (int)((tile - T1) % p.nchunk2); clen = p.chunk_len2; }
    g.j0 = (int)(g.c * clen);
    g.L = (int)(min(p.N, (int64_t)g.j0 + clen) - g.j0);
    g.nst = (g.L + kColsPerStage - 1) / kColsPerStage;
    return g;
}

// What the producer and the operator warps need to know about a step.
struct StepCtx {
    int set, set_next;        // counter sets of this step and the next (mod kSets)
    int ppar;                 // partial buffer of this step; the next step's is ppar ^ 1
    const void* xcur;         // x copy of D read by this step's tiles
    const void* xnext;        // x copy the next step's tiles read (written by this step's solves)
    long long spec_done;      // this step's tiles already streamed during the step before
    int spec;                 // after this step's tiles, stream the next step's first column chunks
    uint64_t t0;              // %globaltimer at the block's start of the phase (diagnostics)
    const unsigned short* order;   // row-block order of the step's tiles (null: index order)
};

// Tile index of column chunk c of row block rb (the inverse of tile_geo).
__device__ __forceinline__ long long tile_index(const SimParams& p, int64_t nrb, int64_t rb, int64_t c) {
    const int64_t nrb_big = min(p.rb_small0, nrb);
    return rb < nrb_big ? rb * p.nchunk + c : nrb_big * p.nchunk + (rb - nrb_big) * p.nchunk2 + c;
}

// Row-block order of a step (warp 0 of each block, the same in every block):
// among the full-width row blocks, and among the narrow-tile ones after them,
// the blocks holding a patch that starts the step on the high-velocity solver
// come first, each group in index order.  Their solves take several times
// longer than the others (tens of secant iterations), so they should start
// early in the stream rather than finish after it.  The order only decides
// when tiles and row chunks are taken, not what they compute.
constexpr int kMaxOrder = 256;
__device__ void rb_order(const SimParams& p, int set, unsigned short* order) {
    const int lane = threadIdx.x & 31;
    const int nrb = (int)p.n_rb, s0 = (int)min(p.rb_small0, (int64_t)nrb);
    const unsigned* hot = p.rb_hot + (int64_t)set * p.rb_stride;
    // the flags of row blocks lane + 32 j, loaded at once (nrb <= kMaxOrder)
    unsigned bits = 0;
#pragma unroll
    for (int j = 0; j < kMaxOrder / 32; ++j) {
        const int b = lane + 32 * j;
        if (b < nrb && __ldcg(hot + b) != 0u) bits |= 1u << j;
    }
    int pos = 0;
    for (int grp = 0; grp < 2; ++grp) {
        const int lo = grp ? s0 : 0, hi = grp ? nrb : s0;
        for (int want = 1; want >= 0; --want)
            for (int j = lo / 32; j * 32 < hi; ++j) {
                const int b = lane + 32 * j;
                const bool take = b >= lo && b < hi && (((bits >> j) & 1u) == (unsigned)want);
                const unsigned m = __ballot_sync(0xffffffffu, take);
                if (take) order[pos + __popc(m & ((1u << lane) - 1u))] = (unsigned short)b;
                pos += __popc(m);
            }
    }
}

// Tiles of the next step streamed during a step's tail: column chunks
// c < min(c_spec, nchunk) of the full-width row blocks, column-major
// (u -> rb = u % nrb_reg, c = u / nrb_reg), so the x they need -- the slip of
// the first patches, solved early in the step -- is ready first.
__device__ __forceinline__ void spec_shape(const SimParams& p, int64_t nrb, int64_t* nrb_reg, int64_t* n_spec) {
    *nrb_reg = min(p.rb_small0, nrb);
    *n_spec = (int64_t)min(p.c_spec, p.nchunk) * *nrb_reg;
}

// Zero counter set s (tile and early-tile counters, solve chunk counter,
// row-block completion and solved-chunk counts, diagnostics maxima and, with
// `hot`, the row-block order flags).  Called by every thread of one block, with
// no other block using the set.
__device__ __forceinline__ void reset_counter_set(const SimParams& p, int s, bool hot, int tid, int nthr) {
    if (tid == 0) {
        atomicExch(p.tile_ctr + s, 0ull);
        atomicExch(p.spec_ctr + s, 0ull);
        atomicExch(p.solve_ctr + s, 0ull);
    }
    unsigned* a = p.rb_done + (int64_t)s * p.rb_stride;
    unsigned* b = p.rb_solved + (int64_t)s * p.rb_stride;
    unsigned* h = p.rb_hot + (int64_t)s * p.rb_stride;
    for (int64_t k = tid; k < p.n_rb; k += nthr) {
        a[k] = 0u;
        b[k] = 0u;
        if (hot) h[k] = 0u;
    }
    if (tid < 4) p.tmax[s * 4 + tid] = 0ull;
}

// Claim the next early tile: its index, or -1 once n are claimed, the counter
// is closed (every block's solves are in), or p.spec_stop blocks have arrived
// at the step's barrier (a tile claimed later would still be streaming when
// the step is decided and hold its block's next step back).  A compare-and-swap, so
// a closed counter keeps the number of tiles claimed; bounded -- a tile left
// unclaimed is streamed by its own step.
__device__ __forceinline__ long long claim_spec(const SimParams& p, unsigned long long* ctr, int64_t n) {
    if (*(volatile unsigned*)p.bar_count >= (unsigned)p.spec_stop) return -1;
    unsigned long long v = ld_acquire_u64(ctr);
    for (int k = 0; k < 256; ++k) {
        if ((v & kSpecClosed) != 0 || (long long)v >= (long long)n) return -1;
        const unsigned long long w = atomicCAS(ctr, v, v + 1);
        if (w == v) return (long long)v;
        v = w;
    }
    return -1;
}

// Producer (one lane): fill the next stage of the ring -- the next stage of the
// tile being filled, else the first stage of the next tile: this step's tiles
// from the global counter (skipping those streamed during the step before),
// then, when the step streams ahead, the next step's first column chunks once
// the slip they read is solved, then the end marker.  A tile's first stage
// also carries its x chunk, from the instance-interleaved copy of D.  Returns
// false when a bounded wait ran out.
template <class M, int R>
__device__ __forceinline__ bool produce_stage(const SimParams& p, Pipe& pp, typename M::X* xs, int64_t nrb,
                                              int64_t ntiles, uint64_t pol, const StepCtx& sc) {
    using X = typename M::X;
    constexpr int VEC = M::VEC;
    constexpr int EB = kGranule / VEC;   // bytes per stored entry
    constexpr int64_t rows_per_blk = (int64_t)kOpThreads * VEC;
    const uint32_t n = pp.filled;
    const int slot = (int)(n % kStages);
    // the stage this slot held last must be released by every operator warp
    if (n >= (uint32_t)kStages && !mbar_wait(pp.empty + slot, ((n - kStages) / kStages) & 1u, kWaitLimitNs))
        return false;
    if (pp.ftile == -2 || (pp.ftile >= 0 && pp.fq >= pp.fnst)) {
        int64_t nrb_reg, n_spec;
        spec_shape(p, nrb, &nrb_reg, &n_spec);
        pp.ftile = -1;
        while (pp.fphase < 2) {
            if (pp.fphase == 0) {            // this step
                // the step's own tiles: every tile but the sc.spec_done early
                // ones (column-major prefix over the full-width row blocks:
                // chunks c < cfull of each, and chunk cfull of row blocks < rem),
                // row block after row block in the step's order
                const long long k = (long long)atomicAdd(p.tile_ctr + sc.set, 1ull);
                if (k >= ntiles - sc.spec_done) { pp.fphase = (sc.spec && n_spec > 0) ? 1 : 2; continue; }
                const int64_t cfull = nrb_reg > 0 ? sc.spec_done / nrb_reg : 0;
                const int64_t rem = nrb_reg > 0 ? sc.spec_done % nrb_reg : 0;
                long long t = -1, left = k;
                for (int64_t pos = 0; pos < nrb; ++pos) {
                    const int64_t rb = sc.order ? (int64_t)sc.order[pos] : pos;
                    const int64_t c0 = rb < nrb_reg ? cfull + (rb < rem ? 1 : 0) : 0;
                    const int64_t cnt = (rb < nrb_reg ? p.nchunk : p.nchunk2) - c0;
                    if (left < cnt) { t = tile_index(p, nrb, rb, c0 + left); break; }
                    left -= cnt;
                }
                if (t < 0) { pp.fphase = (sc.spec && n_spec > 0) ? 1 : 2; continue; }   // (not reached)
                pp.ftile = t;
                pp.fnext = 0;
                break;
            }
            // the next step (fphase 1)
            const long long u = claim_spec(p, p.spec_ctr + sc.set_next, n_spec);
            if (u < 0) { pp.fphase = 2; continue; }
            const int64_t rb = u % nrb_reg, c = u / nrb_reg;
            const long long t = rb * p.nchunk + c;
            // its x chunk: the slip of patches [j0, j0 + L), solved in this step
            const TileGeo g = tile_geo(p, nrb, t);
            const unsigned need = (unsigned)(R * (rows_per_blk / solve_rows(p)));   // solve chunks per row block
            const uint64_t t0 = globaltimer_ns();
            for (int64_t b = g.j0 / rows_per_blk; b <= (int64_t)(g.j0 + g.L - 1) / rows_per_blk; ++b)
                while (ld_acquire_u32(p.rb_solved + sc.set * p.rb_stride + b) < need) {
                    if (globaltimer_ns() - t0 > kWaitLimitNs || *(volatile int*)p.gerr != 0) return false;
                    __nanosleep(200);
                }
            fence_proxy_async_global();
            pp.ftile = t;
            pp.fnext = 1;
            break;
        }
        if (pp.ftile >= 0) {
            pp.fq = 0;
            pp.fnst = tile_geo(p, nrb, pp.ftile).nst;
            pp.fseq++;
        }
    }
    StageDesc* d = pp.desc + slot;
    uint64_t* m = pp.full + slot;
    if (pp.ftile == -1) {              // end marker: completes the phase without bytes
        d->tile = -1;
        mbar_arrive(m);
        pp.filled = n + 1;
        return true;
    }
    const TileGeo g = tile_geo(p, nrb, pp.ftile);
    const int q = pp.fq;
    const int xb = pp.fseq & 1;
    if (q == 0) {
        // the x buffer was last read by the tile before the previous one; its
        // last stage is released already unless that was within kStages stages
        const uint32_t prev = pp.last_stage[xb];
        if (prev != kNoStage && prev + kStages > n &&
            !mbar_wait(pp.empty + (prev % kStages), (prev / kStages) & 1u, kWaitLimitNs))
            return false;
    }
    d->tile = pp.ftile;
    d->q = q;
    d->nst = g.nst;
    d->seq = pp.fseq;
    d->next = pp.fnext;
    const int nc = (int)min((int64_t)kColsPerStage, g.L - (int64_t)q * kColsPerStage);
    const uint32_t bytes = (uint32_t)nc * kSegBytes;
    // x: the tile's columns rounded up to 4 (the copy is padded past N)
    const uint32_t xbytes = q == 0 ? (uint32_t)(((g.L + 3) / 4 * 4) * R * sizeof(X)) : 0u;
    fence_proxy_async();
    mbar_expect_tx(m, 2u * bytes + xbytes);
    unsigned char* st = pp.stages + (size_t)slot * kStageBytes;
    // tile-contiguous layout: the nc columns of this row block are one run of
    // nc * kSegBytes in each matrix -> one bulk copy per matrix
    const int64_t off = (((int64_t)g.rb * p.N + g.j0 + (int64_t)q * kColsPerStage) * rows_per_blk) * EB;
    bulk_g2s(st, reinterpret_cast<const unsigned char*>(p.E) + off, bytes, m, pol);
    bulk_g2s(st + (size_t)kColsPerStage * kSegBytes, reinterpret_cast<const unsigned char*>(p.Kn) + off, bytes, m,
             pol);
    if (q == 0) {
        const X* xsrc = reinterpret_cast<const X*>(pp.fnext ? sc.xnext : sc.xcur);
        bulk_g2s(xs + (size_t)xb * p.xbuf, xsrc + (int64_t)g.j0 * R, xbytes, m, pol);
    }
    if (q == g.nst - 1) pp.last_stage[xb] = n;
    pp.fq = q + 1;
    pp.filled = n + 1;
    return true;
}

// Producer role (one lane of warp kProducerWarp): walk this step's tiles (and
// the next step's first column chunks when the step streams ahead) and keep
// the ring full -- every fill waits only for the release of the slot's
// previous stage by the operator warps -- until the end marker is issued.  On
// a failed wait it drains the copies it issued (bounded) and returns false.
template <class M, int R>
__device__ bool produce_tiles(const SimParams& p, Pipe& pp, typename M::X* xs, const StepCtx& sc) {
    constexpr int64_t rows_per_blk = (int64_t)kOpThreads * M::VEC;
    const int64_t nrb = (p.N + rows_per_blk - 1) / rows_per_blk;
    const int64_t ntiles = min(p.rb_small0, nrb) * p.nchunk + (nrb - min(p.rb_small0, nrb)) * p.nchunk2;
    const uint64_t pol = l2_evict_first_policy();
    fence_proxy_async_global();
    pp.ftile = -2;
    pp.fphase = 0;
    do {
        if (!produce_stage<M, R>(p, pp, xs, nrb, ntiles, pol, sc)) {
            atomicExch(p.gerr, QDFN_ERR_TIMEOUT);
            const uint32_t from = pp.filled > (uint32_t)kStages ? pp.filled - kStages : 0u;
            for (uint32_t k = from; k < pp.filled; ++k)
                mbar_wait(pp.full + (k % kStages), (k / kStages) & 1u, kWaitLimitNs);
            return false;
        }
    } while (pp.ftile != -1);
    return true;
}

// Operator role (warps [0, kOpWarps)): consume the stage ring tile after tile.
// Each thread owns VEC receiver rows of the current tile's row block and
// accumulates the products of all R instances; at a tile's last stage it
// writes its partials, and each warp then counts itself into the row block's
// completion counter (kOpWarps arrivals per tile).
template <class M, int R>
__device__ bool dense_matvec(const SimParams& p, Pipe& pp, typename M::X* xs, const StepCtx& sc) {
    using X = typename M::X;
    constexpr int VEC = M::VEC;
    constexpr int64_t rows_per_blk = (int64_t)kOpThreads * VEC;
    const int64_t N = p.N;
    const int64_t nrb = (N + rows_per_blk - 1) / rows_per_blk;
    bool ok = true;
    // FP64 storage: fs/fn are the accumulators.  FP32 storage: fs/fn sum
    // kFoldStages stages, then fold error-free into the pairs (h, l).
    X fs[R][VEC], fn[R][VEC];
    float hs[R][VEC], ls[R][VEC], hn[R][VEC], ln[R][VEC];
    TileGeo g{};
    int64_t i0 = 0;
    const X* xsb = xs;
    while (ok) {
        const uint32_t n = pp.consumed;
        const int slot = (int)(n % kStages);
        if (!mbar_wait(pp.full + slot, (n / kStages) & 1u, kWaitLimitNs)) { ok = false; break; }
        const StageDesc d = pp.desc[slot];
        if (d.q == 0 && d.tile >= 0) {   // a new tile
            g = tile_geo(p, nrb, d.tile);
            i0 = (int64_t)g.rb * rows_per_blk + (int64_t)threadIdx.x * VEC;
            xsb = xs + (size_t)(d.seq & 1) * p.xbuf;
#pragma unroll
            for (int r = 0; r < R; ++r)
#pragma unroll
                for (int v = 0; v < VEC; ++v) {
                    fs[r][v] = 0; fn[r][v] = 0;
                    hs[r][v] = 0.f; ls[r][v] = 0.f; hn[r][v] = 0.f; ln[r][v] = 0.f;
                }
        }
        if (d.tile >= 0 && i0 < N) {
            const int q = d.q;
            const int nc = (int)min((int64_t)kColsPerStage, g.L - (int64_t)q * kColsPerStage);
            const unsigned char* st = pp.stages + (size_t)slot * kStageBytes + (size_t)threadIdx.x * kGranule;
#pragma unroll
            for (int cc = 0; cc < kColsPerStage; ++cc) {
                if (cc < nc) {
                    X e[VEC], k[VEC], x[R];
                    M::sload(st + (size_t)cc * kSegBytes, e);
                    M::sload(st + (size_t)(kColsPerStage + cc) * kSegBytes, k);
                    xload<X, R>(xsb + ((int64_t)q * kColsPerStage + cc) * R, x);
#pragma unroll
                    for (int r = 0; r < R; ++r)
#pragma unroll
                        for (int v = 0; v < VEC; ++v) {
                            fs[r][v] = fma(e[v], x[r], fs[r][v]);
                            fn[r][v] = fma(k[v], x[r], fn[r][v]);
                        }
                }
            }
            if constexpr (sizeof(X) == 4) {
                if ((q + 1) % kFoldStages == 0 || q == d.nst - 1) {
#pragma unroll
                    for (int r = 0; r < R; ++r)
#pragma unroll
                        for (int v = 0; v < VEC; ++v) {
                            two_sum_acc(hs[r][v], ls[r][v], (float)fs[r][v]);
                            two_sum_acc(hn[r][v], ln[r][v], (float)fn[r][v]);
                            fs[r][v] = 0;
                            fn[r][v] = 0;
                        }
                }
            }
        }
        // release the slot: one arrival per warp; the producer refills it once
        // every warp has arrived, the other warps run ahead into filled stages
        __syncwarp();
        if ((threadIdx.x & 31) == 0) mbar_arrive(pp.empty + slot);
        pp.consumed = n + 1;
        if (d.tile < 0) break;             // end marker
        if (d.q == d.nst - 1) {            // the tile is complete: partials, then publish
            if (i0 < N) {
#pragma unroll
                for (int r = 0; r < R; ++r)
#pragma unroll
                    for (int v = 0; v < VEC; ++v) {
                        const int64_t i = i0 + v;
                        if (i < N) {
                            // the tile's step selects the partial buffer
                            const int64_t o = (int64_t)(sc.ppar ^ d.next) * p.part_stride +
                                              ((int64_t)g.c * R + r) * N + i;
                            if constexpr (sizeof(X) == 8) {
                                p.part_s[o] = fs[r][v];
                                p.part_n[o] = fn[r][v];
                            } else {   // the pair itself: no FP64 work in this phase
                                reinterpret_cast<float2*>(p.part_s)[o] = make_float2(hs[r][v], ls[r][v]);
                                reinterpret_cast<float2*>(p.part_n)[o] = make_float2(hn[r][v], ln[r][v]);
                            }
                        }
                    }
            }
            __threadfence();
            __syncwarp();
            if ((threadIdx.x & 31) == 0) {
                const unsigned old = atomicAdd(p.rb_done + (d.next ? sc.set_next : sc.set) * p.rb_stride + g.rb, 1u);
                // diagnostics: when the step's last row block became complete
                if (!d.next && sc.t0 != 0 && old + 1 == (unsigned)chunks_of_rb(p, g.rb) * kOpWarps)
                    atomicMax(p.tmax + sc.set * 4 + 3, (unsigned long long)(globaltimer_ns() - sc.t0));
            }
        }
    }
    if (!ok) {   // the producer drains the copies it issued
        atomicExch(p.gerr, QDFN_ERR_TIMEOUT);
        return false;
    }
    return true;
}

// Time control of the next step (Main_D :162-201) from the reduced statistics
// of the current state: max V and NaN flag over the controlled set, min |V/A|,
// whether any |V/A| was usable.  Returns the step size; *empty reports an
// empty minimum (Julia's `minimum` of an empty set).
__device__ __forceinline__ double next_dt(const SimParams& p, double vmax, double vnan, double dtmin, double any,
                                          double dt_prev, bool* empty) {
    *empty = (any == 0);
    if (vnan != 0) vmax = NAN;
    dtmin = dtmin / p.dt_cut;
    double DtRef;
    if (vmax > p.switch_v) DtRef = p.rupture_dt;
    else if (dtmin > p.max_dt) DtRef = p.max_dt;
    else DtRef = dtmin;
    double Dt = dt_prev;
    if (DtRef <= p.rupture_dt) Dt = DtRef;
    else if (Dt < DtRef / 1.2) Dt = Dt * 1.2;
    else Dt = DtRef;
    return Dt;
}

// The two state buffers of the step loop; `cur` holds the state at the start
// of a step, `nxt` receives the solves' results and becomes `cur` when the
// step is accepted.
struct StateView {
    double *V, *D, *theta, *fric, *accel, *sig_old;
    int* sw;
};
__device__ __forceinline__ StateView state_view(const SimParams& p, int which) {
    if (which == 0) return {p.V, p.D, p.theta, p.fric, p.accel, p.sig_old, p.sw};
    return {p.Vn, p.Dn, p.thn, p.fn, p.accel_n, p.sn, p.sw_n};
}

// The persistent loop of one context, run by its p.nblk blocks; `blk` is this
// block's index among them (blk for a single-context launch, the
// block's rank within its member for an ensemble launch).
template <class M, int R, bool HM>
__device__ __forceinline__ void sim_run(const SimParams& p, int64_t nsteps, const int blk) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    using X = typename M::X;
    // dense: [stage ring | mbarriers, stage descriptors | two x buffers];
    // H-matrix: [x | rank accumulators]
    X* xs = reinterpret_cast<X*>(HM ? smem_raw : smem_raw + kPipeBytes + kMbarBytes);
    double* hacc = reinterpret_cast<double*>(smem_raw + (size_t)R * hmat::kChunk * sizeof(X));
    Pipe pipe;
    if constexpr (!HM) pipe_init(pipe, smem_raw);
    // s_dt: Dt of the current step; s_dtn: the next step's, decided with the
    // reductions of the current one; s_dta: the last accepted Dt (what the
    // host keeps, and the next launch's controller starts from)
    __shared__ double s_T[kMaxInst], s_dt[kMaxInst], s_dtn[kMaxInst], s_dta[kMaxInst];
    __shared__ double s_rdt[kMaxInst];   // 1/s_dt, correctly rounded, formed before each solve pass
    __shared__ int64_t s_step[kMaxInst], s_nrec[kMaxInst];
    __shared__ int s_done[kMaxInst], s_fail[kMaxInst], s_stop, s_par;
    __shared__ int s_fill_stop, s_fill_counted;   // fill mode: every member has its nsteps; this one counted
    __shared__ int s_iter;
    // this block's reduction of a solve pass, as order-preserving keys (exact
    // min/max, integer pipe), one set per instance: [0] min flag, [1] min Dt,
    // [2] any instability 4, [3] min error; for the next step's time control
    // [4] max V, [5] V is NaN, [6] min |V/A|, [7] any |V/A| usable
    __shared__ unsigned long long s_red[kMaxInst][8];
    // each CTA measures the budget from its own start; the reductions make the
    // stop decision common to all CTAs
    const uint64_t deadline = globaltimer_ns() + p.budget_ns;
    // device counters kept by thread 0 in shared memory (no registers held
    // across the phases): [0..3] phases, [4..5] P3 split, [6..7] operator /
    // solver warps of the overlapped phase, [8..9] the same for the slowest
    // block of each step, [10] running mark, [11] P3 mark, [12..13] chunk maxima
    __shared__ unsigned long long s_tm[14];
    if (threadIdx.x < 14) s_tm[threadIdx.x] = 0;
    if (threadIdx.x == 0) s_tm[10] = globaltimer_ns();
    unsigned long long n_iter = 0, n_steps = 0;
    unsigned n_lo = 0, it_lo = 0, n_hi = 0, it_hi = 0;   // solves / secant iterations of this thread
    auto lap = [&](int k) {
        if (threadIdx.x == 0) { const uint64_t t = globaltimer_ns(); s_tm[k] += t - s_tm[10]; s_tm[10] = t; }
    };
    const int64_t N = p.N, Ns = p.N - p.Nload;
    const int64_t nthreads = (int64_t)p.nblk * kSimThreads;
    const int64_t gtid = (int64_t)blk * kSimThreads + threadIdx.x;
    int phase = 0;  // parity selector of the reduction buffer
    if (threadIdx.x < R) {
        s_T[threadIdx.x] = p.T[threadIdx.x];
        s_dt[threadIdx.x] = p.dt[threadIdx.x];
        s_dta[threadIdx.x] = p.dt[threadIdx.x];
        s_step[threadIdx.x] = p.step[threadIdx.x];
        s_nrec[threadIdx.x] = p.nrec[threadIdx.x];
        s_fail[threadIdx.x] = p.status[threadIdx.x];
    }
    if (threadIdx.x == 0) { s_stop = 0; s_par = 0; s_fill_stop = 0; s_fill_counted = 0; }
    // fill mode: whether every member has taken its nsteps (read into each
    // block's reduction slot, so that the member's blocks decide together)
    auto fill_seen = [&](int64_t it) -> double {
        if (p.fill_ctr == nullptr || it + 1 < nsteps) return 0.0;
        return *(volatile unsigned*)p.fill_ctr >= p.fill_need ? 1.0 : 0.0;
    };
    auto red_slot = [&](int ph, int64_t blk, int r) -> double* {
        return p.red + (((int64_t)(ph & 1) * p.nblk + blk) * R + r) * kRedSlots;
    };
    auto red_init = [&]() {
        if (threadIdx.x < R * 8) {
            const int k = threadIdx.x % 8;
            // neutral elements: min fields +inf, max fields -inf (flags start at 1 / 0)
            const double v0[8] = {1.0, INFINITY, 0.0, 0.0, -INFINITY, 0.0, INFINITY, 0.0};
            s_red[threadIdx.x / 8][k] = ord_key(v0[k]);
        }
    };
    auto red_min = [&](int r, int k, double x) { atomicMin(&s_red[r][k], ord_key(x)); };
    auto red_max = [&](int r, int k, double x) { atomicMax(&s_red[r][k], ord_key(x)); };

    // ------------------------------------------------------------ prologue
    // time control of the first step from the state as it stands (later steps
    // take theirs from the solves that produce their state), the solver
    // switches, the counters of step 0 and the operator's copy of D
    {
        double v[kMaxInst][4];
        for (int r = 0; r < R; ++r) { v[r][0] = -INFINITY; v[r][1] = 0; v[r][2] = INFINITY; v[r][3] = 0; }
        for (int64_t q = gtid; q < (int64_t)R * N; q += nthreads) {
            const int r = (int)(q / N);
            const int64_t i = q - (int64_t)r * N;
            const double Vo = p.V[q];
            p.sw[q] = Vo > p.switch_v ? 1 : 0;
            if constexpr (!HM) {
                const double d0 = (sizeof(X) == 4 && p.rowsum_e) ? p.D[(int64_t)r * N] : 0.0;
                reinterpret_cast<X*>(p.xd)[i * R + r] = (X)(p.D[q] - d0);
            }
            const bool ctl = p.has_unstable[r] ? (p.unstable[q] != 0) : (i < Ns);
            if (ctl) {
                if (isnan(Vo)) v[r][1] = 1;
                else v[r][0] = fmax(v[r][0], Vo);
                const double qa = fabs(Vo / p.accel[q]);
                if (!isnan(qa) && qa != 0) { v[r][3] = 1; v[r][2] = fmin(v[r][2], qa); }
            }
        }
        if constexpr (!HM) fence_proxy_async_global();
        const int ops[4] = {0, 0, 1, 0};
        block_reduce<4>(v, ops, R);
        if (threadIdx.x == 0) {
            for (int r = 0; r < R; ++r) {
                double* s = red_slot(phase, blk, r);
                s[4] = v[r][0]; s[5] = v[r][1]; s[6] = v[r][2]; s[7] = v[r][3];
                s[8] = (globaltimer_ns() > deadline) ? 1.0 : 0.0;
                s[9] = 0.0;
            }
            if (blk == 0 && HM) atomicExch(p.tile_ctr, 0ull);
        }
        if (!HM && sizeof(X) == 4 && p.rowsum_e && blk == 0 && threadIdx.x < R)
            p.dref[threadIdx.x] = p.D[(int64_t)threadIdx.x * N];   // step 0's offset
        if (!HM && blk == 0) {   // the counter sets of steps 0 and 1
            reset_counter_set(p, 0, true, threadIdx.x, blockDim.x);
            reset_counter_set(p, 1, true, threadIdx.x, blockDim.x);
            __threadfence();
        }
        if (!grid_barrier(p, deadline)) return;
        if ((threadIdx.x >> 5) < R) {
            const int r = threadIdx.x >> 5;
            const int ops5[5] = {0, 0, 1, 0, 0};
            double f[5];
            grid_fields<5>(p.red + (int64_t)(phase & 1) * p.nblk * R * kRedSlots + 4, p.nblk, R, r, ops5, f);
            if ((threadIdx.x & 31) == 0) {
                if (f[4] != 0) s_stop = 1;   // benign race: every writer stores 1
                bool empty;
                s_dt[r] = next_dt(p, f[0], f[1], f[2], f[3], s_dt[r], &empty);
                if (empty && s_fail[r] == 0) s_fail[r] = QDFN_ERR_EMPTY;
            }
        }
        phase++;
        __syncthreads();
    }
    lap(0);

    for (int64_t it = 0; it < nsteps || p.fill_ctr != nullptr; ++it) {
        {
            int stop = s_stop;
            for (int r = 0; r < R; ++r) stop |= (s_fail[r] != 0);
            if (stop) break;
        }
        if (it >= nsteps) {   // fill mode: this member has its steps
            if (blk == 0 && threadIdx.x == 0 && !s_fill_counted) {
                s_fill_counted = 1;
                atomicAdd(p.fill_ctr, 1u);
            }
            if (s_fill_stop) break;
        }
        const int par = s_par;             // which buffer holds the current state
        // the next step's offset: this state's slip of patch 0 (the x copy this
        // step's solves write holds D_next - dref_next)
        const bool offs = !HM && sizeof(X) == 4 && p.rowsum_e != nullptr;
        if (offs && blk == 0 && threadIdx.x < R)
            p.dref[((it + 1) & 1) * R + threadIdx.x] = (par ? p.Dn : p.D)[(int64_t)threadIdx.x * N];
        const int cpar = (int)(it % kSets);   // which counter set this step uses
        const int cnext = (int)((it + 1) % kSets);
        if (threadIdx.x < R) s_done[threadIdx.x] = 0;
        // FP32/BF16 dense: the step's row-block order (rows that start on the
        // high-velocity solver first), from flags the previous step's solves set
        // (double-buffered: the solver warps of the step before may have formed
        // this one's order, and the early-tile count, in its first pass)
        __shared__ unsigned short s_order[2][kMaxOrder];
        __shared__ long long s_next_valid;       // step whose order/early count is precomputed
        __shared__ long long s_next_spec_done;
        if (it == 0 && threadIdx.x == 0) s_next_valid = -1;   // (read after the barrier below)
        const bool use_order = !HM && sizeof(X) == 4 && p.rb_ordered && p.n_rb <= kMaxOrder;
        const bool pre = it > 0 && s_next_valid == it;
        if (use_order && !pre && threadIdx.x < 32) rb_order(p, cpar, s_order[it & 1]);
        if (threadIdx.x >= 32 && threadIdx.x < 32 + R) s_rdt[threadIdx.x - 32] = 1.0 / s_dt[threadIdx.x - 32];
        red_init();
        __syncthreads();
        const X* xdc = reinterpret_cast<const X*>(p.xd) + (size_t)par * p.xd_stride;
        // FP32/BF16: after its own tiles a step streams the next step's first
        // column chunks (not on the last step of a launch, whose next step
        // belongs to another launch)
        StepCtx sc{cpar, cnext, (int)(it & 1), xdc,
                   reinterpret_cast<const X*>(p.xd) + (size_t)(par ^ 1) * p.xd_stride, 0,
                   (!HM && sizeof(X) == 4 && p.c_spec > 0 && (it + 1 < nsteps || p.fill_ctr != nullptr)) ? 1 : 0};
        sc.order = use_order ? s_order[it & 1] : nullptr;
        if (pre) sc.spec_done = s_next_spec_done;
        // one (instance r, patch i) item of a solve pass; pass 0 of a step also
        // forms the row's operator products.  pair: the item runs on a lane
        // pair (lanes 2k, 2k+1, both called with it); the even lane writes the
        // results, the next step's solver switch and Accel, and this item's
        // share of the step reductions.
        // buffer pointers are selected where used, so none is held across the solve
#define QDFN_CUR(a, b) (par ? p.b : p.a)
#define QDFN_NXT(a, b) (par ? p.a : p.b)
        auto solve_item = [&](int64_t q, int r, int64_t i, bool first, bool pair) {
            const bool writer = !pair || (threadIdx.x & 1) == 0;
            // the row's products: formed here in a step's first pass (and kept
            // in registers for this solve), read back in a retry pass
            double tld_q = 0.0, knd_q = 0.0;
            // (H-matrix: a step's first pass forms the products block-wide
            // before its solves, hmat::row_sums_block, so every solve reads them)
            if (first) {
                if constexpr (!HM) {
                    double ss, sn;
                    if (pair) {   // the even lane sums the shear partials, the odd lane the normal ones
                        const unsigned pm = 3u << (threadIdx.x & 30);
                        const double mine = sum_partials_side<sizeof(X) == 4>(p, r, i, (int)(threadIdx.x & 1), sc.ppar);
                        ss = __shfl_sync(pm, mine, (int)(threadIdx.x & 30));
                        sn = __shfl_sync(pm, mine, (int)(threadIdx.x & 30) + 1);
                    } else {
                        sum_partials<sizeof(X) == 4>(p, r, i, ss, sn, sc.ppar);
                    }
                    if (offs) {   // the products of D = x + dref
                        const double dr = p.dref[(it & 1) * R + r];
                        ss = fma(dr, p.rowsum_e[i], ss);
                        sn = fma(dr, p.rowsum_n[i], sn);
                    }
                    tld_q = -ss;   // ELSM * (0 - DispOld)
                    knd_q = sn;    // StiffnessMatrixNormal * DispOld
                    if (writer) {
                        p.tld[q] = tld_q;
                        p.knd[q] = knd_q;
                    }
                }
            } else {
                tld_q = p.tld[q];
                knd_q = p.knd[q];
            }
            const double Dt = s_dt[r];
            double dsn = 0, dss = 0, dsp = 0;
            if (p.n_ext > 0) {
                const double tq = p.interp_at_told ? s_T[r] : s_T[r] + Dt;
                sim::interp_ext(p.n_ext, p.ext_t, p.ext_n, p.ext_s, p.ext_p, N, i, tq, dsn, dss, dsp);
            }
            double sig = knd_q + p.sigma0[q] + dsn;
            if (sig < p.sigma_min) sig = p.sigma_min;
            const double VOld = QDFN_CUR(V, Vn)[q];
            double Vnew;
            if (i < Ns) {
                sim::PatchIn pin;
                pin.DispOld = QDFN_CUR(D, Dn)[q]; pin.FrictionOld = QDFN_CUR(fric, fn)[q];
                pin.ThetaOld = QDFN_CUR(theta, thn)[q];
                pin.VOld = VOld; pin.Friction0 = p.F0[q]; pin.a = p.a[q]; pin.b = p.b[q];
                pin.Dc = p.Dc[q]; pin.K_Self = p.kself[i]; pin.Omega = p.omega[q];
                pin.rDc = p.rDc[q]; pin.ra = p.ra[q]; pin.rDt = s_rdt[r];
                pin.Mass = p.mass[q]; pin.sigma = sig; pin.TLD = 0.0 + tld_q;
                pin.dtau = dss; pin.sigma_old = QDFN_CUR(sig_old, sn)[q]; pin.tau0 = p.tau0[q];
                int err = 0;
                sim::PatchOut o;
                const int swq = QDFN_CUR(sw, sw_n)[q];
                if (swq == 1) {
                    o = pair ? sim::solve_highv_pair(pin, Dt, p.eta, p.alpha_evo, p.evolution_dr, err)
                             : sim::solve_highv(pin, Dt, p.eta, p.alpha_evo, p.evolution_dr, err);
                } else if (pair) {
                    o = sim::solve_lowv_pair(pin, Dt, p.eta, p.alpha_evo, p.evolution_dr, p.switch_v, err);
                } else {
                    o = sim::solve_lowv(pin, Dt, p.eta, p.alpha_evo, p.evolution_dr, p.switch_v, err);
                }
                if (!writer) return;
                if (p.sw_used) p.sw_used[q] = (unsigned char)swq;
                QDFN_NXT(V, Vn)[q] = o.V; QDFN_NXT(fric, fn)[q] = o.Friction; QDFN_NXT(D, Dn)[q] = o.Disp;
                QDFN_NXT(theta, thn)[q] = o.Theta; QDFN_NXT(sig_old, sn)[q] = sig;
                p.dtall[q] = o.Dt; p.instab[q] = o.Instab; p.flag[q] = o.Flag;
                if (swq == 1) { ++n_hi; it_hi += o.Iterations; }
                else { ++n_lo; it_lo += o.Iterations; }
                if (err) red_min(r, 3, (double)err);
                if (o.Flag != 1) red_min(r, 0, (double)o.Flag);
                red_min(r, 1, o.Dt);
                if (o.Instab == 4) red_max(r, 2, 1.0);
                if (o.Flag == 0) {   // Main_D :242-249, applied by the patch's owner
                    if (o.Instab == 3) QDFN_CUR(sw, sw_n)[q] = 1;
                    else if (o.Instab == 4) QDFN_CUR(sw, sw_n)[q] = 0;
                }
                Vnew = o.V;
                if constexpr (!HM) {
                    const double d0 = offs ? QDFN_CUR(D, Dn)[(int64_t)r * N] : 0.0;
                    reinterpret_cast<X*>(p.xd)[(size_t)(par ^ 1) * p.xd_stride + i * R + r] = (X)(o.Disp - d0);
                }
            } else {
                if (!writer) return;   // loading faults (Solvers :370-377)
                if (p.sw_used) p.sw_used[q] = 2;
                const double Vc = p.Vconst[q];
                const double Dn = QDFN_CUR(D, Dn)[q] + Vc * Dt;
                QDFN_NXT(V, Vn)[q] = Vc; QDFN_NXT(fric, fn)[q] = QDFN_CUR(fric, fn)[q]; QDFN_NXT(D, Dn)[q] = Dn;
                QDFN_NXT(theta, thn)[q] = QDFN_CUR(theta, thn)[q]; QDFN_NXT(sig_old, sn)[q] = 1e10;
                p.dtall[q] = Dt;
                p.instab[q] = 0; p.flag[q] = 1;
                red_min(r, 1, Dt);
                Vnew = Vc;
                if constexpr (!HM) {
                    const double d0 = offs ? QDFN_CUR(D, Dn)[(int64_t)r * N] : 0.0;
                    reinterpret_cast<X*>(p.xd)[(size_t)(par ^ 1) * p.xd_stride + i * R + r] = (X)(Dn - d0);
                }
            }
            if constexpr (!HM) fence_proxy_async_global();
            // the next step's Accel, solver switch and time-control statistics
            // (Main_D :265-319 then :162-201) -- final once the step is accepted,
            // since an accepted pass keeps its Dt
            const double A = sim::div_by(Vnew - VOld, sim::recip_pre(Dt, s_rdt[r]));   // (Vnew - VOld) / Dt
            QDFN_NXT(accel, accel_n)[q] = A;
            QDFN_NXT(sw, sw_n)[q] = Vnew > p.switch_v ? 1 : 0;
            if constexpr (!HM) {   // the next step streams and solves this row block early
                if (Vnew > p.switch_v) atomicOr(p.rb_hot + cnext * p.rb_stride + i / p.ld, 1u);
            }
            if (p.has_unstable[r] ? (p.unstable[q] != 0) : (i < Ns)) {
                if (isnan(Vnew)) red_max(r, 5, 1.0);
                else red_max(r, 4, Vnew);
                const double qa = fabs(Vnew / A);
                if (!isnan(qa) && qa != 0) { red_max(r, 7, 1.0); red_min(r, 6, qa); }
            }
        };
#undef QDFN_CUR
#undef QDFN_NXT
        // ---------------------------------------------------------- P2
        if constexpr (HM) {
            const double* Dcur = par ? p.Dn : p.D;
            hmat::pass_a<X, R>(p.h, Dcur, N, xs, hacc);
            // pass B's low-rank tasks wait for this step's pass-A count, not a grid barrier
            if (!hmat::pass_b<X, R>(p.h, Dcur, N, (unsigned long long)(it + 1) * (unsigned long long)p.h.n_lr,
                                    kWaitLimitNs, p.gerr))
                atomicExch(p.gerr, QDFN_ERR_TIMEOUT);
            if (!grid_barrier(p, deadline)) return;
        } else if constexpr (sizeof(X) == 8) {
            // FP64 storage: the operator's FMAs already load the FP64 pipe that
            // the solves need, so the phases run one after the other
            __shared__ int s_op_fail;
            if (threadIdx.x == 0) s_op_fail = 0;
            __syncthreads();
            const uint64_t t_f0 = globaltimer_ns();
            sc.t0 = t_f0;
            if ((threadIdx.x >> 5) < kOpWarps) {
                if (!dense_matvec<M, R>(p, pipe, xs, sc)) s_op_fail = 1;
            } else if (threadIdx.x == kProducerWarp * 32) {
                if (!produce_tiles<M, R>(p, pipe, xs, sc)) s_op_fail = 1;
            }
            if (threadIdx.x == 0) s_tm[6] += globaltimer_ns() - t_f0;
            __syncthreads();
            if (s_op_fail) return;
            if (!grid_barrier(p, deadline)) return;
        } else {
            // Operator and solve pass 0, overlapped.  Warps [0, kOpWarps) stream
            // the operator tiles (HBM-bound); the solver warps take row chunks
            // (32 rows, one lane per patch; 16 on lane pairs) of every row block
            // whose column chunks are all in and solve them (FP64-bound), so the
            // two share each SM.  In a step that streams
            // ahead the operator warps then stream the next step's tiles; in the
            // last step of a launch they join the solving instead.  A row's
            // solve needs only its own operator products, so the result is the
            // same as running the phases one after the other.
            __shared__ int s_fused_fail;
            __shared__ int s_held;       // row chunks this block holds (grabbed, not yet solved)
            __shared__ unsigned long long s_t_solve;
            __shared__ int s_p3_abort;   // the solver warps' grid barrier gave up
            if (threadIdx.x == 0) { s_fused_fail = 0; s_t_solve = 0; s_held = 0; s_p3_abort = 0; }
            __syncthreads();
            const uint64_t t_f0 = globaltimer_ns();
            sc.t0 = t_f0;
            const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
            // a step that streams ahead: the operator warps and the producer
            // stream to the end (early tiles included) and do not solve; the
            // solver warps then run the first reduction pass on their own
            const bool dec = sc.spec != 0;
            bool solve = true;
            if (warp < kOpWarps) {
                if (!dense_matvec<M, R>(p, pipe, xs, sc)) { s_fused_fail = 1; solve = false; }
                if (dec) solve = false;
                if (threadIdx.x == 0) {
                    const uint64_t d = globaltimer_ns() - t_f0;
                    s_tm[6] += d;
                    atomicMax(p.tmax + cpar * 4, (unsigned long long)d);
                }
            } else if (warp == kProducerWarp) {   // lane 0 fills the ring, then the warp solves
                int pok = 1;
                if (lane == 0) {
                    // this step's tiles already streamed during the step before
                    int64_t nrb_reg, n_spec;
                    spec_shape(p, p.n_rb, &nrb_reg, &n_spec);
                    if (!pre)
                        sc.spec_done =
                            (long long)min((int64_t)(ld_acquire_u64(p.spec_ctr + cpar) & ~kSpecClosed), n_spec);
                    pok = produce_tiles<M, R>(p, pipe, xs, sc) ? 1 : 0;
                }
                pok = __shfl_sync(0xffffffffu, pok, 0);
                if (!pok) { s_fused_fail = 1; solve = false; }
                if (dec) solve = false;
            }
            if (solve) {
                constexpr int64_t rpb = (int64_t)kOpThreads * M::VEC;   // operator row block
                const int crows = solve_rows(p);
                const int64_t cpr = rpb / crows;     // row chunks per block and instance
                const int64_t nk = p.n_rb * R * cpr;
                const unsigned* rbd = p.rb_done + cpar * p.rb_stride;
                for (;;) {
                    // a block holds at most hold_cap chunks at a time, so that the
                    // chunks of the last row blocks, which complete together at
                    // the end of the stream, spread over the SMs
                    unsigned long long k = 0;
                    int okh = 1;
                    if (lane == 0) {
                        if (atomicAdd(&s_held, 1) >= p.hold_cap) {
                            const uint64_t t0 = globaltimer_ns();
                            do {
                                atomicSub(&s_held, 1);
                                if (globaltimer_ns() - t0 > kWaitLimitNs || *(volatile int*)p.gerr != 0) {
                                    okh = 0;
                                    break;
                                }
                                __nanosleep(128);
                            } while (atomicAdd(&s_held, 1) >= p.hold_cap);
                        }
                        if (okh) k = atomicAdd(p.solve_ctr + cpar, 1ull);
                    }
                    okh = __shfl_sync(0xffffffffu, okh, 0);
                    if (!okh) {
                        if (lane == 0) atomicExch(p.gerr, QDFN_ERR_TIMEOUT);
                        s_fused_fail = 1;
                        break;
                    }
                    k = __shfl_sync(0xffffffffu, k, 0);
                    if ((int64_t)k >= nk) {
                        if (lane == 0) atomicSub(&s_held, 1);
                        break;
                    }
                    const int64_t rbp = (int64_t)k / (R * cpr), rem = (int64_t)k % (R * cpr);
                    const int64_t rb = sc.order ? (int64_t)sc.order[rbp] : rbp;   // in the step's order
                    const int r = (int)(rem / cpr);
                    const int64_t i0 = rb * rpb + (rem % cpr) * crows;
                    const int64_t i = i0 + (crows == 32 ? lane : (lane >> 1));
                    if (i0 < N) prefetch_chunk(p, par, r, i0, crows);
                    int ok = 1;
                    if (lane == 0) {   // bounded wait for the row block's last column chunk
                        const unsigned need = (unsigned)chunks_of_rb(p, rb) * kOpWarps;   // one per warp and tile
                        if (ld_acquire_u32(rbd + rb) < need) {
                            const uint64_t t0 = globaltimer_ns();
                            while (ld_acquire_u32(rbd + rb) < need) {
                                if (globaltimer_ns() - t0 > kWaitLimitNs || *(volatile int*)p.gerr != 0) {
                                    ok = 0;
                                    break;
                                }
                                __nanosleep(256);
                            }
                        }
                    }
                    ok = __shfl_sync(0xffffffffu, ok, 0);
                    if (!ok) {
                        if (lane == 0) { atomicExch(p.gerr, QDFN_ERR_TIMEOUT); atomicSub(&s_held, 1); }
                        s_fused_fail = 1;
                        break;
                    }
                    const uint64_t t_ready = globaltimer_ns();
                    // pair_solve 0: the even lane alone solves the patch with the one-lane
                    // solver (same results; the lane-pair check uses it); 2: every lane
                    // solves its own patch with the one-lane solver -- fewer FP64
                    // operations per patch (no duplicated secant step), longer chains
                    if (i < N && (p.pair_solve != 0 || (lane & 1) == 0))
                        solve_item((int64_t)r * N + i, r, i, true, p.pair_solve == 1);
                    __syncwarp();
                    if (lane == 0) {
                        atomicSub(&s_held, 1);
                        __threadfence();   // the chunk's x copy of D is written (and proxy-fenced)
                        atomicAdd(p.rb_solved + cpar * p.rb_stride + rb, 1u);
                        atomicMax(p.tmax + cpar * 4 + 2, (unsigned long long)(globaltimer_ns() - t_ready));
                    }
                }
                if (lane == 0) atomicMax(&s_t_solve, (unsigned long long)(globaltimer_ns() - t_f0));
            }
            if (dec && warp >= kOpWarps && warp < kProducerWarp) {
                // The step's first reduction pass, by the solver warps alone,
                // while the operator warps finish the early tiles they hold.
                // Every solver thread runs the same barriers (named barrier 1)
                // and takes the same branches; none returns before the block
                // meets again below.
                const int gt = threadIdx.x - kOpThreads;
                solver_sync();   // the block's solves are in (s_red complete)
                if (gt == 0) s_tm[11] = globaltimer_ns();
                if (blk == 0) {
                    // the counter set two steps ahead (its last users have passed
                    // a grid barrier since)
                    reset_counter_set(p, (int)((it + 2) % kSets), true, gt, kSolverThreads);
                    __threadfence();
                }
                if (gt == 0) {
                    const double late = (globaltimer_ns() > deadline) ? 1.0 : 0.0;
                    for (int r = 0; r < R; ++r) {
                        double* sl = red_slot(phase, blk, r);
                        for (int k = 0; k < 8; ++k) sl[k] = ord_val(s_red[r][k]);
                        sl[8] = late;
                        sl[9] = fill_seen(it);
                    }
                }
                const uint64_t t_items = gt == 0 ? globaltimer_ns() : 0;
                // (the last block to arrive closes the next step's early-tile
                // counter: their number is final for every block leaving it)
                if (!grid_barrier_solvers(p, deadline, p.spec_ctr + cnext)) {
                    if (gt == 0) s_p3_abort = 1;
                } else {
                    if (gt == 0) {
                        const uint64_t t = globaltimer_ns();
                        s_tm[4] += t_items - s_tm[11];
                        s_tm[5] += t - t_items;
                        s_tm[11] = t;
                        if (blk == 0 && it > 0) {   // the previous step's maxima are complete
                            const int ps = (int)((it + kSets - 1) % kSets);
                            s_tm[8] += __ldcg(p.tmax + ps * 4);
                            s_tm[9] += __ldcg(p.tmax + ps * 4 + 1);
                            s_tm[12] += __ldcg(p.tmax + ps * 4 + 2);
                            s_tm[13] += __ldcg(p.tmax + ps * 4 + 3);
                        }
                    }
                    const int r = gt >> 5;
                    if (r == kSolverWarps - 1 && r >= R) {
                        // the next step's row order and early-tile count: final
                        // now unless this step retries (then they are formed again)
                        if (use_order) rb_order(p, cnext, s_order[(it + 1) & 1]);
                        if ((threadIdx.x & 31) == 0) {
                            int64_t nrb_reg, n_spec;
                            spec_shape(p, p.n_rb, &nrb_reg, &n_spec);
                            s_next_spec_done = (long long)min(
                                (int64_t)(ld_acquire_u64(p.spec_ctr + cnext) & ~kSpecClosed), n_spec);
                            s_next_valid = it + 1;
                        }
                    }
                    if (r < R) {
                        const int ops[10] = {1, 1, 0, 1, 0, 0, 1, 0, 0, 0};
                        double f[10];
                        grid_fields<10>(p.red + (int64_t)(phase & 1) * p.nblk * R * kRedSlots, p.nblk, R, r,
                                        ops, f);
                        const double mflag = f[0], mdt = f[1], any4 = f[2], err = f[3];
                        if ((threadIdx.x & 31) == 0) {
                            if (f[8] != 0) s_stop = 1;
                            if (f[9] != 0) s_fill_stop = 1;
                            if (err != 0) { s_fail[r] = (int)err; s_done[r] = 1; }
                            else if (mflag == 0) {
                                s_dt[r] = any4 != 0 ? 1e-3 : mdt;
                            } else {
                                s_dt[r] = mdt;   // Main_D :262 Dt = minimum(Dt_All)
                                s_done[r] = 1;
                                bool empty;
                                s_dtn[r] = next_dt(p, f[4], f[5], f[6], f[7], mdt, &empty);
                                if (empty && s_fail[r] == 0) s_fail[r] = QDFN_ERR_EMPTY;
                            }
                        }
                    }
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                s_tm[7] += s_t_solve;
                atomicMax(p.tmax + cpar * 4 + 1, s_t_solve);
            }
            if (s_fused_fail || s_p3_abort) return;
        }
        lap(1);
        // ---------------------------------------------------------- P3
        // pass 0 already ran in the solver warps when the step streamed ahead
        const bool pass0_done = !HM && sizeof(X) == 4 && sc.spec != 0;
        if (pass0_done) { phase++; n_iter++; }
        if (threadIdx.x == 0) {
            s_iter = pass0_done ? 1 : 0;
            if (!pass0_done) s_tm[11] = globaltimer_ns();
        }
        __syncthreads();
        bool more = true;
        if (pass0_done) {
            int all = 1;
            for (int r = 0; r < R; ++r) all &= s_done[r];
            more = !all;
            // a retry discards the next step's early tiles: every block must
            // have finished those it holds before their counters are reset
            if (more && threadIdx.x == 0) s_next_valid = -1;
            if (more && !grid_barrier(p, deadline)) return;
        }
        while (more) {
            const int first = (s_iter == 0);
            if (HM || sizeof(X) == 8 || !first) {   // FP32/BF16 dense pass 0 ran alongside the operator
                if (!first) {
                    red_init();
                    if (threadIdx.x < R) s_rdt[threadIdx.x] = 1.0 / s_dt[threadIdx.x];
                    __syncthreads();
                }
                // every CTA takes an equal contiguous range of (instance, patch)
                // items: the solves are FP64-pipe bound, so the per-SM item count
                // sets the pass time
                const int64_t per_cta = ((int64_t)R * N + p.nblk - 1) / p.nblk;
                const int64_t q_end = min((int64_t)R * N, (int64_t)blk * per_cta + per_cta);
                bool prod_here = first != 0;   // the solve item forms its own row's products
                if constexpr (HM) {
                    if (first) {   // the block's row sums first, spread over all its threads
                        hmat::row_sums_block<R>(p.h, N, p.kself, p.tld, p.knd, (int64_t)blk * per_cta, q_end);
                        __syncthreads();
                        prod_here = false;
                    }
                }
                for (int64_t q = (int64_t)blk * per_cta + threadIdx.x; q < q_end; q += kSimThreads) {
                    const int r = (int)(q / N);
                    if (s_done[r]) continue;
                    solve_item(q, r, q - (int64_t)r * N, prod_here, false);
                }
            }
            if (!HM && blk == 0 && (first || s_iter == 1)) {
                // pass 0: reset the counter set two steps ahead (its last users
                // have passed a grid barrier since; the next step's early tiles
                // will use it).
                // First retry pass: this step's slip changes, so the next step's
                // early tiles are discarded -- their counters start again (the
                // order flags stay: the retry's solves add to them, and the
                // order only decides when work is taken, not its result)
                reset_counter_set(p, first ? (int)((it + 2) % kSets) : cnext, first, threadIdx.x, blockDim.x);
                __threadfence();
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                const double late = (globaltimer_ns() > deadline) ? 1.0 : 0.0;
                for (int r = 0; r < R; ++r) {
                    double* s = red_slot(phase, blk, r);
                    for (int k = 0; k < 8; ++k) s[k] = ord_val(s_red[r][k]);
                    s[8] = late;
                    s[9] = fill_seen(it);
                }
            }
            const uint64_t t_items = threadIdx.x == 0 ? globaltimer_ns() : 0;
            if (!grid_barrier(p, deadline)) return;
            {   // CTA 0: own solves + block reduction, then the wait for the grid
                if (threadIdx.x == 0) {
                    const uint64_t t = globaltimer_ns();
                    s_tm[4] += t_items - s_tm[11];
                    s_tm[5] += t - t_items;
                    s_tm[11] = t;
                }
                if (!HM && first && blk == 0 && threadIdx.x == 0) {   // every block has stored its max
                    // (a step that streamed ahead had its maxima read by the step after)
                    const bool prev_ahead = it > 0 && sizeof(X) == 4 && p.c_spec > 0;
                    for (int k = prev_ahead ? 0 : 1; k < 2; ++k) {
                        const int ss = k == 0 ? (int)((it + kSets - 1) % kSets) : cpar;
                        s_tm[8] += __ldcg(p.tmax + ss * 4);
                        s_tm[9] += __ldcg(p.tmax + ss * 4 + 1);
                        s_tm[12] += __ldcg(p.tmax + ss * 4 + 2);
                        s_tm[13] += __ldcg(p.tmax + ss * 4 + 3);
                    }
                }
            }
            if ((threadIdx.x >> 5) < R) {
                const int r = threadIdx.x >> 5;
                if (!s_done[r]) {
                    const int ops[10] = {1, 1, 0, 1, 0, 0, 1, 0, 0, 0};
                    double f[10];
                    grid_fields<10>(p.red + (int64_t)(phase & 1) * p.nblk * R * kRedSlots, p.nblk, R, r, ops,
                                    f);
                    const double mflag = f[0], mdt = f[1], any4 = f[2], err = f[3];
                    if ((threadIdx.x & 31) == 0) {
                        if (f[8] != 0) s_stop = 1;   // benign race: every writer stores 1
                        if (f[9] != 0) s_fill_stop = 1;
                        if (err != 0) { s_fail[r] = (int)err; s_done[r] = 1; }
                        else if (mflag == 0) {
                            s_dt[r] = any4 != 0 ? 1e-3 : mdt;
                        } else {
                            s_dt[r] = mdt;   // Main_D :262 Dt = minimum(Dt_All)
                            s_done[r] = 1;
                            bool empty;      // the next step's Dt from this state
                            s_dtn[r] = next_dt(p, f[4], f[5], f[6], f[7], mdt, &empty);
                            if (empty && s_fail[r] == 0) s_fail[r] = QDFN_ERR_EMPTY;
                        }
                    }
                }
            }
            __syncthreads();
            phase++;
            n_iter++;
            if (threadIdx.x == 0) s_iter++;
            __syncthreads();
            int all = 1;
            for (int r = 0; r < R; ++r) all &= s_done[r];
            if (all) break;
            if (s_iter > kRetryCap) {
                if (threadIdx.x < R && !s_done[threadIdx.x]) s_fail[threadIdx.x] = QDFN_ERR_RETRIES;
                __syncthreads();
                break;
            }
        }
        {   // an instance that failed in its solves keeps the state it had
            int solvefail = 0;
            for (int r = 0; r < R; ++r) solvefail |= (s_fail[r] != 0 && s_fail[r] != QDFN_ERR_EMPTY);
            if (solvefail) break;
        }
        lap(2);
        // ---------------------------------------------------------- P4
        // the step is accepted: history record, time, and the buffers swap
        {
            int rec = 0;
            for (int r = 0; r < R; ++r) {
                const int64_t gstep = s_step[r] + 1;
                rec |= (p.record_step > 0 && gstep % p.record_step == 0 && s_nrec[r] < p.max_records);
            }
            if (rec) {
                const StateView nxt = state_view(p, par ^ 1);
                for (int64_t q = gtid; q < (int64_t)R * N; q += nthreads) {
                    const int r = (int)(q / N);
                    const int64_t i = q - (int64_t)r * N;
                    const int64_t gstep = s_step[r] + 1;
                    if (p.record_step > 0 && gstep % p.record_step == 0 && s_nrec[r] < p.max_records) {
                        const int64_t o = ((int64_t)r * p.max_records + s_nrec[r]) * N + i;
                        p.hV[o] = nxt.V[q]; p.hD[o] = nxt.D[q]; p.hth[o] = nxt.theta[q]; p.hs[o] = nxt.sig_old[q];
                        if (i == 0) {
                            p.hT[(int64_t)r * p.max_records + s_nrec[r]] = s_T[r];
                            p.hDt[(int64_t)r * p.max_records + s_nrec[r]] = s_dt[r];
                        }
                    }
                }
            }
        }
        __syncthreads();
        if (threadIdx.x < R) {
            const int r = threadIdx.x;
            const int64_t gstep = s_step[r] + 1;
            if (p.record_step > 0 && gstep % p.record_step == 0 && s_nrec[r] < p.max_records)
                s_nrec[r]++;
            s_T[r] = s_T[r] + s_dt[r];
            s_step[r] = gstep;
            s_dta[r] = s_dt[r];
            s_dt[r] = s_dtn[r];
        }
        if (threadIdx.x == 0) s_par = par ^ 1;
        __syncthreads();
        lap(3);
        n_steps++;
    }
    // fill mode: a member that ended before its nsteps (a failure) still counts,
    // so that the others stop
    if (p.fill_ctr != nullptr && blk == 0 && threadIdx.x == 0 && !s_fill_counted) atomicAdd(p.fill_ctr, 1u);
    // the state back into the host-visible buffers when it ended in the others
    if (s_par) {
        const StateView a = state_view(p, 0), b = state_view(p, 1);
        for (int64_t q = gtid; q < (int64_t)R * N; q += nthreads) {
            a.V[q] = b.V[q]; a.D[q] = b.D[q]; a.theta[q] = b.theta[q];
            a.fric[q] = b.fric[q]; a.accel[q] = b.accel[q]; a.sig_old[q] = b.sig_old[q];
        }
    }
    if (blk == 0 && threadIdx.x == 0 && p.prof) {
        for (int k = 0; k < 4; ++k) atomicAdd(p.prof + k, s_tm[k]);
        atomicAdd(p.prof + 4, n_iter);
        atomicAdd(p.prof + 5, n_steps);
        for (int k = 0; k < 6; ++k) atomicAdd(p.prof + 10 + k, s_tm[4 + k]);
        atomicAdd(p.prof + 16, s_tm[12]);
        atomicAdd(p.prof + 17, s_tm[13]);
    }
    if (p.prof) {   // solver work of every thread, one atomic per warp and counter
        unsigned long long w[4] = {n_lo, it_lo, n_hi, it_hi};   // widened before the sums
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            for (int o = 16; o > 0; o >>= 1) w[k] += __shfl_xor_sync(0xffffffffu, w[k], o);
            if ((threadIdx.x & 31) == 0 && w[k]) atomicAdd(p.prof + 6 + k, w[k]);
        }
    }
    if (blk == 0 && threadIdx.x < R) {
        const int r = threadIdx.x;
        p.T[r] = s_T[r];
        p.dt[r] = s_dta[r];
        p.step[r] = s_step[r];
        p.nrec[r] = s_nrec[r];
        p.status[r] = s_fail[r];
        if (s_stop && s_fail[r] == 0) atomicExch(p.gerr, QDFN_ERR_TIMEOUT);
    }
}

template <class M, int R, bool HM>
__global__ void __launch_bounds__(kSimThreads, 1) k_sim(SimParams p, int64_t nsteps) {
    sim_run<M, R, HM>(p, nsteps, (int)blockIdx.x);
}

// Ensemble launch: one cooperative grid runs several contexts ("members") of
// the same operator format and instance count side by side, each on its own
// contiguous range of blocks with its own barrier words, counters and state.
// Block b runs member map[b].x as its block map[b].y.  Each block copies its
// member's parameters into shared memory once.
template <class M, int R>
__global__ void __launch_bounds__(kSimThreads, 1) k_sim_members(const SimParams* __restrict__ members,
                                                                 const int2* __restrict__ map,
                                                                 int64_t nsteps) {
    __shared__ __align__(16) SimParams sp;
    static_assert(sizeof(SimParams) % 8 == 0, "SimParams copied in 8-byte words");
    const int2 mb = map[blockIdx.x];
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(members + mb.x);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&sp);
    for (int k = threadIdx.x; k < (int)(sizeof(SimParams) / 8); k += blockDim.x) dst[k] = src[k];
    __syncthreads();
    sim_run<M, R, false>(sp, nsteps, mb.y);
}

// x copy of D for the operator-only kernel: [patch][instance] in the operator's type
template <class X, int R>
__global__ void k_fill_xd(SimParams p) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)R * p.N) return;
    const int r = (int)(q / p.N);
    const double d0 = (sizeof(X) == 4 && p.rowsum_e) ? p.D[(int64_t)r * p.N] : 0.0;
    reinterpret_cast<X*>(p.xd)[(q - (int64_t)r * p.N) * R + r] = (X)(p.D[q] - d0);
}

// Operator-only kernel (qdfn_apply_operator): one pass of P2 + chunk reduction.
template <class M, int R>
__global__ void __launch_bounds__(kSimThreads, 1) k_apply(SimParams p) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    using X = typename M::X;
    Pipe pipe;
    pipe_init(pipe, smem_raw);
    X* xs = reinterpret_cast<X*>(smem_raw + kPipeBytes + kMbarBytes);
    const int warp = threadIdx.x >> 5;
    const StepCtx sc{0, 1, 0, p.xd, p.xd, 0, 0};
    if (warp < kOpWarps) dense_matvec<M, R>(p, pipe, xs, sc);          // the operator role
    else if (threadIdx.x == kProducerWarp * 32) produce_tiles<M, R>(p, pipe, xs, sc);
}

template <class X, int R>
__global__ void __launch_bounds__(kSimThreads, 1) k_hmat_a(SimParams p) {
    extern __shared__ unsigned char smem_raw[];
    hmat::pass_a<X, R>(p.h, p.D, p.N, reinterpret_cast<X*>(smem_raw),
                       reinterpret_cast<double*>(smem_raw + (size_t)R * hmat::kChunk * sizeof(X)));
}
template <class X, int R>
__global__ void __launch_bounds__(kSimThreads, 1) k_hmat_b(SimParams p) {
    extern __shared__ unsigned char smem_raw[];
    hmat::pass_b<X, R>(p.h, p.D, p.N, 0ull, kWaitLimitNs, p.gerr);   // pass A ran in the launch before
}
// receiver-row sums of the operator-only H product: 32 rows per 256-thread
// block (eight threads per row: four per matrix)
template <int R>
__global__ void k_hmat_rows(SimParams p) {
    const int64_t q0 = (int64_t)blockIdx.x * (blockDim.x / 8);
    const int64_t q1 = min((int64_t)R * p.N, q0 + (int64_t)(blockDim.x / 8));
    hmat::row_sums_block<R>(p.h, p.N, p.kself, p.tld, p.knd, q0, q1);
}

template <bool kPairs>
__global__ void k_chunk_reduce(SimParams p) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)p.R * p.N) return;
    const int r = (int)(q / p.N);
    const int64_t i = q - (int64_t)r * p.N;
    double ss, sn;
    sum_partials<kPairs>(p, r, i, ss, sn);
    if (kPairs && p.rowsum_e) {   // D = x + D(patch 0), as k_fill_xd wrote x
        const double d0 = p.D[(int64_t)r * p.N];
        ss = fma(d0, p.rowsum_e[i], ss);
        sn = fma(d0, p.rowsum_n[i], sn);
    }
    p.tld[q] = -ss;
    p.knd[q] = sn;
}

// ---------------------------------------------------------------------------
// conversion kernel: ELSM = K_ij/K_ii and Kn in the chosen format, in the
// tile-contiguous layout -- receivers in blocks of rpb rows (the operator
// tile height), and within a block all source columns back to back:
// entry (i, j) at ((i / rpb) * N + j) * rpb + i % rpb.  Rows past N are zero.
__global__ void k_convert(const double* __restrict__ Ks, const double* __restrict__ Knm,
                          int64_t N, int64_t ld_in, int layout, int64_t rpb, int prec,
                          void* E, void* Kn, double* kself) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // receiver
    const int64_t j = blockIdx.y;                                        // source (loops)
    const int64_t nrows = (N + rpb - 1) / rpb * rpb;
    for (int64_t jj = j; jj < N; jj += gridDim.y) {
        if (i >= nrows) continue;
        double e = 0.0, k = 0.0;
        if (i < N) {
            const int64_t in = layout == QDFN_LAYOUT_COL ? jj * ld_in + i : i * ld_in + jj;
            const int64_t dd = layout == QDFN_LAYOUT_COL ? i * ld_in + i : i * ld_in + i;
            const double kii = Ks[dd];
            e = (i == jj) ? 0.0 : Ks[in] / kii;   // Main_D :58-62
            k = Knm[in];
            if (jj == 0) kself[i] = fabs(kii);
        }
        const int64_t o = ((i / rpb) * N + jj) * rpb + i % rpb;
        if (prec == QDFN_FP64) {
            reinterpret_cast<double*>(E)[o] = e;
            reinterpret_cast<double*>(Kn)[o] = k;
        } else if (prec == QDFN_FP32) {
            reinterpret_cast<float*>(E)[o] = (float)e;
            reinterpret_cast<float*>(Kn)[o] = (float)k;
        } else {
            auto split = [](double x) -> uint32_t {
                const __nv_bfloat16 hi = __double2bfloat16(x);
                const double rem = x - (double)__bfloat162float(hi);
                const __nv_bfloat16 lo = __double2bfloat16(rem);
                return ((uint32_t)__bfloat16_as_ushort(hi) << 16) | (uint32_t)__bfloat16_as_ushort(lo);
            };
            reinterpret_cast<uint32_t*>(E)[o] = split(e);
            reinterpret_cast<uint32_t*>(Kn)[o] = split(k);
        }
    }
}

// Row sums of the stored FP32 / BF16 hi+lo operator in FP64 (the values the
// products multiply, decoded as the operator warps decode them): one thread
// per receiver row, stepping over the source columns of its row block
// (consecutive rows are consecutive words).
__global__ void k_rowsum(int64_t N, int64_t rpb, int prec, const void* E, const void* Kn, double* rse,
                         double* rsn) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int64_t base = (i / rpb) * N * rpb + i % rpb;
    double se = 0.0, sn = 0.0;
    for (int64_t j = 0; j < N; ++j) {
        const int64_t o = base + j * rpb;
        if (prec == QDFN_FP32) {
            se += (double)reinterpret_cast<const float*>(E)[o];
            sn += (double)reinterpret_cast<const float*>(Kn)[o];
        } else {
            const uint32_t a = reinterpret_cast<const uint32_t*>(E)[o], b = reinterpret_cast<const uint32_t*>(Kn)[o];
            se += (double)(__uint_as_float(a & 0xFFFF0000u) + __uint_as_float(a << 16));
            sn += (double)(__uint_as_float(b & 0xFFFF0000u) + __uint_as_float(b << 16));
        }
    }
    rse[i] = se;
    rsn[i] = sn;
}

}  // namespace
}  // namespace qdfn
