// Persistent earthquake-cycle kernel and the simulation-context C ABI.
//
// One cooperative launch advances every instance of a context by `nsteps` time
// steps.  Per step (scripts/Functions_RSFDFN3DMain_D.jl:146-322):
//   P1  solver switch (VOld > SwitchV) and the time-step control reductions
//       (max V and min |V/Accel| over the unstable patches, :163-187) -- once
//       per launch; afterwards folded into each step's solve pass
//   P2  elastic operator: one pass over the shear (K_ij/K_ii) and normal
//       matrices computes both products for all instances at once
//   P3  per-patch secant solves (SolveOneTimeStep, Functions_Solvers.jl:334),
//       then the retry decision (:240-253) -- repeated until every instance
//       accepts its step
//   P4  history record, T += Dt, Accel, state buffers swap (:265-319)
// With the dense FP32/BF16 operator, P2 and P3's first pass overlap within each
// block (operator warps stream tiles, solver warps solve each row block as its
// tiles complete), the operator warps go on to the next step's tiles whose
// slip is already solved, and the solver warps run P3's reductions and grid
// barrier on their own meanwhile.  Every CTA reduces the per-CTA partials
// itself, so all CTAs hold identical step scalars without another round trip.
// Grid barriers are a counter/generation pair with a bounded wait on
// %globaltimer: a wait that outlives the deadline sets QDFN_ERR_TIMEOUT and the
// kernel returns.  The launch is cooperative, so all CTAs are co-resident.
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

struct SimParams {
    int64_t N, Nload, ld;
    int R;
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
    int pair_solve;                  // overlapped phase: one lane pair per patch (else the even lanes alone)
    int rb_ordered;                  // FP32/BF16 dense: row blocks with high-velocity patches first
    int c_spec;                      // dense: column chunks of the next step streamed during a step's tail
    int spec_stop;                   // no early-tile claims once this many blocks reached the step's barrier
    unsigned long long* tmax;        // [kSets][4] per-step max over blocks of (operator end, solver end,
                                     // chunk ready->solved, last row block complete), ns
};

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
        if (prev == gridDim.x - 1) {
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
static_assert(hmat::kTileRows == kSimThreads, "H-matrix row tiles are one row per thread");
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
        if (prev == gridDim.x - 1) {
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
            const unsigned need = (unsigned)(R * (rows_per_blk / 16));   // solve chunks per row block
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

template <class M, int R, bool HM>
__global__ void __launch_bounds__(kSimThreads, 1) k_sim(SimParams p, int64_t nsteps) {
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
    const int64_t nthreads = (int64_t)gridDim.x * kSimThreads;
    const int64_t gtid = (int64_t)blockIdx.x * kSimThreads + threadIdx.x;
    int phase = 0;  // parity selector of the reduction buffer
    if (threadIdx.x < R) {
        s_T[threadIdx.x] = p.T[threadIdx.x];
        s_dt[threadIdx.x] = p.dt[threadIdx.x];
        s_dta[threadIdx.x] = p.dt[threadIdx.x];
        s_step[threadIdx.x] = p.step[threadIdx.x];
        s_nrec[threadIdx.x] = p.nrec[threadIdx.x];
        s_fail[threadIdx.x] = p.status[threadIdx.x];
    }
    if (threadIdx.x == 0) { s_stop = 0; s_par = 0; }
    auto red_slot = [&](int ph, int64_t blk, int r) -> double* {
        return p.red + (((int64_t)(ph & 1) * gridDim.x + blk) * R + r) * kRedSlots;
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
            if constexpr (!HM) reinterpret_cast<X*>(p.xd)[i * R + r] = (X)p.D[q];
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
                double* s = red_slot(phase, blockIdx.x, r);
                s[4] = v[r][0]; s[5] = v[r][1]; s[6] = v[r][2]; s[7] = v[r][3];
                s[8] = (globaltimer_ns() > deadline) ? 1.0 : 0.0;
            }
            if (blockIdx.x == 0 && HM) atomicExch(p.tile_ctr, 0ull);
        }
        if (!HM && blockIdx.x == 0) {   // the counter sets of steps 0 and 1
            reset_counter_set(p, 0, true, threadIdx.x, blockDim.x);
            reset_counter_set(p, 1, true, threadIdx.x, blockDim.x);
            __threadfence();
        }
        if (!grid_barrier(p, deadline)) return;
        if ((threadIdx.x >> 5) < R) {
            const int r = threadIdx.x >> 5;
            const int ops5[5] = {0, 0, 1, 0, 0};
            double f[5];
            grid_fields<5>(p.red + (int64_t)(phase & 1) * gridDim.x * R * kRedSlots + 4, gridDim.x, R, r, ops5, f);
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

    for (int64_t it = 0; it < nsteps; ++it) {
        {
            int stop = s_stop;
            for (int r = 0; r < R; ++r) stop |= (s_fail[r] != 0);
            if (stop) break;
        }
        const int par = s_par;             // which buffer holds the current state
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
                   (!HM && sizeof(X) == 4 && p.c_spec > 0 && it + 1 < nsteps) ? 1 : 0};
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
            if (first) {
                if constexpr (HM) {
                    // main_H :241-248: H_load (0 - D) ./ -K_Self and H_n D
                    const double ss = hmat::row_sum<R>(p.h, 0, N, i, r);
                    p.tld[q] = (-ss) / -p.kself[i];
                    p.knd[q] = hmat::row_sum<R>(p.h, 1, N, i, r);
                } else {
                    double ss, sn;
                    if (pair) {   // the even lane sums the shear partials, the odd lane the normal ones
                        const unsigned pm = 3u << (threadIdx.x & 30);
                        const double mine = sum_partials_side<sizeof(X) == 4>(p, r, i, (int)(threadIdx.x & 1), sc.ppar);
                        ss = __shfl_sync(pm, mine, (int)(threadIdx.x & 30));
                        sn = __shfl_sync(pm, mine, (int)(threadIdx.x & 30) + 1);
                    } else {
                        sum_partials<sizeof(X) == 4>(p, r, i, ss, sn, sc.ppar);
                    }
                    if (writer) {
                        p.tld[q] = -ss;   // ELSM * (0 - DispOld)
                        p.knd[q] = sn;    // StiffnessMatrixNormal * DispOld
                    }
                    if (pair) __syncwarp(3u << (threadIdx.x & 30));   // the odd lane reads them below
                }
            }
            const double Dt = s_dt[r];
            double dsn = 0, dss = 0, dsp = 0;
            if (p.n_ext > 0) {
                const double tq = p.interp_at_told ? s_T[r] : s_T[r] + Dt;
                sim::interp_ext(p.n_ext, p.ext_t, p.ext_n, p.ext_s, p.ext_p, N, i, tq, dsn, dss, dsp);
            }
            double sig = p.knd[q] + p.sigma0[q] + dsn;
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
                pin.Mass = p.mass[q]; pin.sigma = sig; pin.TLD = 0.0 + p.tld[q];
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
                if constexpr (!HM) reinterpret_cast<X*>(p.xd)[(size_t)(par ^ 1) * p.xd_stride + i * R + r] = (X)o.Disp;
            } else {
                if (!writer) return;   // loading faults (Solvers :370-377)
                const double Vc = p.Vconst[q];
                const double Dn = QDFN_CUR(D, Dn)[q] + Vc * Dt;
                QDFN_NXT(V, Vn)[q] = Vc; QDFN_NXT(fric, fn)[q] = QDFN_CUR(fric, fn)[q]; QDFN_NXT(D, Dn)[q] = Dn;
                QDFN_NXT(theta, thn)[q] = QDFN_CUR(theta, thn)[q]; QDFN_NXT(sig_old, sn)[q] = 1e10;
                p.dtall[q] = Dt;
                p.instab[q] = 0; p.flag[q] = 1;
                red_min(r, 1, Dt);
                Vnew = Vc;
                if constexpr (!HM) reinterpret_cast<X*>(p.xd)[(size_t)(par ^ 1) * p.xd_stride + i * R + r] = (X)Dn;
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
            if (!grid_barrier(p, deadline)) return;
            hmat::pass_b<X, R>(p.h, Dcur, N, xs);
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
            // the operator tiles (HBM-bound); the solver warps take 16-row chunks
            // of every row block whose column chunks are all in and solve them
            // (FP64-bound), so the two share each SM.  In a step that streams
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
                constexpr int64_t cpr = rpb / 16;     // 16-row chunks (one lane pair per row) per block and instance
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
                    const int64_t i = rb * rpb + (rem % cpr) * 16 + (lane >> 1);
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
                    // QDFN_PAIR_SOLVE=0: the even lane alone solves the patch with the
                    // one-lane solver (same results; the lane-pair check uses it)
                    if (i < N && (p.pair_solve || (lane & 1) == 0))
                        solve_item((int64_t)r * N + i, r, i, true, p.pair_solve != 0);
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
                if (blockIdx.x == 0) {
                    // the counter set two steps ahead (its last users have passed
                    // a grid barrier since)
                    reset_counter_set(p, (int)((it + 2) % kSets), true, gt, kSolverThreads);
                    __threadfence();
                }
                if (gt == 0) {
                    const double late = (globaltimer_ns() > deadline) ? 1.0 : 0.0;
                    for (int r = 0; r < R; ++r) {
                        double* sl = red_slot(phase, blockIdx.x, r);
                        for (int k = 0; k < 8; ++k) sl[k] = ord_val(s_red[r][k]);
                        sl[8] = late;
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
                        if (blockIdx.x == 0 && it > 0) {   // the previous step's maxima are complete
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
                        const int ops[9] = {1, 1, 0, 1, 0, 0, 1, 0, 0};
                        double f[9];
                        grid_fields<9>(p.red + (int64_t)(phase & 1) * gridDim.x * R * kRedSlots, gridDim.x, R, r,
                                       ops, f);
                        const double mflag = f[0], mdt = f[1], any4 = f[2], err = f[3];
                        if ((threadIdx.x & 31) == 0) {
                            if (f[8] != 0) s_stop = 1;
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
                const int64_t per_cta = ((int64_t)R * N + gridDim.x - 1) / gridDim.x;
                const int64_t q_end = min((int64_t)R * N, (int64_t)blockIdx.x * per_cta + per_cta);
                for (int64_t q = (int64_t)blockIdx.x * per_cta + threadIdx.x; q < q_end; q += kSimThreads) {
                    const int r = (int)(q / N);
                    if (s_done[r]) continue;
                    solve_item(q, r, q - (int64_t)r * N, first != 0, false);
                }
            }
            if (!HM && blockIdx.x == 0 && (first || s_iter == 1)) {
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
                    double* s = red_slot(phase, blockIdx.x, r);
                    for (int k = 0; k < 8; ++k) s[k] = ord_val(s_red[r][k]);
                    s[8] = late;
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
                if (!HM && first && blockIdx.x == 0 && threadIdx.x == 0) {   // every block has stored its max
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
                    const int ops[9] = {1, 1, 0, 1, 0, 0, 1, 0, 0};
                    double f[9];
                    grid_fields<9>(p.red + (int64_t)(phase & 1) * gridDim.x * R * kRedSlots, gridDim.x, R, r, ops,
                                   f);
                    const double mflag = f[0], mdt = f[1], any4 = f[2], err = f[3];
                    if ((threadIdx.x & 31) == 0) {
                        if (f[8] != 0) s_stop = 1;   // benign race: every writer stores 1
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
    // the state back into the host-visible buffers when it ended in the others
    if (s_par) {
        const StateView a = state_view(p, 0), b = state_view(p, 1);
        for (int64_t q = gtid; q < (int64_t)R * N; q += nthreads) {
            a.V[q] = b.V[q]; a.D[q] = b.D[q]; a.theta[q] = b.theta[q];
            a.fric[q] = b.fric[q]; a.accel[q] = b.accel[q]; a.sig_old[q] = b.sig_old[q];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && p.prof) {
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
    if (blockIdx.x == 0 && threadIdx.x < R) {
        const int r = threadIdx.x;
        p.T[r] = s_T[r];
        p.dt[r] = s_dta[r];
        p.step[r] = s_step[r];
        p.nrec[r] = s_nrec[r];
        p.status[r] = s_fail[r];
        if (s_stop && s_fail[r] == 0) atomicExch(p.gerr, QDFN_ERR_TIMEOUT);
    }
}

// x copy of D for the operator-only kernel: [patch][instance] in the operator's type
template <class X, int R>
__global__ void k_fill_xd(SimParams p) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)R * p.N) return;
    const int r = (int)(q / p.N);
    reinterpret_cast<X*>(p.xd)[(q - (int64_t)r * p.N) * R + r] = (X)p.D[q];
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
    hmat::pass_b<X, R>(p.h, p.D, p.N, reinterpret_cast<X*>(smem_raw));
}
template <int R>
__global__ void k_hmat_rows(SimParams p) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)R * p.N) return;
    const int r = (int)(q / p.N);
    const int64_t i = q - (int64_t)r * p.N;
    p.tld[q] = (-hmat::row_sum<R>(p.h, 0, p.N, i, r)) / -p.kself[i];
    p.knd[q] = hmat::row_sum<R>(p.h, 1, p.N, i, r);
}

template <bool kPairs>
__global__ void k_chunk_reduce(SimParams p) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)p.R * p.N) return;
    const int r = (int)(q / p.N);
    const int64_t i = q - (int64_t)r * p.N;
    double ss, sn;
    sum_partials<kPairs>(p, r, i, ss, sn);
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

}  // namespace
}  // namespace qdfn

// ===========================================================================
// Context
using namespace qdfn;

struct qdfn_ctx {
    int64_t N = 0, Nload = 0, ld = 0;
    int R = 1;
    int prec = -1;
    int hmat = 0;
    qdfn_problem prob{};
    double eta = 0;
    // device buffers
    std::vector<void*> allocs;
    double *a, *b, *Dc, *F0, *tau0, *sigma0, *Vconst, *mass, *omega, *kself;
    double *ra = nullptr, *rDc = nullptr;
    unsigned char* unstable;
    int* has_unstable;
    double *V, *D, *theta, *fric, *accel, *sig_old, *Vn, *Dn, *thn, *fn, *sn, *dtall, *tld, *knd;
    int *instab, *flag, *sw, *sw_n;
    double* accel_n;
    double *part_s = nullptr, *part_n = nullptr;
    double *T, *dt;
    int64_t *step, *nrec;
    int* status;
    double *hT, *hDt, *hV, *hD, *hth, *hs;
    unsigned *bar_count, *bar_gen;
    double* red = nullptr;
    int* gerr;
    unsigned long long* prof;
    unsigned long long* tile_ctr;
    unsigned long long* solve_ctr;
    unsigned long long* spec_ctr;
    unsigned* rb_done;
    unsigned* rb_solved;
    unsigned* rb_hot;
    int64_t part_stride = 0;
    unsigned long long* tmax;
    void* E = nullptr;
    void* Kn = nullptr;
    int64_t n_ext = 0;
    double *ext_t = nullptr, *ext_n = nullptr, *ext_s = nullptr, *ext_p = nullptr;
    int nblocks = 0, nblocks_override = 0, nchunk = 1, nchunk2 = 1;
    int64_t chunk_len = 0, chunk_len2 = 0, rb_small0 = 0;
    void* xd = nullptr;              // x copies of D (dense), two
    int64_t xbuf = 0;                // elements per shared-memory x buffer
    int64_t xd_stride = 0, rb_stride = 0;
    int hold_cap = 8;                // row chunks a block may hold at once (QDFN_SOLVE_HOLD)
    int pair_solve = 1;              // lane-pair solves in the overlapped phase (QDFN_PAIR_SOLVE=0: one lane)
    int rb_ordered = 1;              // high-velocity row blocks first (QDFN_RB_ORDER=0: index order)
    int c_spec = 64;                 // next-step column chunks streamed in a step's tail (QDFN_SPEC_COLS;
                                     // at most the chunks of a full-width row block, so 64: all of them)
    int spec_stop_pct = 100;         // % of blocks at the barrier that ends early-tile claims (QDFN_SPEC_STOP)
    hmat::Ops hops{};
    std::vector<void*> hbufs;       // H-matrix device buffers
    size_t smem = 0;
    cudaStream_t pending = nullptr;
    int* host_status = nullptr;      // pinned: [0] error flag, [1..] instance status (run completion)
    bool running = false;

    template <class T>
    int dalloc(T** p, size_t n) {
        void* q = nullptr;
        if (cudaMalloc(&q, n * sizeof(T) + 16) != cudaSuccess)
            return fail(QDFN_ERR_NOMEM, "cudaMalloc failed");
        cudaMemset(q, 0, n * sizeof(T) + 16);
        allocs.push_back(q);
        *p = reinterpret_cast<T*>(q);
        return QDFN_OK;
    }
    void release(void* q) {
        if (!q) return;
        auto it = std::find(allocs.begin(), allocs.end(), q);
        if (it != allocs.end()) { cudaFree(q); allocs.erase(it); }
    }
    ~qdfn_ctx() {
        for (void* q : allocs) cudaFree(q);
        if (host_status) cudaFreeHost(host_status);
    }
};

namespace {

// kernel instance count is rounded up to 1, 2, 4; extra instances replicate
// instance 0 and are ignored
int kernel_R(int R) { return R <= 1 ? 1 : R <= 2 ? 2 : 4; }

int h2d(void* dst, const void* src, size_t bytes) {
    QDFN_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return QDFN_OK;
}

SimParams make_params(qdfn_ctx* c, uint64_t budget_ns) {
    SimParams p{};
    p.N = c->N; p.Nload = c->Nload; p.ld = c->ld; p.R = kernel_R(c->R);
    p.evolution_dr = c->prob.evolution_dr; p.interp_at_told = c->prob.interp_at_told; p.hmat = c->hmat;
    p.eta = c->eta; p.sigma_min = c->prob.sigma_min; p.switch_v = c->prob.switch_v;
    p.dt_cut = c->prob.dt_cut; p.rupture_dt = c->prob.rupture_dt; p.max_dt = c->prob.max_dt;
    p.alpha_evo = c->prob.alpha_evo;
    p.record_step = c->prob.record_step; p.max_records = c->prob.max_records;
    p.a = c->a; p.b = c->b; p.Dc = c->Dc; p.F0 = c->F0; p.tau0 = c->tau0; p.sigma0 = c->sigma0;
    p.ra = c->ra; p.rDc = c->rDc;
    p.Vconst = c->Vconst; p.mass = c->mass; p.omega = c->omega; p.kself = c->kself;
    p.unstable = c->unstable; p.has_unstable = c->has_unstable;
    p.n_ext = c->n_ext; p.ext_t = c->ext_t; p.ext_n = c->ext_n; p.ext_s = c->ext_s; p.ext_p = c->ext_p;
    p.E = c->E; p.Kn = c->Kn; p.nchunk = c->nchunk; p.chunk_len = c->chunk_len;
    p.xd = c->xd; p.xbuf = c->xbuf; p.xd_stride = c->xd_stride; p.rb_stride = c->rb_stride;
    p.nchunk2 = c->nchunk2; p.chunk_len2 = c->chunk_len2; p.rb_small0 = c->rb_small0;
    p.V = c->V; p.D = c->D; p.theta = c->theta; p.fric = c->fric; p.accel = c->accel; p.sig_old = c->sig_old;
    p.Vn = c->Vn; p.Dn = c->Dn; p.thn = c->thn; p.fn = c->fn; p.sn = c->sn; p.dtall = c->dtall;
    p.tld = c->tld; p.knd = c->knd; p.instab = c->instab; p.flag = c->flag; p.sw = c->sw;
    p.sw_n = c->sw_n; p.accel_n = c->accel_n;
    p.part_s = c->part_s; p.part_n = c->part_n; p.part_stride = c->part_stride;
    p.spec_ctr = c->spec_ctr; p.rb_solved = c->rb_solved; p.c_spec = c->c_spec; p.rb_hot = c->rb_hot;
    p.spec_stop = std::max(1, (c->nblocks * c->spec_stop_pct + 99) / 100);
    p.T = c->T; p.dt = c->dt; p.step = c->step; p.nrec = c->nrec; p.status = c->status;
    p.hT = c->hT; p.hDt = c->hDt; p.hV = c->hV; p.hD = c->hD; p.hth = c->hth; p.hs = c->hs;
    p.bar_count = c->bar_count; p.bar_gen = c->bar_gen; p.red = c->red; p.gerr = c->gerr;
    p.prof = c->prof;
    p.tile_ctr = c->tile_ctr;
    p.solve_ctr = c->solve_ctr;
    p.rb_done = c->rb_done;
    p.tmax = c->tmax;
    p.hold_cap = c->hold_cap;
    p.pair_solve = c->pair_solve;
    p.rb_ordered = c->rb_ordered;
    p.n_rb = c->ld > 0 ? (c->N + c->ld - 1) / c->ld : 0;
    p.h = c->hops;
    p.budget_ns = budget_ns;
    return p;
}

using SimKernel = void (*)(SimParams, int64_t);
using ApplyKernel = void (*)(SimParams);

template <class M, bool HM>
SimKernel pick_sim(int R) {
    switch (R) {
        case 1: return k_sim<M, 1, HM>;
        case 2: return k_sim<M, 2, HM>;
        default: return k_sim<M, 4, HM>;
    }
}
SimKernel sim_kernel(int prec, int R, bool hm) {
    if (hm) return prec == QDFN_FP64 ? pick_sim<FmtF64, true>(R) : pick_sim<FmtF32, true>(R);
    if (prec == QDFN_FP64) return pick_sim<FmtF64, false>(R);
    if (prec == QDFN_FP32) return pick_sim<FmtF32, false>(R);
    return pick_sim<FmtBF16x2, false>(R);
}
template <class M>
ApplyKernel pick_apply(int R) {
    switch (R) {
        case 1: return k_apply<M, 1>;
        case 2: return k_apply<M, 2>;
        default: return k_apply<M, 4>;
    }
}
ApplyKernel apply_kernel(int prec, int R) {
    if (prec == QDFN_FP64) return pick_apply<FmtF64>(R);
    if (prec == QDFN_FP32) return pick_apply<FmtF32>(R);
    return pick_apply<FmtBF16x2>(R);
}
template <class X>
void hmat_apply_kernels(int R, ApplyKernel* a, ApplyKernel* b, ApplyKernel* rows) {
    switch (R) {
        case 1: *a = k_hmat_a<X, 1>; *b = k_hmat_b<X, 1>; *rows = k_hmat_rows<1>; break;
        case 2: *a = k_hmat_a<X, 2>; *b = k_hmat_b<X, 2>; *rows = k_hmat_rows<2>; break;
        default: *a = k_hmat_a<X, 4>; *b = k_hmat_b<X, 4>; *rows = k_hmat_rows<4>; break;
    }
}

int configure_launch(qdfn_ctx* c) {
    const int Rk = kernel_R(c->R);
    const int vec = c->prec == QDFN_FP64 ? 1 : 2;
    const size_t xsz = c->prec == QDFN_FP64 ? 8 : 4;
    const int dev_sms = num_sms();
    if (dev_sms <= 0) return fail(QDFN_ERR_CUDA, "no CUDA device");
    // the SMs this context's runs may use (qdfn_set_blocks caps them so that
    // several contexts run side by side); the tiling is sized for them
    const int sms = c->nblocks_override > 0 ? std::min(dev_sms, c->nblocks_override) : dev_sms;
    SimKernel k = sim_kernel(c->prec, c->R, c->hmat != 0);
    int64_t want_blocks;
    if (c->hmat) {
        c->smem = (size_t)Rk * hmat::kChunk * xsz + (size_t)hmat::kMaxRank * Rk * sizeof(double);
        c->nchunk = c->nchunk2 = 0;
        c->chunk_len = c->chunk_len2 = c->rb_small0 = 0;
        want_blocks = std::max<int64_t>(c->hops.n_tiles, c->hops.n_lr);
    } else {
        // column chunks of at most 2048 sources staged in shared memory per instance,
        // enough (row block, chunk) tiles for >= 2 per SM
        const int64_t rows_per_blk = (int64_t)kOpThreads * vec;
        const int64_t nrb = (c->N + rows_per_blk - 1) / rows_per_blk;
        // tiles per SM and step before the guided tail (tuning knob QDFN_TILES_PER_SM)
        int64_t tiles_per_sm = 4;
        if (const char* e = std::getenv("QDFN_TILES_PER_SM")) tiles_per_sm = std::max(1, std::min(64, std::atoi(e)));
        if (const char* e = std::getenv("QDFN_SOLVE_HOLD")) c->hold_cap = std::max(1, std::min(64, std::atoi(e)));
        if (const char* e = std::getenv("QDFN_PAIR_SOLVE")) c->pair_solve = std::atoi(e) != 0 ? 1 : 0;
        if (const char* e = std::getenv("QDFN_RB_ORDER")) c->rb_ordered = std::atoi(e) != 0 ? 1 : 0;
        if (const char* e = std::getenv("QDFN_SPEC_COLS")) c->c_spec = std::max(0, std::min(64, std::atoi(e)));
        if (const char* e = std::getenv("QDFN_SPEC_STOP")) c->spec_stop_pct = std::max(1, std::min(100, std::atoi(e)));
        int64_t want_chunks = std::max<int64_t>(1, (tiles_per_sm * sms + nrb - 1) / nrb);
        int64_t clen = (c->N + want_chunks - 1) / want_chunks;
        // two x buffers (R x chunk x elem each) share the 227 KB with the 192 KB stage ring
        const int64_t cmax = std::max<int64_t>(64, (int64_t)(15 * 1024) / (Rk * (int64_t)xsz));
        clen = (std::min<int64_t>(std::max<int64_t>(clen, 64), std::min<int64_t>(2048, cmax)) + 7) / 8 * 8;
        c->chunk_len = clen;
        c->nchunk = (int)((c->N + clen - 1) / clen);
        // the row blocks of the last two waves of tiles are streamed by their own
        // step only, in tiles of 1/tail_div of the width (QDFN_TAIL_DIV; 1 by
        // default: full width; 0: no such row blocks, every row block open to
        // the next step's early tiles)
        int64_t tail_div = 1;
        if (const char* e = std::getenv("QDFN_TAIL_DIV")) tail_div = std::max(0, std::min(16, std::atoi(e)));
        const int64_t td = std::max<int64_t>(1, tail_div);
        c->chunk_len2 = std::max<int64_t>(8, ((clen + td - 1) / td + 7) / 8 * 8);
        c->nchunk2 = (int)((c->N + c->chunk_len2 - 1) / c->chunk_len2);
        int64_t waves = 2;   // (QDFN_TAIL_WAVES)
        if (const char* e = std::getenv("QDFN_TAIL_WAVES")) waves = std::max(1, std::min(16, std::atoi(e)));
        const int64_t nsmall =
            tail_div == 0 ? 0 : std::min<int64_t>(nrb, (waves * sms + c->nchunk2 - 1) / c->nchunk2);
        c->rb_small0 = nrb - nsmall;
        // one x buffer: the chunk's columns rounded up to 4 (bulk copies move
        // multiples of 16 bytes), in 128-byte units
        c->xbuf = (((clen + 3) / 4 * 4) * Rk * (int64_t)xsz + 127) / 128 * 128 / (int64_t)xsz;
        c->smem = (size_t)kPipeBytes + kMbarBytes + 2 * (size_t)c->xbuf * xsz;
        want_blocks = (nrb - nsmall) * c->nchunk + nsmall * c->nchunk2;
    }
    QDFN_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->smem));
    int occ = 0;
    QDFN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kSimThreads, c->smem));
    if (occ < 1) return fail(QDFN_ERR_CUDA, "simulation kernel cannot be resident");
    const int64_t work_items = (int64_t)Rk * c->N;
    int64_t nb = std::min<int64_t>((int64_t)sms * occ, std::max<int64_t>(1, want_blocks));
    nb = std::max<int64_t>(1, std::min<int64_t>(nb, std::max<int64_t>((work_items + 31) / 32, 1)));
    if (c->nblocks_override > 0) nb = std::min<int64_t>(nb, c->nblocks_override);
    c->nblocks = (int)nb;
    if (c->hmat) {
        ApplyKernel a, b, rows;
        if (c->prec == QDFN_FP64) hmat_apply_kernels<double>(Rk, &a, &b, &rows);
        else hmat_apply_kernels<float>(Rk, &a, &b, &rows);
        QDFN_CUDA(cudaFuncSetAttribute(a, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->smem));
        QDFN_CUDA(cudaFuncSetAttribute(b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->smem));
    } else {
        ApplyKernel ka = apply_kernel(c->prec, c->R);
        QDFN_CUDA(cudaFuncSetAttribute(ka, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->smem));
    }
    c->release(c->part_s);
    c->release(c->part_n);
    c->release(c->red);
    c->part_s = c->part_n = nullptr;
    int rc;
    if (!c->hmat) {
        c->release(c->xd);
        c->xd = nullptr;
        // x copy of D: N columns padded to a multiple of 8 (+8), read in runs of 4
        // elements per x copy (two: current and next step), a multiple of 32 so
        // that the second copy starts 16-byte aligned like the first (bulk copies
        // need 16-byte aligned sources)
        c->xd_stride = (((int64_t)c->N + 16) * Rk + 31) / 32 * 32;
        if ((rc = c->dalloc(reinterpret_cast<unsigned char**>(&c->xd), 2 * (size_t)c->xd_stride * xsz))) return rc;
        if ((reinterpret_cast<uintptr_t>(c->xd) | (uintptr_t)(c->xd_stride * xsz)) % 16 != 0)
            return fail(QDFN_ERR_INVALID, "x copy of D not 16-byte aligned");
        const size_t slots = (size_t)std::max(c->nchunk, c->nchunk2);
        c->part_stride = (int64_t)slots * Rk * c->N;   // two buffers: this step's and the next's
        if ((rc = c->dalloc(&c->part_s, 2 * (size_t)c->part_stride))) return rc;
        if ((rc = c->dalloc(&c->part_n, 2 * (size_t)c->part_stride))) return rc;
    }
    if ((rc = c->dalloc(&c->red, (size_t)2 * c->nblocks * Rk * kRedSlots))) return rc;
    return QDFN_OK;
}

}  // namespace

extern "C" int qdfn_ctx_create(qdfn_ctx** out, const qdfn_problem* pr) {
    if (!out || !pr) return fail(QDFN_ERR_INVALID, "null argument");
    *out = nullptr;
    const int64_t N = pr->N;
    if (N < 1) return fail(QDFN_ERR_INVALID, "N must be >= 1");
    if (pr->Nload < 0 || pr->Nload > N) return fail(QDFN_ERR_INVALID, "Nload out of range");
    if (pr->n_inst < 1 || pr->n_inst > kMaxInst) return fail(QDFN_ERR_INVALID, "n_inst must be 1..4");
    if (!pr->a || !pr->b || !pr->Dc || !pr->theta_i || !pr->V_i || !pr->f_i || !pr->sigma0 ||
        !pr->V_const || !pr->mass)
        return fail(QDFN_ERR_INVALID, "null per-patch array");
    if (pr->record_step < 0 || pr->max_records < 0) return fail(QDFN_ERR_INVALID, "negative record sizes");
    if (!(pr->G > 0) || !(pr->rho > 0)) return fail(QDFN_ERR_INVALID, "G and rho must be positive");
    auto* c = new qdfn_ctx();
    c->N = N; c->Nload = pr->Nload; c->R = pr->n_inst; c->prob = *pr;
    c->eta = pr->G / 2 / std::sqrt(pr->G / pr->rho);
    const int Rk = kernel_R(c->R);
    const size_t RN = (size_t)Rk * N;
    int rc = 0;
#define A(ptr, n) if (!rc) rc = c->dalloc(&c->ptr, n)
    A(a, RN); A(b, RN); A(Dc, RN); A(F0, RN); A(tau0, RN); A(sigma0, RN); A(Vconst, RN);
    A(ra, RN); A(rDc, RN);
    A(mass, RN); A(omega, RN); A(kself, (size_t)N); A(unstable, RN); A(has_unstable, (size_t)Rk);
    // the six host-visible state fields in one block, in the order of the
    // state-transfer calls, so that contiguous host buffers move in one copy
    double* state6 = nullptr;
    if (!rc) rc = c->dalloc(&state6, 6 * RN);
    if (!rc) {
        c->V = state6; c->D = state6 + RN; c->theta = state6 + 2 * RN;
        c->fric = state6 + 3 * RN; c->accel = state6 + 4 * RN; c->sig_old = state6 + 5 * RN;
    }
    A(Vn, RN); A(Dn, RN); A(thn, RN); A(fn, RN); A(sn, RN); A(dtall, RN); A(tld, RN); A(knd, RN);
    A(instab, RN); A(flag, RN); A(sw, RN); A(sw_n, RN); A(accel_n, RN);
    double* Tdt = nullptr;           // T and dt side by side, for the same reason
    if (!rc) rc = c->dalloc(&Tdt, 2 * (size_t)Rk);
    if (!rc) { c->T = Tdt; c->dt = Tdt + Rk; }
    A(step, (size_t)Rk); A(nrec, (size_t)Rk); A(status, (size_t)Rk);
    const size_t hr = (size_t)Rk * std::max<int64_t>(pr->max_records, 1);
    A(hT, hr); A(hDt, hr); A(hV, hr * N); A(hD, hr * N); A(hth, hr * N); A(hs, hr * N);
    // launch control words side by side: [0] error flag, [1] barrier arrivals,
    // [2] barrier generation -- the first two are cleared by one memset per launch
    int* ctrl = nullptr;
    if (!rc) rc = c->dalloc(&ctrl, 4);
    if (!rc) {
        c->gerr = ctrl;
        c->bar_count = reinterpret_cast<unsigned*>(ctrl + 1);
        c->bar_gen = reinterpret_cast<unsigned*>(ctrl + 2);
    }
    A(prof, kCounters); A(tile_ctr, kSets); A(spec_ctr, kSets);
    // per-step counters, kSets sets used by steps in turn (a step uses one, streams
    // ahead into the next, and resets the one two ahead)
    c->rb_stride = (N + kOpThreads - 1) / kOpThreads;   // row blocks have >= kOpThreads rows
    A(solve_ctr, kSets); A(tmax, 4 * kSets); A(rb_done, kSets * (size_t)c->rb_stride);
    A(rb_solved, kSets * (size_t)c->rb_stride); A(rb_hot, kSets * (size_t)c->rb_stride);
#undef A
    if (rc) { delete c; return rc; }
    // host-side initialisation (Main_D :41-131): padded instances replicate instance 0
    std::vector<double> ha(RN), hb(RN), hDc(RN), hF0(RN), htau0(RN), hs0(RN), hVc(RN), hm(RN),
        hth(RN), hV(RN), hf(RN), hzero(RN, 0.0);
    std::vector<unsigned char> hun(RN);
    std::vector<int> hhas(Rk, 0);
    for (int r = 0; r < Rk; ++r) {
        const int src = r < c->R ? r : 0;
        for (int64_t i = 0; i < N; ++i) {
            const size_t q = (size_t)r * N + i, s = (size_t)src * N + i;
            ha[q] = pr->a[s]; hb[q] = pr->b[s]; hDc[q] = pr->Dc[s];
            hth[q] = pr->theta_i[s]; hV[q] = pr->V_i[s]; hf[q] = pr->f_i[s];
            hs0[q] = pr->sigma0[s]; hVc[q] = pr->V_const[s]; hm[q] = pr->mass[s];
            if (pr->V_i[s] / sim::kV0 < 0 || pr->theta_i[s] * sim::kV0 / pr->Dc[s] < 0) {
                delete c;
                return fail(QDFN_ERR_DOMAIN, "log of a negative number in Friction0");
            }
            hF0[q] = pr->f_i[s] - pr->a[s] * std::log(pr->V_i[s] / sim::kV0) -
                     pr->b[s] * std::log(pr->theta_i[s] * sim::kV0 / pr->Dc[s]);
            htau0[q] = pr->sigma0[s] * pr->f_i[s];
            hun[q] = (pr->a[s] - pr->b[s] < 0) ? 1 : 0;
            if (hun[q]) hhas[r] = 1;
        }
    }
    // the solvers divide by a and Dc through their reciprocals: IEEE 1/x,
    // correctly rounded here as on the device
    std::vector<double> hra(RN), hrDc(RN);
    for (size_t q = 0; q < RN; ++q) { hra[q] = 1.0 / ha[q]; hrDc[q] = 1.0 / hDc[q]; }
    std::vector<double> ones(Rk, 1.0), zeros(Rk, 0.0);
    std::vector<int64_t> z64(Rk, 0);
    std::vector<int> z32(Rk, 0);
    if ((rc = h2d(c->a, ha.data(), RN * 8)) || (rc = h2d(c->b, hb.data(), RN * 8)) ||
        (rc = h2d(c->ra, hra.data(), RN * 8)) || (rc = h2d(c->rDc, hrDc.data(), RN * 8)) ||
        (rc = h2d(c->Dc, hDc.data(), RN * 8)) || (rc = h2d(c->F0, hF0.data(), RN * 8)) ||
        (rc = h2d(c->tau0, htau0.data(), RN * 8)) || (rc = h2d(c->sigma0, hs0.data(), RN * 8)) ||
        (rc = h2d(c->Vconst, hVc.data(), RN * 8)) || (rc = h2d(c->mass, hm.data(), RN * 8)) ||
        (rc = h2d(c->unstable, hun.data(), RN)) || (rc = h2d(c->has_unstable, hhas.data(), Rk * 4)) ||
        (rc = h2d(c->V, hV.data(), RN * 8)) || (rc = h2d(c->theta, hth.data(), RN * 8)) ||
        (rc = h2d(c->fric, hf.data(), RN * 8)) || (rc = h2d(c->sig_old, hs0.data(), RN * 8)) ||
        (rc = h2d(c->D, hzero.data(), RN * 8)) || (rc = h2d(c->accel, hzero.data(), RN * 8)) ||
        (rc = h2d(c->T, zeros.data(), Rk * 8)) || (rc = h2d(c->dt, ones.data(), Rk * 8)) ||
        (rc = h2d(c->step, z64.data(), Rk * 8)) || (rc = h2d(c->nrec, z64.data(), Rk * 8)) ||
        (rc = h2d(c->status, z32.data(), Rk * 4))) {
        delete c;
        return rc;
    }
    *out = c;
    return QDFN_OK;
}

extern "C" int qdfn_ctx_destroy(qdfn_ctx* ctx) {
    if (!ctx) return QDFN_OK;
    if (ctx->running) cudaStreamSynchronize(ctx->pending);
    delete ctx;
    return QDFN_OK;
}

namespace {

void release_hmat(qdfn_ctx* c);

// Converts FP64 Ks/Kn already on the device into the stored operator.
int set_dense_device(qdfn_ctx* c, const double* dKs, const double* dKn, int64_t ld_in, int layout,
                     int precision, cudaStream_t st) {
    const int64_t N = c->N;
    release_hmat(c);
    c->release(c->E);
    c->release(c->Kn);
    c->E = c->Kn = nullptr;
    c->prec = precision;
    c->hmat = 0;
    // ld holds the tile height (rows per block): 16 bytes per thread row group
    const size_t esz = precision == QDFN_FP64 ? 8 : 4;
    c->ld = (int64_t)kOpThreads * (int64_t)(kGranule / esz);   // operator row block
    const int64_t nrows = (N + c->ld - 1) / c->ld * c->ld;
    const size_t mbytes = (size_t)N * nrows * esz;
    unsigned char *dE = nullptr, *dK = nullptr;
    int rc = c->dalloc(&dE, mbytes);
    if (!rc) rc = c->dalloc(&dK, mbytes);
    if (rc) return rc;
    c->E = dE;
    c->Kn = dK;
    dim3 grid((unsigned)((nrows + 255) / 256), (unsigned)std::min<int64_t>(N, 65535));
    k_convert<<<grid, 256, 0, st>>>(dKs, dKn, N, ld_in, layout, c->ld, precision, c->E, c->Kn, c->kself);
    QDFN_CUDA(cudaGetLastError());
    QDFN_CUDA(cudaStreamSynchronize(st));
    // Omega = sqrt(K_Self / M) (Main_D :56); K_ii = 0 cannot normalise a row
    std::vector<double> ks(N), m((size_t)kernel_R(c->R) * N), om(m.size());
    QDFN_CUDA(cudaMemcpy(ks.data(), c->kself, N * 8, cudaMemcpyDeviceToHost));
    QDFN_CUDA(cudaMemcpy(m.data(), c->mass, m.size() * 8, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < N; ++i)
        if (ks[i] == 0.0) return fail(QDFN_ERR_INVALID, "zero self stiffness K_ii");
    for (size_t q = 0; q < m.size(); ++q) {
        const double x = ks[q % N] / m[q];
        if (x < 0) return fail(QDFN_ERR_DOMAIN, "sqrt of a negative number in Omega");
        om[q] = std::sqrt(x);
    }
    if ((rc = h2d(c->omega, om.data(), om.size() * 8))) return rc;
    return configure_launch(c);
}

int check_dense_args(qdfn_ctx* c, const void* Ks, const void* Kn, int64_t ld_in, int layout, int precision) {
    if (!c || !Ks || !Kn) return fail(QDFN_ERR_INVALID, "null argument");
    if (precision != QDFN_FP64 && precision != QDFN_FP32 && precision != QDFN_BF16X2)
        return fail(QDFN_ERR_INVALID, "unknown precision");
    if (layout != QDFN_LAYOUT_ROW && layout != QDFN_LAYOUT_COL)
        return fail(QDFN_ERR_INVALID, "unknown layout");
    if (ld_in < c->N) return fail(QDFN_ERR_INVALID, "ld < N");
    return QDFN_OK;
}

}  // namespace

extern "C" int qdfn_set_dense(qdfn_ctx* c, const double* Ks, const double* Kn, int64_t ld_in,
                              int layout, int precision) {
    int rc = check_dense_args(c, Ks, Kn, ld_in, layout, precision);
    if (rc) return rc;
    const int64_t N = c->N;
    double *tS = nullptr, *tN = nullptr;
    const size_t inbytes = (size_t)N * ld_in * sizeof(double);
    if (cudaMalloc(&tS, inbytes) != cudaSuccess) return fail(QDFN_ERR_NOMEM, "staging buffer");
    if (cudaMalloc(&tN, inbytes) != cudaSuccess) { cudaFree(tS); return fail(QDFN_ERR_NOMEM, "staging buffer"); }
    cudaError_t e1 = cudaMemcpy(tS, Ks, inbytes, cudaMemcpyHostToDevice);
    cudaError_t e2 = cudaMemcpy(tN, Kn, inbytes, cudaMemcpyHostToDevice);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
        cudaFree(tS); cudaFree(tN);
        return cuda_fail(e1 != cudaSuccess ? e1 : e2, "cudaMemcpy (set_dense)");
    }
    rc = set_dense_device(c, tS, tN, ld_in, layout, precision, nullptr);
    cudaFree(tS);
    cudaFree(tN);
    return rc;
}

extern "C" int qdfn_set_dense_dev(qdfn_ctx* c, const double* Ks, const double* Kn, int64_t ld_in,
                                  int layout, int precision, void* stream) {
    int rc = check_dense_args(c, Ks, Kn, ld_in, layout, precision);
    if (rc) return rc;
    return set_dense_device(c, Ks, Kn, ld_in, layout, precision, (cudaStream_t)stream);
}

extern "C" int qdfn_set_external_stress(qdfn_ctx* c, int64_t nt, const double* t,
                                        const double* dsn, const double* dtau, const double* dp) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (nt < 0) return fail(QDFN_ERR_INVALID, "nt < 0");
    c->release(c->ext_t); c->release(c->ext_n); c->release(c->ext_s); c->release(c->ext_p);
    c->ext_t = c->ext_n = c->ext_s = c->ext_p = nullptr;
    c->n_ext = 0;
    if (nt == 0) return QDFN_OK;
    if (!t || !dsn || !dtau || !dp) return fail(QDFN_ERR_INVALID, "null external-stress array");
    int rc;
    const size_t n = (size_t)nt * c->N;
    if ((rc = c->dalloc(&c->ext_t, nt)) || (rc = c->dalloc(&c->ext_n, n)) ||
        (rc = c->dalloc(&c->ext_s, n)) || (rc = c->dalloc(&c->ext_p, n)))
        return rc;
    if ((rc = h2d(c->ext_t, t, nt * 8)) || (rc = h2d(c->ext_n, dsn, n * 8)) ||
        (rc = h2d(c->ext_s, dtau, n * 8)) || (rc = h2d(c->ext_p, dp, n * 8)))
        return rc;
    c->n_ext = nt;
    return QDFN_OK;
}

extern "C" int qdfn_run_async(qdfn_ctx* c, int64_t nsteps, double timeout_s, void* stream) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (c->prec < 0) return fail(QDFN_ERR_STATE, "no operator set (qdfn_set_dense first)");
    if (nsteps < 0) return fail(QDFN_ERR_INVALID, "nsteps < 0");
    if (nsteps == 0) return QDFN_OK;
    const double budget = timeout_s > 0 ? timeout_s : 1e6;
    const uint64_t budget_ns = (uint64_t)(budget * 1e9);
    cudaStream_t st = (cudaStream_t)stream;
    // error flag and barrier arrivals (adjacent); the kernel resets its own counters
    QDFN_CUDA(cudaMemsetAsync(c->gerr, 0, 2 * sizeof(int), st));
    SimParams p = make_params(c, budget_ns);
    SimKernel k = sim_kernel(c->prec, c->R, c->hmat != 0);
    void* args[] = {&p, &nsteps};
    QDFN_CUDA(cudaLaunchCooperativeKernel((const void*)k, dim3(c->nblocks), dim3(kSimThreads), args,
                                          c->smem, st));
    c->pending = st;
    c->running = true;
    return QDFN_OK;
}

extern "C" int qdfn_sync(qdfn_ctx* c) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (!c->running) return QDFN_OK;
    c->running = false;
    QDFN_CUDA(cudaStreamSynchronize(c->pending));
    int gerr = 0;
    QDFN_CUDA(cudaMemcpy(&gerr, c->gerr, sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<int> st(kernel_R(c->R));
    QDFN_CUDA(cudaMemcpy(st.data(), c->status, st.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (int r = 0; r < c->R; ++r)
        if (st[r] != 0) return fail(st[r], "instance " + std::to_string(r) + " stopped");
    if (gerr != 0) return fail(gerr, "device loop stopped early");
    return QDFN_OK;
}

extern "C" int qdfn_run(qdfn_ctx* c, int64_t nsteps, double timeout_s) {
    int rc = qdfn_run_async(c, nsteps, timeout_s, nullptr);
    if (rc) return rc;
    return qdfn_sync(c);
}

extern "C" int qdfn_kernels_per_run(const qdfn_ctx* c) { return c ? 1 : 0; }

extern "C" int qdfn_set_blocks(qdfn_ctx* c, int nblocks) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (nblocks < 0) return fail(QDFN_ERR_INVALID, "nblocks < 0");
    if (c->running) return fail(QDFN_ERR_STATE, "a run is in flight");
    c->nblocks_override = nblocks;
    return c->prec < 0 ? QDFN_OK : configure_launch(c);
}

extern "C" int qdfn_get_blocks(const qdfn_ctx* c) { return c ? c->nblocks : -1; }

extern "C" int qdfn_get_counters(const qdfn_ctx* c, int64_t* out, int n) {
    if (!c || !out || n < 0) return fail(QDFN_ERR_INVALID, "null argument");
    unsigned long long v[kCounters];
    QDFN_CUDA(cudaMemcpy(v, c->prof, sizeof(v), cudaMemcpyDeviceToHost));
    for (int k = 0; k < n && k < kCounters; ++k) out[k] = (int64_t)v[k];
    return QDFN_OK;
}

extern "C" int qdfn_get_state(const qdfn_ctx* c, int inst, double* V, double* D, double* theta,
                              double* friction, double* accel, double* sigma_old, double* T,
                              double* dt, int64_t* step) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (inst < 0 || inst >= c->R) return fail(QDFN_ERR_INVALID, "instance out of range");
    const size_t off = (size_t)inst * c->N, n = (size_t)c->N * 8;
    if (V) QDFN_CUDA(cudaMemcpy(V, c->V + off, n, cudaMemcpyDeviceToHost));
    if (D) QDFN_CUDA(cudaMemcpy(D, c->D + off, n, cudaMemcpyDeviceToHost));
    if (theta) QDFN_CUDA(cudaMemcpy(theta, c->theta + off, n, cudaMemcpyDeviceToHost));
    if (friction) QDFN_CUDA(cudaMemcpy(friction, c->fric + off, n, cudaMemcpyDeviceToHost));
    if (accel) QDFN_CUDA(cudaMemcpy(accel, c->accel + off, n, cudaMemcpyDeviceToHost));
    if (sigma_old) QDFN_CUDA(cudaMemcpy(sigma_old, c->sig_old + off, n, cudaMemcpyDeviceToHost));
    if (T) QDFN_CUDA(cudaMemcpy(T, c->T + inst, 8, cudaMemcpyDeviceToHost));
    if (dt) QDFN_CUDA(cudaMemcpy(dt, c->dt + inst, 8, cudaMemcpyDeviceToHost));
    if (step) QDFN_CUDA(cudaMemcpy(step, c->step + inst, 8, cudaMemcpyDeviceToHost));
    return QDFN_OK;
}

extern "C" int qdfn_set_state(qdfn_ctx* c, int inst, const double* V, const double* D,
                              const double* theta, const double* friction, const double* accel,
                              const double* sigma_old, double T, double dt, int64_t step) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (inst < 0 || inst >= c->R) return fail(QDFN_ERR_INVALID, "instance out of range");
    const size_t off = (size_t)inst * c->N, n = (size_t)c->N * 8;
    if (V) QDFN_CUDA(cudaMemcpy(c->V + off, V, n, cudaMemcpyHostToDevice));
    if (D) QDFN_CUDA(cudaMemcpy(c->D + off, D, n, cudaMemcpyHostToDevice));
    if (theta) QDFN_CUDA(cudaMemcpy(c->theta + off, theta, n, cudaMemcpyHostToDevice));
    if (friction) QDFN_CUDA(cudaMemcpy(c->fric + off, friction, n, cudaMemcpyHostToDevice));
    if (accel) QDFN_CUDA(cudaMemcpy(c->accel + off, accel, n, cudaMemcpyHostToDevice));
    if (sigma_old) QDFN_CUDA(cudaMemcpy(c->sig_old + off, sigma_old, n, cudaMemcpyHostToDevice));
    QDFN_CUDA(cudaMemcpy(c->T + inst, &T, 8, cudaMemcpyHostToDevice));
    QDFN_CUDA(cudaMemcpy(c->dt + inst, &dt, 8, cudaMemcpyHostToDevice));
    QDFN_CUDA(cudaMemcpy(c->step + inst, &step, 8, cudaMemcpyHostToDevice));
    return QDFN_OK;
}

namespace {
// Field copies of a state transfer; a field whose device and host buffers both
// follow the previous one's (device fields are `dstride` bytes apart, host
// buffers are packed: the caller's arrays for consecutive fields end to end)
// joins its copy, so packed host buffers move in one copy per direction.
struct CopyList {
    struct Run { char* dev; char* host; size_t bytes, dstride; int nf; };
    Run runs[9];
    int n = 0;
    void add(void* dev, const void* host, size_t bytes, size_t dstride) {
        if (!host) return;
        char* d = (char*)dev;
        char* h = (char*)const_cast<void*>(host);
        if (n > 0) {
            Run& r = runs[n - 1];
            if (r.dstride == bytes && r.bytes == bytes * r.nf && d == r.dev + bytes * r.nf &&
                h == r.host + bytes * r.nf) {   // both sides continue the run
                r.nf++;
                r.bytes += bytes;
                return;
            }
        }
        runs[n++] = Run{d, h, bytes, dstride, 1};
    }
    int run(cudaMemcpyKind kind, cudaStream_t st) {
        for (int k = 0; k < n; ++k) {
            const Run& r = runs[k];
            if (kind == cudaMemcpyHostToDevice) QDFN_CUDA(cudaMemcpyAsync(r.dev, r.host, r.bytes, kind, st));
            else QDFN_CUDA(cudaMemcpyAsync(r.host, r.dev, r.bytes, kind, st));
        }
        return QDFN_OK;
    }
};
}  // namespace

extern "C" int qdfn_set_state_all(qdfn_ctx* c, const double* V, const double* D, const double* theta,
                                  const double* friction, const double* accel, const double* sigma_old,
                                  const double* T, const double* dt, const int64_t* step, void* stream) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (c->running) return fail(QDFN_ERR_STATE, "a run is in flight (qdfn_sync or qdfn_get_state_all first)");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = (size_t)c->R * c->N * 8, ns = (size_t)c->R * 8;
    const size_t rn = (size_t)kernel_R(c->R) * c->N * 8, rs = (size_t)kernel_R(c->R) * 8;
    CopyList cl;
    cl.add(c->V, V, n, rn); cl.add(c->D, D, n, rn); cl.add(c->theta, theta, n, rn);
    cl.add(c->fric, friction, n, rn); cl.add(c->accel, accel, n, rn); cl.add(c->sig_old, sigma_old, n, rn);
    cl.add(c->T, T, ns, rs); cl.add(c->dt, dt, ns, rs); cl.add(c->step, step, ns, rs);
    return cl.run(cudaMemcpyHostToDevice, st);
}

extern "C" int qdfn_get_state_all(qdfn_ctx* c, double* V, double* D, double* theta, double* friction,
                                  double* accel, double* sigma_old, double* T, double* dt, int64_t* step,
                                  void* stream, int wait) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    cudaStream_t st = (cudaStream_t)stream;
    const bool completes = c->running && c->pending == st;
    if (c->running && !completes) return fail(QDFN_ERR_STATE, "the run in flight is on another stream");
    if (completes && !wait) return fail(QDFN_ERR_INVALID, "reading the state of a run in flight needs wait=1");
    const size_t n = (size_t)c->R * c->N * 8, ns = (size_t)c->R * 8;
    const size_t rn = (size_t)kernel_R(c->R) * c->N * 8, rs = (size_t)kernel_R(c->R) * 8;
    CopyList cl;
    cl.add(c->V, V, n, rn); cl.add(c->D, D, n, rn); cl.add(c->theta, theta, n, rn);
    cl.add(c->fric, friction, n, rn); cl.add(c->accel, accel, n, rn); cl.add(c->sig_old, sigma_old, n, rn);
    cl.add(c->T, T, ns, rs); cl.add(c->dt, dt, ns, rs); cl.add(c->step, step, ns, rs);
    if (int rc = cl.run(cudaMemcpyDeviceToHost, st)) return rc;
    if (completes) {   // the run's outcome travels with the state: one synchronisation
        if (!c->host_status) QDFN_CUDA(cudaHostAlloc(&c->host_status, (1 + kMaxInst) * sizeof(int), 0));
        QDFN_CUDA(cudaMemcpyAsync(c->host_status, c->gerr, sizeof(int), cudaMemcpyDeviceToHost, st));
        QDFN_CUDA(cudaMemcpyAsync(c->host_status + 1, c->status, c->R * sizeof(int), cudaMemcpyDeviceToHost, st));
    }
    if (!wait) return QDFN_OK;
    QDFN_CUDA(cudaStreamSynchronize(st));
    if (completes) {
        c->running = false;
        for (int r = 0; r < c->R; ++r)
            if (c->host_status[1 + r] != 0)
                return fail(c->host_status[1 + r], "instance " + std::to_string(r) + " stopped");
        if (c->host_status[0] != 0) return fail(c->host_status[0], "device loop stopped early");
    }
    return QDFN_OK;
}

extern "C" int qdfn_get_history(const qdfn_ctx* c, int inst, double* T, double* Dt, double* V,
                                double* D, double* theta, double* sigma, int64_t* nrec) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (inst < 0 || inst >= c->R) return fail(QDFN_ERR_INVALID, "instance out of range");
    int64_t n = 0;
    QDFN_CUDA(cudaMemcpy(&n, c->nrec + inst, 8, cudaMemcpyDeviceToHost));
    if (nrec) *nrec = n;
    if (n == 0) return QDFN_OK;
    const size_t off1 = (size_t)inst * c->prob.max_records;
    const size_t offN = off1 * c->N;
    const size_t bytesN = (size_t)n * c->N * 8;
    if (T) QDFN_CUDA(cudaMemcpy(T, c->hT + off1, n * 8, cudaMemcpyDeviceToHost));
    if (Dt) QDFN_CUDA(cudaMemcpy(Dt, c->hDt + off1, n * 8, cudaMemcpyDeviceToHost));
    if (V) QDFN_CUDA(cudaMemcpy(V, c->hV + offN, bytesN, cudaMemcpyDeviceToHost));
    if (D) QDFN_CUDA(cudaMemcpy(D, c->hD + offN, bytesN, cudaMemcpyDeviceToHost));
    if (theta) QDFN_CUDA(cudaMemcpy(theta, c->hth + offN, bytesN, cudaMemcpyDeviceToHost));
    if (sigma) QDFN_CUDA(cudaMemcpy(sigma, c->hs + offN, bytesN, cudaMemcpyDeviceToHost));
    return QDFN_OK;
}

extern "C" int qdfn_apply_operator(qdfn_ctx* c, const double* D, double* tld, double* knd) {
    if (!c || !D || !tld || !knd) return fail(QDFN_ERR_INVALID, "null argument");
    if (c->prec < 0) return fail(QDFN_ERR_STATE, "no operator set");
    const size_t n = (size_t)c->R * c->N * 8;
    std::vector<double> saved(n / 8);
    QDFN_CUDA(cudaMemcpy(saved.data(), c->D, n, cudaMemcpyDeviceToHost));
    QDFN_CUDA(cudaMemcpy(c->D, D, n, cudaMemcpyHostToDevice));
    SimParams p = make_params(c, 0);
    const int64_t tot = (int64_t)kernel_R(c->R) * c->N;
    if (c->hmat) {
        ApplyKernel a, b, rows;
        if (c->prec == QDFN_FP64) hmat_apply_kernels<double>(kernel_R(c->R), &a, &b, &rows);
        else hmat_apply_kernels<float>(kernel_R(c->R), &a, &b, &rows);
        a<<<c->nblocks, kSimThreads, c->smem>>>(p);
        QDFN_CUDA(cudaGetLastError());
        b<<<c->nblocks, kSimThreads, c->smem>>>(p);
        QDFN_CUDA(cudaGetLastError());
        rows<<<(unsigned)((tot + 255) / 256), 256>>>(p);
        QDFN_CUDA(cudaGetLastError());
    } else {
        QDFN_CUDA(cudaMemset(c->tile_ctr, 0, sizeof(unsigned long long)));
        const unsigned fb = (unsigned)((tot + 255) / 256);
        switch ((c->prec == QDFN_FP64 ? 10 : 0) + kernel_R(c->R)) {
            case 1: k_fill_xd<float, 1><<<fb, 256>>>(p); break;
            case 2: k_fill_xd<float, 2><<<fb, 256>>>(p); break;
            case 4: k_fill_xd<float, 4><<<fb, 256>>>(p); break;
            case 11: k_fill_xd<double, 1><<<fb, 256>>>(p); break;
            case 12: k_fill_xd<double, 2><<<fb, 256>>>(p); break;
            default: k_fill_xd<double, 4><<<fb, 256>>>(p); break;
        }
        QDFN_CUDA(cudaGetLastError());
        apply_kernel(c->prec, c->R)<<<c->nblocks, kSimThreads, c->smem>>>(p);
        QDFN_CUDA(cudaGetLastError());
        if (c->prec == QDFN_FP64) k_chunk_reduce<false><<<(unsigned)((tot + 255) / 256), 256>>>(p);
        else k_chunk_reduce<true><<<(unsigned)((tot + 255) / 256), 256>>>(p);
        QDFN_CUDA(cudaGetLastError());
    }
    QDFN_CUDA(cudaDeviceSynchronize());
    QDFN_CUDA(cudaMemcpy(tld, c->tld, n, cudaMemcpyDeviceToHost));
    QDFN_CUDA(cudaMemcpy(knd, c->knd, n, cudaMemcpyDeviceToHost));
    QDFN_CUDA(cudaMemcpy(c->D, saved.data(), n, cudaMemcpyHostToDevice));
    return QDFN_OK;
}

extern "C" int qdfn_get_kself(const qdfn_ctx* c, double* kself) {
    if (!c || !kself) return fail(QDFN_ERR_INVALID, "null argument");
    if (c->prec < 0) return fail(QDFN_ERR_STATE, "no operator set");
    QDFN_CUDA(cudaMemcpy(kself, c->kself, c->N * 8, cudaMemcpyDeviceToHost));
    return QDFN_OK;
}

namespace {

template <class T>
void put(std::vector<unsigned char>& buf, size_t off_elems, double v) {
    reinterpret_cast<T*>(buf.data())[off_elems] = (T)v;
}

void release_hmat(qdfn_ctx* c) {
    for (void* q : c->hbufs) c->release(q);
    c->hbufs.clear();
    c->hops = hmat::Ops{};
}

template <class T>
int dcopy(qdfn_ctx* c, const T* src, size_t n, T** dst) {
    int rc = c->dalloc(dst, n);
    if (rc) return rc;
    c->hbufs.push_back(*dst);
    if (n) QDFN_CUDA(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return QDFN_OK;
}

}  // namespace

extern "C" int qdfn_set_hmatrix(qdfn_ctx* c, int64_t nb, const int64_t* range, const int64_t* rank_s,
                                const double* const* U_s, const double* const* Vt_s,
                                const double* const* D_s, const int64_t* rank_n,
                                const double* const* U_n, const double* const* Vt_n,
                                const double* const* D_n, int precision) {
    if (!c || !range || !rank_s || !rank_n) return fail(QDFN_ERR_INVALID, "null argument");
    if (nb < 1) return fail(QDFN_ERR_INVALID, "nb must be >= 1");
    if (precision != QDFN_FP64 && precision != QDFN_FP32)
        return fail(QDFN_ERR_INVALID, "H-matrix blocks are stored in QDFN_FP64 or QDFN_FP32");
    const int64_t N = c->N;
    const int Rk = kernel_R(c->R);
    const size_t esz = precision == QDFN_FP64 ? 8 : 4;
    // validate and lay out
    std::vector<hmat::Blk> blk(2 * nb);
    size_t store = 0;
    int64_t toff = 0, slot = 0;
    std::vector<double> kself(N, 0.0);
    for (int side = 0; side < 2; ++side) {
        const int64_t* rank = side == 0 ? rank_s : rank_n;
        const double* const* U = side == 0 ? U_s : U_n;
        const double* const* Vt = side == 0 ? Vt_s : Vt_n;
        const double* const* Dm = side == 0 ? D_s : D_n;
        for (int64_t b = 0; b < nb; ++b) {
            const int64_t s0 = range[4 * b], s1 = range[4 * b + 1], r0 = range[4 * b + 2], r1 = range[4 * b + 3];
            if (s0 < 0 || r0 < 0 || s1 < s0 || r1 < r0 || s1 >= N || r1 >= N)
                return fail(QDFN_ERR_INVALID, "block range out of [0, N)");
            hmat::Blk& B = blk[side * nb + b];
            B.s0 = s0; B.ns = s1 - s0 + 1; B.r0 = r0; B.nr = r1 - r0 + 1;
            if (B.nr > ((int64_t)1 << 20) * hmat::kTileRows) return fail(QDFN_ERR_INVALID, "block too tall");
            B.slot = slot;
            slot += B.nr;
            if (rank[b] < 0) {
                if (!Dm || !Dm[b]) return fail(QDFN_ERR_INVALID, "dense block without data");
                B.rank = -1;
                B.off_a = (int64_t)store;
                store += (size_t)B.ns * B.nr;
                B.off_b = 0; B.toff = 0;
            } else {
                if (rank[b] > hmat::kMaxRank) return fail(QDFN_ERR_INVALID, "low-rank block rank above 128");
                if (!U || !Vt || (rank[b] > 0 && (!U[b] || !Vt[b])))
                    return fail(QDFN_ERR_INVALID, "low-rank block without factors");
                if (s0 == r0 && s1 == r1 && side == 0)
                    return fail(QDFN_ERR_INVALID, "diagonal shear block must be dense (K_Self)");
                B.rank = (int32_t)rank[b];
                B.off_a = (int64_t)store;
                store += (size_t)B.rank * B.ns;
                B.off_b = (int64_t)store;
                store += (size_t)B.rank * B.nr;
                B.toff = toff;
                toff += B.rank;
            }
        }
    }
    // pack (converted to the storage type); the shear diagonal is zeroed and
    // K_Self = -K_ii taken from it (StiffnessTransitionToLoading)
    std::vector<unsigned char> hbuf(store * esz + 16);
    auto putv = [&](size_t o, double v) {
        if (esz == 8) put<double>(hbuf, o, v); else put<float>(hbuf, o, v);
    };
    for (int side = 0; side < 2; ++side) {
        const double* const* U = side == 0 ? U_s : U_n;
        const double* const* Vt = side == 0 ? Vt_s : Vt_n;
        const double* const* Dm = side == 0 ? D_s : D_n;
        for (int64_t b = 0; b < nb; ++b) {
            const hmat::Blk& B = blk[side * nb + b];
            if (B.rank < 0) {
                const bool diag = side == 0 && B.s0 == B.r0 && B.ns == B.nr;
                for (int64_t i = 0; i < B.nr; ++i)
                    for (int64_t j = 0; j < B.ns; ++j) {
                        double v = Dm[b][i * B.ns + j];
                        if (diag && i == j) { kself[B.r0 + i] = -v; v = 0.0; }
                        putv(B.off_a + j * B.nr + i, v);   // D^T
                    }
            } else {
                for (int64_t kk = 0; kk < B.rank; ++kk) {
                    for (int64_t j = 0; j < B.ns; ++j) putv(B.off_a + kk * B.ns + j, Vt[b][kk * B.ns + j]);
                    for (int64_t i = 0; i < B.nr; ++i) putv(B.off_b + kk * B.nr + i, U[b][i * B.rank + kk]);
                }
            }
        }
    }
    // receiver-row CSR of partial slots, block order, per side
    std::vector<int64_t> rowptr(2 * (N + 1), 0), rowslot((size_t)slot);
    for (int side = 0; side < 2; ++side) {
        int64_t* rp = rowptr.data() + side * (N + 1);
        for (int64_t b = 0; b < nb; ++b) {
            const hmat::Blk& B = blk[side * nb + b];
            for (int64_t i = 0; i < B.nr; ++i) rp[B.r0 + i + 1]++;
        }
        for (int64_t i = 0; i < N; ++i) rp[i + 1] += rp[i];
    }
    {
        const int64_t base_n = rowptr[N];  // shear slots first in rowslot
        std::vector<int64_t> fill(2 * N, 0);
        for (int side = 0; side < 2; ++side) {
            const int64_t* rp = rowptr.data() + side * (N + 1);
            for (int64_t b = 0; b < nb; ++b) {
                const hmat::Blk& B = blk[side * nb + b];
                for (int64_t i = 0; i < B.nr; ++i) {
                    const int64_t row = B.r0 + i;
                    rowslot[(side ? base_n : 0) + rp[row] + fill[side * N + row]++] = B.slot + i;
                }
            }
        }
        // normal rows index rowslot from base_n: shift the normal CSR
        for (int64_t i = 0; i <= N; ++i) rowptr[(N + 1) + i] += base_n;
    }
    std::vector<int64_t> lr, tiles;
    for (int64_t q = 0; q < 2 * nb; ++q) {
        if (blk[q].rank >= 0 && blk[q].rank > 0) lr.push_back(q);
        const int64_t nt = (blk[q].nr + hmat::kTileRows - 1) / hmat::kTileRows;
        for (int64_t t = 0; t < nt; ++t) tiles.push_back((q << 20) | t);
    }
    // device copies
    release_hmat(c);
    c->release(c->E); c->release(c->Kn);
    c->E = c->Kn = nullptr;
    int rc;
    hmat::Blk* dblk; unsigned char* dstore; int64_t *dlr, *dtiles, *drp, *drs; double *dt, *dpart;
    if ((rc = dcopy(c, blk.data(), blk.size(), &dblk)) || (rc = dcopy(c, hbuf.data(), hbuf.size(), &dstore)) ||
        (rc = dcopy(c, lr.data(), lr.size(), &dlr)) || (rc = dcopy(c, tiles.data(), tiles.size(), &dtiles)) ||
        (rc = dcopy(c, rowptr.data(), rowptr.size(), &drp)) ||
        (rc = dcopy(c, rowslot.data(), rowslot.size(), &drs)))
        return rc;
    if ((rc = c->dalloc(&dt, (size_t)std::max<int64_t>(toff, 1) * Rk))) return rc;
    c->hbufs.push_back(dt);
    if ((rc = c->dalloc(&dpart, (size_t)std::max<int64_t>(slot, 1) * Rk))) return rc;
    c->hbufs.push_back(dpart);
    hmat::Ops& h = c->hops;
    h.blk = dblk; h.nb = nb; h.store = dstore; h.lr_list = dlr; h.n_lr = (int64_t)lr.size();
    h.tile_list = dtiles; h.n_tiles = (int64_t)tiles.size(); h.t = dt; h.part = dpart;
    h.rowptr = drp; h.rowslot = drs;
    c->prec = precision;
    c->hmat = 1;
    c->ld = 0;
    if ((rc = h2d(c->kself, kself.data(), N * 8))) return rc;
    // Omega = sqrt(K_Self / Mass) (Main_H :72)
    std::vector<double> m((size_t)Rk * N), om(m.size());
    QDFN_CUDA(cudaMemcpy(m.data(), c->mass, m.size() * 8, cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < m.size(); ++q) {
        const double x = kself[q % N] / m[q];
        if (x < 0) return fail(QDFN_ERR_DOMAIN, "sqrt of a negative number in Omega (K_ii > 0)");
        om[q] = std::sqrt(x);
    }
    if ((rc = h2d(c->omega, om.data(), om.size() * 8))) return rc;
    return configure_launch(c);
}
