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
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "adjoint_kernels.h"
#include "ensemble_kernels.h"
#include "sim_kernel.cuh"


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
    double *la = nullptr, *lth0 = nullptr;   // ln(V_i/V0), ln(theta_i V0/Dc): F0's derivatives (adjoint)
    double* dref = nullptr;                   // [2][R] reference slip of the FP32/BF16 x copy
    double *rowsum_e = nullptr, *rowsum_n = nullptr;   // [N] row sums of the stored FP32/BF16 operator
    unsigned char* sw_used = nullptr;         // adjoint recording: solver of each patch in the next launch
    double *ra = nullptr, *rDc = nullptr;
    unsigned char* unstable;
    int* has_unstable;
    double *V, *D, *theta, *fric, *accel, *sig_old, *Vn, *Dn, *thn, *fn, *sn, *dtall, *tld, *knd;
    int *instab, *flag, *sw, *sw_n;
    double* accel_n;
    double *part_s = nullptr, *part_n = nullptr;
    size_t part_cap = 0, partn_cap = 0, red_cap = 0, xd_cap = 0;   // elements held by the work buffers
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
    int pair_solve = 2;              // overlapped-phase solves: 2 one lane per patch, 32-row chunks; 1 lane
                                     // pairs, 16-row chunks; 0 even lanes alone (QDFN_PAIR_SOLVE)
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
    qdfn_ensemble* ens = nullptr;    // the ensemble this context is a member of

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
    p.nblk = c->nblocks;
    p.sw_used = c->sw_used;
    p.dref = c->dref;
    const bool offs = !c->hmat && c->prec != QDFN_FP64 && c->rowsum_e;
    p.rowsum_e = offs ? c->rowsum_e : nullptr;
    p.rowsum_n = offs ? c->rowsum_n : nullptr;
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
    if (const char* e = std::getenv("QDFN_PAIR_SOLVE")) c->pair_solve = std::max(0, std::min(2, std::atoi(e)));
    int64_t want_blocks;
    if (c->hmat) {
        c->smem = (size_t)Rk * hmat::kChunk * xsz + (size_t)hmat::kMaxRank * Rk * sizeof(double);
        c->nchunk = c->nchunk2 = 0;
        c->chunk_len = c->chunk_len2 = c->rb_small0 = 0;
        want_blocks = (std::max<int64_t>(c->hops.n_tiles, c->hops.n_lr) + kSimThreads / 32 - 1) / (kSimThreads / 32);
    } else {
        // column chunks of at most 2048 sources staged in shared memory per instance,
        // enough (row block, chunk) tiles for >= 2 per SM
        const int64_t rows_per_blk = (int64_t)kOpThreads * vec;
        const int64_t nrb = (c->N + rows_per_blk - 1) / rows_per_blk;
        // tiles per SM and step before the guided tail (tuning knob QDFN_TILES_PER_SM)
        int64_t tiles_per_sm = 4;
        if (const char* e = std::getenv("QDFN_TILES_PER_SM")) tiles_per_sm = std::max(1, std::min(64, std::atoi(e)));
        if (const char* e = std::getenv("QDFN_SOLVE_HOLD")) c->hold_cap = std::max(1, std::min(64, std::atoi(e)));
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
    // work buffers kept when large enough (a re-division of an ensemble's SMs
    // re-sizes every member): every launch rewrites them before reading
    auto ensure = [&](auto** ptr, size_t n, size_t& cap) -> int {
        if (*ptr && cap >= n) return QDFN_OK;
        c->release(*ptr);
        *ptr = nullptr;
        cap = n;
        return c->dalloc(ptr, n);
    };
    int rc;
    if (!c->hmat) {
        // x copy of D: N columns padded to a multiple of 8 (+8), read in runs of 4
        // elements per x copy (two: current and next step), a multiple of 32 so
        // that the second copy starts 16-byte aligned like the first (bulk copies
        // need 16-byte aligned sources)
        c->xd_stride = (((int64_t)c->N + 16) * Rk + 31) / 32 * 32;
        if ((rc = ensure(reinterpret_cast<unsigned char**>(&c->xd), 2 * (size_t)c->xd_stride * xsz, c->xd_cap)))
            return rc;
        if ((reinterpret_cast<uintptr_t>(c->xd) | (uintptr_t)(c->xd_stride * xsz)) % 16 != 0)
            return fail(QDFN_ERR_INVALID, "x copy of D not 16-byte aligned");
        const size_t slots = (size_t)std::max(c->nchunk, c->nchunk2);
        c->part_stride = (int64_t)slots * Rk * c->N;   // two buffers: this step's and the next's
        if ((rc = ensure(&c->part_s, 2 * (size_t)c->part_stride, c->part_cap))) return rc;
        if ((rc = ensure(&c->part_n, 2 * (size_t)c->part_stride, c->partn_cap))) return rc;
    }
    if ((rc = ensure(&c->red, (size_t)2 * c->nblocks * Rk * kRedSlots, c->red_cap))) return rc;
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
    A(la, RN); A(lth0, RN); A(dref, 2 * (size_t)Rk);
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
    std::vector<double> hla(RN), hlth(RN);
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
            hla[q] = std::log(pr->V_i[s] / sim::kV0);
            hlth[q] = std::log(pr->theta_i[s] * sim::kV0 / pr->Dc[s]);
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
        (rc = h2d(c->status, z32.data(), Rk * 4)) || (rc = h2d(c->la, hla.data(), RN * 8)) ||
        (rc = h2d(c->lth0, hlth.data(), RN * 8))) {
        delete c;
        return rc;
    }
    *out = c;
    return QDFN_OK;
}

namespace {
void ensemble_detach(qdfn_ensemble* e, qdfn_ctx* c);
}

extern "C" int qdfn_ctx_destroy(qdfn_ctx* ctx) {
    if (!ctx) return QDFN_OK;
    if (ctx->running) cudaStreamSynchronize(ctx->pending);
    if (ctx->ens) ensemble_detach(ctx->ens, ctx);
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
    c->release(c->rowsum_e);
    c->release(c->rowsum_n);
    c->rowsum_e = c->rowsum_n = nullptr;
    if (precision != QDFN_FP64) {   // the x copy's offset needs the stored matrices' row sums
        if ((rc = c->dalloc(&c->rowsum_e, (size_t)N)) || (rc = c->dalloc(&c->rowsum_n, (size_t)N))) return rc;
        k_rowsum<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(N, c->ld, precision, c->E, c->Kn, c->rowsum_e,
                                                              c->rowsum_n);
        QDFN_CUDA(cudaGetLastError());
    }
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

namespace {
bool ensemble_running(const qdfn_ensemble* e);
void ensemble_member_ran(qdfn_ensemble* e);
}

extern "C" int qdfn_run_async(qdfn_ctx* c, int64_t nsteps, double timeout_s, void* stream) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (c->ens && ensemble_running(c->ens)) return fail(QDFN_ERR_STATE, "the context's ensemble has a run in flight");
    if (c->ens) ensemble_member_ran(c->ens);   // its busy time moves outside the ensemble's readback
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
// ===========================================================================
// Adjoint of the stepped system (no counterpart in the reference, which has
// no derivatives): the reverse-mode gradient of a loss on the trajectory with
// respect to the per-patch a, b and Dc.
//
// The forward window runs one step per launch and keeps the state every
// `cp` steps (checkpoints, cp ~ sqrt(nsteps) by default).  The reverse sweep
// takes the segments last to first: it restores the segment's checkpoint,
// replays its steps one per launch recording each step's state, TLD, sigma
// and solver (the tape), and walks the tape backwards.  Per step: the
// per-patch vector-Jacobian products of the converged solves (adjoint.cuh,
// FP64 dual numbers), the transposed stiffness products E^T and Kn^T over the
// stored operator (FP32 or FP64, as in the forward), and the time step's
// adjoint routed through the controller (Main_D :162-201): through the patch
// that set min |V/Accel| / DtCut, through 1.2 x the previous step's Dt, or
// nowhere (RuptureDt, MaximumDt); retried steps scale it by their halvings.
namespace {

struct DevMem {
    std::vector<void*> ptrs;
    template <class T>
    int get(T** p, size_t n) {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess)
            return fail(QDFN_ERR_NOMEM, "adjoint buffers");
        ptrs.push_back(q);
        *p = reinterpret_cast<T*>(q);
        return QDFN_OK;
    }
    ~DevMem() {
        for (void* q : ptrs) cudaFree(q);
    }
};

// one launch of `nsteps` steps on st, as qdfn_run_async (no status check)
int launch_steps(qdfn_ctx* c, int64_t nsteps, uint64_t budget_ns, cudaStream_t st) {
    QDFN_CUDA(cudaMemsetAsync(c->gerr, 0, 2 * sizeof(int), st));
    SimParams p = make_params(c, budget_ns);
    SimKernel k = sim_kernel(c->prec, c->R, c->hmat != 0);
    void* args[] = {&p, &nsteps};
    QDFN_CUDA(cudaLaunchCooperativeKernel((const void*)k, dim3(c->nblocks), dim3(kSimThreads), args, c->smem, st));
    return QDFN_OK;
}

int run_status(qdfn_ctx* c, cudaStream_t st) {
    QDFN_CUDA(cudaStreamSynchronize(st));
    int gerr = 0;
    QDFN_CUDA(cudaMemcpy(&gerr, c->gerr, sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<int> v(kernel_R(c->R));
    QDFN_CUDA(cudaMemcpy(v.data(), c->status, v.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (int r = 0; r < c->R; ++r)
        if (v[r] != 0) return fail(v[r], "instance " + std::to_string(r) + " stopped in the adjoint's forward");
    if (gerr != 0) return fail(gerr, "device loop stopped early in the adjoint's forward");
    return QDFN_OK;
}

// the six host-visible state fields (one block), T/dt and step of a context
struct Snap {
    double* s6;
    double* Tdt;
    int64_t* step;
};
int snap_save(qdfn_ctx* c, const Snap& d, cudaStream_t st) {
    const size_t RN = (size_t)kernel_R(c->R) * c->N, Rk = kernel_R(c->R);
    QDFN_CUDA(cudaMemcpyAsync(d.s6, c->V, 6 * RN * 8, cudaMemcpyDeviceToDevice, st));
    QDFN_CUDA(cudaMemcpyAsync(d.Tdt, c->T, 2 * Rk * 8, cudaMemcpyDeviceToDevice, st));
    QDFN_CUDA(cudaMemcpyAsync(d.step, c->step, Rk * 8, cudaMemcpyDeviceToDevice, st));
    return QDFN_OK;
}
int snap_load(qdfn_ctx* c, const Snap& d, cudaStream_t st) {
    const size_t RN = (size_t)kernel_R(c->R) * c->N, Rk = kernel_R(c->R);
    QDFN_CUDA(cudaMemcpyAsync(c->V, d.s6, 6 * RN * 8, cudaMemcpyDeviceToDevice, st));
    QDFN_CUDA(cudaMemcpyAsync(c->T, d.Tdt, 2 * Rk * 8, cudaMemcpyDeviceToDevice, st));
    QDFN_CUDA(cudaMemcpyAsync(c->step, d.step, Rk * 8, cudaMemcpyDeviceToDevice, st));
    return QDFN_OK;
}

}  // namespace

extern "C" int qdfn_adjoint_run(qdfn_ctx* c, int64_t nsteps, int64_t checkpoint_every, const double* dL_dD_final,
                                int64_t n_seeds, const int64_t* seed_step, const int32_t* seed_inst,
                                const int64_t* seed_patch, const double* seed_dV, const double* seed_dD,
                                const double* seed_dT, double* dL_da, double* dL_db, double* dL_dDc,
                                double timeout_s) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (c->prec < 0 || c->hmat) return fail(QDFN_ERR_STATE, "the adjoint needs a dense operator (qdfn_set_dense)");
    if (c->running || (c->ens && ensemble_running(c->ens))) return fail(QDFN_ERR_STATE, "a run is in flight");
    if (c->prob.alpha_evo != 0.0) return fail(QDFN_ERR_INVALID, "the adjoint supports Alpha_Evo = 0 only");
    if (nsteps < 1) return fail(QDFN_ERR_INVALID, "nsteps must be >= 1");
    if (n_seeds < 0 || (n_seeds > 0 && (!seed_step || !seed_inst || !seed_patch || !seed_dV || !seed_dD || !seed_dT)))
        return fail(QDFN_ERR_INVALID, "seed arrays");
    if (!dL_da || !dL_db || !dL_dDc) return fail(QDFN_ERR_INVALID, "null gradient output");
    const int64_t N = c->N, Ns = c->N - c->Nload;
    const int R = c->R, Rk = kernel_R(c->R);
    const int64_t RN = (int64_t)Rk * N;
    for (int64_t k = 0; k < n_seeds; ++k)
        if (seed_step[k] < 0 || seed_step[k] > nsteps || seed_inst[k] < 0 || seed_inst[k] >= R ||
            seed_patch[k] < -1 || seed_patch[k] >= N)
            return fail(QDFN_ERR_INVALID, "seed " + std::to_string(k) + " out of range");
    int64_t cp = checkpoint_every > 0 ? checkpoint_every : (int64_t)std::ceil(std::sqrt((double)nsteps));
    cp = std::max<int64_t>(1, std::min(cp, nsteps));
    const int64_t nseg = (nsteps + cp - 1) / cp;
    const uint64_t budget_ns = (uint64_t)((timeout_s > 0 ? timeout_s : 1e6) * 1e9);
    cudaStream_t st = nullptr;
    int rc;
    DevMem m;
    // checkpoints (nseg, the state before each segment) and the final state
    std::vector<Snap> ck(nseg + 1);
    for (auto& k : ck)
        if ((rc = m.get(&k.s6, 6 * RN)) || (rc = m.get(&k.Tdt, 2 * Rk)) || (rc = m.get(&k.step, Rk))) return rc;
    // tape of one segment: state s = 0..cp (V, D, theta, accel), steps 1..cp (tld, sigma, solver), T and dt
    double *tV, *tD, *tth, *tA, *ttld, *tsig, *tT, *tdt;
    unsigned char* tsw;
    if ((rc = m.get(&tV, (cp + 1) * RN)) || (rc = m.get(&tD, (cp + 1) * RN)) || (rc = m.get(&tth, (cp + 1) * RN)) ||
        (rc = m.get(&tA, (cp + 1) * RN)) || (rc = m.get(&ttld, cp * RN)) || (rc = m.get(&tsig, cp * RN)) ||
        (rc = m.get(&tsw, cp * RN)) || (rc = m.get(&tT, (cp + 1) * Rk)) || (rc = m.get(&tdt, (cp + 1) * Rk)))
        return rc;
    // adjoint state and work arrays
    double *lV, *lD, *lth, *lA, *oDloc, *oVold, *oThold, *oTLD, *oSig, *ga, *gb, *gDc, *bdt, *btx, *sums, *part,
        *ctl, *addv;
    int64_t* addi;
    int* derr;
    const int nblk = adj_local_blocks(RN);
    const int64_t rpb = c->ld, nrb = (N + rpb - 1) / rpb;
    const int64_t max_add = std::max<int64_t>(n_seeds + Rk, 1);
    if ((rc = m.get(&lV, RN)) || (rc = m.get(&lD, RN)) || (rc = m.get(&lth, RN)) || (rc = m.get(&lA, RN)) ||
        (rc = m.get(&oDloc, RN)) || (rc = m.get(&oVold, RN)) || (rc = m.get(&oThold, RN)) ||
        (rc = m.get(&oTLD, RN)) || (rc = m.get(&oSig, RN)) || (rc = m.get(&ga, RN)) || (rc = m.get(&gb, RN)) ||
        (rc = m.get(&gDc, RN)) || (rc = m.get(&bdt, (int64_t)nblk * Rk)) || (rc = m.get(&btx, (int64_t)nblk * Rk)) ||
        (rc = m.get(&sums, 2 * Rk)) || (rc = m.get(&part, nrb * 2 * RN)) || (rc = m.get(&ctl, 5 * Rk)) ||
        (rc = m.get(&addv, 3 * max_add)) || (rc = m.get(&addi, max_add)) || (rc = m.get(&derr, 1)))
        return rc;
    if ((rc = adj_transpose_prepare(c->prec, Rk, rpb))) return rc;
    for (double* z : {lV, lD, lth, lA, ga, gb, gDc}) QDFN_CUDA(cudaMemsetAsync(z, 0, RN * 8, st));
    QDFN_CUDA(cudaMemsetAsync(derr, 0, sizeof(int), st));

    // ---- forward: one step per launch, a checkpoint every cp steps
    for (int64_t seg = 0; seg < nseg; ++seg) {
        if ((rc = snap_save(c, ck[seg], st))) return rc;
        const int64_t len = std::min(cp, nsteps - seg * cp);
        for (int64_t t = 0; t < len; ++t)
            if ((rc = launch_steps(c, 1, budget_ns, st))) return rc;
        if ((rc = run_status(c, st))) return rc;
    }
    if ((rc = snap_save(c, ck[nseg], st))) return rc;

    // ---- seeds by step
    std::vector<std::vector<int64_t>> by_step(nsteps + 1);
    for (int64_t k = 0; k < n_seeds; ++k) by_step[seed_step[k]].push_back(k);
    std::vector<double> lamT(Rk, 0.0), carry(Rk, 0.0);
    if (dL_dD_final) {
        std::vector<double> h(RN, 0.0);
        std::memcpy(h.data(), dL_dD_final, (size_t)R * N * 8);
        QDFN_CUDA(cudaMemcpy(lD, h.data(), RN * 8, cudaMemcpyHostToDevice));
    }
    // adds seeds of state n and controller terms to (lV, lD, lA), lamT
    std::vector<int64_t> hi;
    std::vector<double> hv;
    auto apply_adds = [&](const std::vector<int64_t>& idx, const std::vector<double>& vV,
                          const std::vector<double>& vD, const std::vector<double>& vA) -> int {
        const int n = (int)idx.size();
        if (n == 0) return QDFN_OK;
        std::vector<double> v(3 * (size_t)n);
        for (int k = 0; k < n; ++k) { v[k] = vV[k]; v[n + k] = vD[k]; v[2 * n + k] = vA[k]; }
        QDFN_CUDA(cudaMemcpy(addi, idx.data(), n * 8, cudaMemcpyHostToDevice));
        QDFN_CUDA(cudaMemcpy(addv, v.data(), 3 * (size_t)n * 8, cudaMemcpyHostToDevice));
        return adj_add(n, addi, addv, lV, lD, lA, st);
    };
    auto seeds_of = [&](int64_t n) -> int {
        std::vector<int64_t> idx;
        std::vector<double> vV, vD, vA;
        for (int64_t k : by_step[n]) {
            lamT[seed_inst[k]] += seed_dT[k];
            if (seed_patch[k] >= 0) {
                idx.push_back((int64_t)seed_inst[k] * N + seed_patch[k]);
                vV.push_back(seed_dV[k]); vD.push_back(seed_dD[k]); vA.push_back(0.0);
            }
        }
        return apply_adds(idx, vV, vD, vA);
    };
    if ((rc = seeds_of(nsteps))) return rc;

    const double rupture = c->prob.rupture_dt, maxdt = c->prob.max_dt, swv = c->prob.switch_v, dtcut = c->prob.dt_cut;
    const bool told = c->prob.interp_at_told != 0;
    // ---- reverse, segment by segment
    for (int64_t seg = nseg - 1; seg >= 0; --seg) {
        const int64_t s0 = seg * cp, len = std::min(cp, nsteps - s0);
        if ((rc = snap_load(c, ck[seg], st))) return rc;
        auto rec_state = [&](int64_t t) -> int {   // tape state t from the context's host-visible state
            QDFN_CUDA(cudaMemcpyAsync(tV + t * RN, c->V, RN * 8, cudaMemcpyDeviceToDevice, st));
            QDFN_CUDA(cudaMemcpyAsync(tD + t * RN, c->D, RN * 8, cudaMemcpyDeviceToDevice, st));
            QDFN_CUDA(cudaMemcpyAsync(tth + t * RN, c->theta, RN * 8, cudaMemcpyDeviceToDevice, st));
            QDFN_CUDA(cudaMemcpyAsync(tA + t * RN, c->accel, RN * 8, cudaMemcpyDeviceToDevice, st));
            QDFN_CUDA(cudaMemcpyAsync(tT + t * Rk, c->T, Rk * 8, cudaMemcpyDeviceToDevice, st));
            QDFN_CUDA(cudaMemcpyAsync(tdt + t * Rk, c->dt, Rk * 8, cudaMemcpyDeviceToDevice, st));
            return QDFN_OK;
        };
        if ((rc = rec_state(0))) return rc;
        for (int64_t t = 1; t <= len; ++t) {
            c->sw_used = tsw + (t - 1) * RN;
            rc = launch_steps(c, 1, budget_ns, st);
            c->sw_used = nullptr;
            if (rc) return rc;
            if ((rc = rec_state(t))) return rc;
            QDFN_CUDA(cudaMemcpyAsync(ttld + (t - 1) * RN, c->tld, RN * 8, cudaMemcpyDeviceToDevice, st));
            QDFN_CUDA(cudaMemcpyAsync(tsig + (t - 1) * RN, c->sig_old, RN * 8, cudaMemcpyDeviceToDevice, st));
        }
        if ((rc = run_status(c, st))) return rc;
        std::vector<double> hdt((len + 1) * Rk), hT((len + 1) * Rk);
        QDFN_CUDA(cudaMemcpy(hdt.data(), tdt, hdt.size() * 8, cudaMemcpyDeviceToHost));
        QDFN_CUDA(cudaMemcpy(hT.data(), tT, hT.size() * 8, cudaMemcpyDeviceToHost));
        for (int64_t t = len; t >= 1; --t) {
            const int64_t n = s0 + t;   // the step taking tape state t-1 to t
            AdjLocalArgs a{};
            a.N = N; a.Ns = Ns; a.R = Rk; a.dr = c->prob.evolution_dr; a.interp_at_told = told ? 1 : 0;
            a.eta = c->eta; a.sigma_min = c->prob.sigma_min;
            a.Vprev = tV + (t - 1) * RN; a.Dprev = tD + (t - 1) * RN; a.thprev = tth + (t - 1) * RN;
            a.Vcur = tV + t * RN; a.tld = ttld + (t - 1) * RN; a.sig = tsig + (t - 1) * RN;
            a.sw = tsw + (t - 1) * RN;
            a.dt = tdt + t * Rk; a.Tprev = tT + (t - 1) * Rk;
            a.pa = c->a; a.pb = c->b; a.pDc = c->Dc; a.F0 = c->F0; a.la = c->la; a.lth0 = c->lth0;
            a.kself = c->kself; a.mass = c->mass; a.omega = c->omega; a.tau0 = c->tau0;
            a.n_ext = c->n_ext; a.ext_t = c->ext_t; a.ext_n = c->ext_n; a.ext_s = c->ext_s; a.ext_p = c->ext_p;
            a.lV = lV; a.lD = lD; a.lth = lth; a.lA = lA;
            a.oDloc = oDloc; a.oVold = oVold; a.oThold = oThold; a.oTLD = oTLD; a.oSig = oSig;
            a.ga = ga; a.gb = gb; a.gDc = gDc; a.blk_dt = bdt; a.blk_tx = btx; a.sums = sums; a.err = derr;
            if ((rc = adj_local(a, st))) return rc;
            AdjTransArgs tr{};
            tr.N = N; tr.rpb = rpb; tr.nrb = nrb; tr.gx = std::max<int64_t>(1, (4 * num_sms() + nrb - 1) / nrb);
            tr.E = c->E; tr.Kn = c->Kn; tr.x_s = oTLD; tr.x_n = oSig; tr.part = part;
            if ((rc = adj_transpose(c->prec, Rk, tr, oDloc, lD, st))) return rc;   // lambda_D of state t-1
            std::swap(lV, oVold);
            std::swap(lth, oThold);
            QDFN_CUDA(cudaMemsetAsync(lA, 0, RN * 8, st));
            if ((rc = adj_dtctl(Rk, N, Ns, tV + (t - 1) * RN, tA + (t - 1) * RN, c->unstable, c->has_unstable, ctl,
                                st)))
                return rc;
            std::vector<double> hs(2 * Rk), hc(5 * Rk);
            QDFN_CUDA(cudaMemcpyAsync(hs.data(), sums, hs.size() * 8, cudaMemcpyDeviceToHost, st));
            QDFN_CUDA(cudaMemcpyAsync(hc.data(), ctl, hc.size() * 8, cudaMemcpyDeviceToHost, st));
            QDFN_CUDA(cudaStreamSynchronize(st));
            // the step's dt: its patches, T_n = T_{n-1} + dt, the external-stress
            // time (TOld + Dt in main, TOld in main_H), the next step's 1.2 Dt
            std::vector<int64_t> idx;
            std::vector<double> vV, vD, vA;
            for (int r = 0; r < Rk; ++r) {
                const double ldt = hs[r] + lamT[r] + (told ? 0.0 : hs[Rk + r]) + carry[r];
                lamT[r] += hs[Rk + r];
                carry[r] = 0.0;
                // the controller that chose this step's Dt, from state t-1
                const double dtn = hdt[t * Rk + r], dtp = hdt[(t - 1) * Rk + r];
                double vmax = hc[r * 5 + 0];
                if (hc[r * 5 + 1] != 0) vmax = NAN;
                const double dtmin = hc[r * 5 + 2] / dtcut;
                const bool usable = hc[r * 5 + 3] != 0;
                int src = 0;   // 0 constant, 1 min |V/A| / DtCut, 2 1.2 x previous Dt
                double ref;
                if (vmax > swv) ref = rupture;
                else if (dtmin > maxdt) ref = maxdt;
                else { ref = dtmin; src = usable ? 1 : 0; }
                double dtc;
                if (ref <= rupture) dtc = ref;
                else if (dtp < ref / 1.2) { dtc = dtp * 1.2; src = 2; }
                else dtc = ref;
                const double sc = dtn / dtc;
                const double e2 = std::log2(sc);
                if (!(sc > 0 && sc <= 1 && std::fabs(e2 - std::round(e2)) < 1e-9)) src = 0;   // e.g. Dt = 1e-3
                if (src == 1) {
                    const int64_t k = (int64_t)hc[r * 5 + 4];
                    double Vk = 0, Ak = 0;
                    QDFN_CUDA(cudaMemcpy(&Vk, tV + (t - 1) * RN + (int64_t)r * N + k, 8, cudaMemcpyDeviceToHost));
                    QDFN_CUDA(cudaMemcpy(&Ak, tA + (t - 1) * RN + (int64_t)r * N + k, 8, cudaMemcpyDeviceToHost));
                    const double q = Vk / Ak, sg = q < 0 ? -1.0 : 1.0;
                    idx.push_back((int64_t)r * N + k);
                    vV.push_back(ldt * sc * sg / (Ak * dtcut));
                    vD.push_back(0.0);
                    vA.push_back(-ldt * sc * sg * Vk / (Ak * Ak * dtcut));
                } else if (src == 2) {
                    carry[r] = 1.2 * sc * ldt;
                }
            }
            if ((rc = apply_adds(idx, vV, vD, vA))) return rc;
            if ((rc = seeds_of(n - 1))) return rc;
        }
    }
    int herr = 0;
    QDFN_CUDA(cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) return fail(QDFN_ERR_DOMAIN, "a converged solve has a vanishing residual derivative");
    QDFN_CUDA(cudaMemcpy(dL_da, ga, (size_t)R * N * 8, cudaMemcpyDeviceToHost));
    QDFN_CUDA(cudaMemcpy(dL_db, gb, (size_t)R * N * 8, cudaMemcpyDeviceToHost));
    QDFN_CUDA(cudaMemcpy(dL_dDc, gDc, (size_t)R * N * 8, cudaMemcpyDeviceToHost));
    // the context ends where the forward window ended
    if ((rc = snap_load(c, ck[nseg], st))) return rc;
    QDFN_CUDA(cudaStreamSynchronize(st));
    return QDFN_OK;
}


extern "C" int qdfn_set_blocks(qdfn_ctx* c, int nblocks) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (nblocks < 0) return fail(QDFN_ERR_INVALID, "nblocks < 0");
    if (c->running) return fail(QDFN_ERR_STATE, "a run is in flight");
    if (c->ens) return fail(QDFN_ERR_STATE, "the context is an ensemble member (qdfn_ensemble_set_blocks)");
    c->nblocks_override = nblocks;
    return c->prec < 0 ? QDFN_OK : configure_launch(c);
}

extern "C" int qdfn_get_blocks(const qdfn_ctx* c) { return c ? c->nblocks : -1; }

extern "C" int qdfn_set_early_cols(qdfn_ctx* c, int cols) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (cols < 0 || cols > 64) return fail(QDFN_ERR_INVALID, "early columns must be in 0..64");
    if (c->running) return fail(QDFN_ERR_STATE, "a run is in flight");
    c->c_spec = cols;
    return QDFN_OK;
}

extern "C" int qdfn_get_early_cols(const qdfn_ctx* c) { return c ? c->c_spec : -1; }

// ===========================================================================
// Ensembles: several contexts advanced by one cooperative launch
//
// Each member keeps its own operator, state, counters and barrier words and
// runs on its own contiguous range of blocks (its share of the SMs), taking
// its own adaptive steps; the members never wait on one another.  One grid
// holds every member, so the co-residency that each member's grid barrier
// needs is the cooperative launch's own guarantee.

struct qdfn_ensemble {
    std::vector<qdfn_ctx*> m;
    std::vector<int> share;              // blocks asked for per member
    std::vector<uint64_t> mark;          // members' busy ns at the last balance
    int prec = -1, Rk = 0;
    int total = 0;                       // blocks of the launch
    size_t smem = 0;
    SimParams* hparams = nullptr;        // pinned [n]
    SimParams* dparams = nullptr;        // device [n]
    int2* dmap = nullptr;                // device [map_cap]: (member, block within it)
    size_t map_cap = 0;
    std::vector<int> configured;         // share each member was last configured for (0: never)
    int* dstat = nullptr;                // device [n] outcome of the last run
    int* hstat = nullptr;                // pinned [n]
    unsigned long long* dbusy = nullptr; // device [n] members' busy ns after the last run
    unsigned long long* hbusy = nullptr; // pinned [n]
    bool busy_valid = false;             // hbusy is current (the last run's, read back)
    unsigned* dfill = nullptr;           // device: members that have taken their steps (fill mode)
    int fill = 0;                        // fill mode on
    XferMember* dxfer = nullptr;         // device [n]: the members' slices of a state transfer
    double* dstage = nullptr;            // device: staging buffer of qdfn_ensemble_{set,get}_state_all
    int64_t stage_words = 0;
    cudaStream_t pending = nullptr;
    bool running = false;
    ~qdfn_ensemble() {
        if (dxfer) cudaFree(dxfer);
        if (dstage) cudaFree(dstage);
        if (hparams) cudaFreeHost(hparams);
        if (hstat) cudaFreeHost(hstat);
        if (hbusy) cudaFreeHost(hbusy);
        if (dbusy) cudaFree(dbusy);
        if (dfill) cudaFree(dfill);
        if (dparams) cudaFree(dparams);
        if (dmap) cudaFree(dmap);
        if (dstat) cudaFree(dstat);
    }
};

namespace {

bool ensemble_running(const qdfn_ensemble* e) { return e->running; }
void ensemble_member_ran(qdfn_ensemble* e) { e->busy_valid = false; }

void ensemble_detach(qdfn_ensemble* e, qdfn_ctx* c) {
    for (auto& x : e->m)
        if (x == c) x = nullptr;
}

// Estimated SM-nanoseconds of one step of a member on one SM: its operator
// bytes at one SM's share of the HBM stream (~44 B/ns) plus its patch solves
// (~450 ns of one SM each, FP64-pipe bound).  Only the starting point of the
// split; qdfn_ensemble_balance re-divides by measured time.
double member_cost(const qdfn_ctx* c) {
    const double esz = c->prec == QDFN_FP64 ? 8.0 : 4.0;
    const double n = (double)c->N;
    return 2.0 * n * n * esz / 44.0 + 450.0 * kernel_R(c->R) * n;
}

// A member's busy ns as the status kernel of the last ensemble run read them.
uint64_t busy_of(const qdfn_ensemble* e, int k) { return (uint64_t)e->hbusy[k]; }

// Member busy time of its runs so far (block 0's phase counters), ns.
uint64_t member_busy_ns(const qdfn_ctx* c) {
    unsigned long long v[4];
    if (cudaMemcpy(v, c->prof, sizeof(v), cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
    return v[0] + v[1] + v[2] + v[3];
}

int ensemble_max_blocks(const qdfn_ensemble* e, size_t smem, int* out) {
    const MembersKernel k = members_kernel(e->prec, e->Rk);
    QDFN_CUDA(cudaFuncSetAttribute((const void*)k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    QDFN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void*)k, kSimThreads, smem));
    if (occ < 1) return fail(QDFN_ERR_CUDA, "ensemble kernel cannot be resident");
    *out = occ * num_sms();
    return QDFN_OK;
}

// Re-sizes every member for its share and rebuilds the block map.
int ensemble_configure(qdfn_ensemble* e) {
    const int n = (int)e->m.size();
    size_t smem = 0;
    int total = 0;
    e->configured.resize(n, 0);
    for (int k = 0; k < n; ++k) {
        qdfn_ctx* c = e->m[k];
        if (e->configured[k] != e->share[k] || c->nblocks_override != e->share[k]) {
            c->nblocks_override = e->share[k];
            int rc = configure_launch(c);
            if (rc) return rc;
            e->configured[k] = e->share[k];
        }
        smem = std::max(smem, c->smem);
        total += c->nblocks;
    }
    int cap = 0;
    int rc = ensemble_max_blocks(e, smem, &cap);
    if (rc) return rc;
    if (total > cap)
        return fail(QDFN_ERR_INVALID, "the members need " + std::to_string(total) + " blocks; " +
                                          std::to_string(cap) + " fit on the GPU at once");
    std::vector<int2> map;
    map.reserve(total);
    for (int k = 0; k < n; ++k)
        for (int b = 0; b < e->m[k]->nblocks; ++b) map.push_back(make_int2(k, b));
    if (map.size() > e->map_cap) {   // kept across re-divisions: sized for the largest grid
        if (e->dmap) cudaFree(e->dmap);
        e->dmap = nullptr;
        e->map_cap = std::max(map.size(), (size_t)cap);
        QDFN_CUDA(cudaMalloc(&e->dmap, sizeof(int2) * e->map_cap));
    }
    QDFN_CUDA(cudaMemcpy(e->dmap, map.data(), sizeof(int2) * map.size(), cudaMemcpyHostToDevice));
    e->total = total;
    e->smem = smem;
    return QDFN_OK;
}

int ensemble_check(const qdfn_ensemble* e) {
    if (!e) return fail(QDFN_ERR_INVALID, "null ensemble");
    for (size_t k = 0; k < e->m.size(); ++k) {
        const qdfn_ctx* c = e->m[k];
        if (!c) return fail(QDFN_ERR_STATE, "member " + std::to_string(k) + " was destroyed");
        if (c->prec != e->prec || c->hmat || kernel_R(c->R) != e->Rk)
            return fail(QDFN_ERR_STATE, "member " + std::to_string(k) + " changed its operator");
        if (c->running) return fail(QDFN_ERR_STATE, "member " + std::to_string(k) + " has a run in flight");
    }
    return QDFN_OK;
}

}  // namespace

extern "C" int qdfn_ensemble_shares(int n, const double* cost, int nsm, int* out) {
    if (n < 1 || !cost || !out) return fail(QDFN_ERR_INVALID, "null or empty argument");
    if (n > nsm) return fail(QDFN_ERR_INVALID, std::to_string(n) + " members need at least as many SMs");
    double cmax = 0;
    for (int k = 0; k < n; ++k) {
        if (!(cost[k] > 0) || !std::isfinite(cost[k])) return fail(QDFN_ERR_INVALID, "costs must be positive");
        cmax = std::max(cmax, cost[k]);
    }
    // Member k on b blocks takes cost[k] / b.  The smallest makespan T whose
    // shares ceil(cost[k] / T) fit in nsm blocks (bisection on T), then the
    // blocks left over one by one to the member with the longest time.
    auto need = [&](double T) {
        long long s = 0;
        for (int k = 0; k < n; ++k) s += (long long)std::max(1.0, std::ceil(cost[k] / T * (1 - 1e-12)));
        return s;
    };
    double lo = cmax / nsm, hi = cmax;   // need(hi) = n <= nsm
    for (int it = 0; it < 200 && hi - lo > 1e-12 * hi; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (need(mid) <= nsm) hi = mid; else lo = mid;
    }
    int used = 0;
    for (int k = 0; k < n; ++k) {
        out[k] = (int)std::max(1.0, std::ceil(cost[k] / hi * (1 - 1e-12)));
        used += out[k];
    }
    while (used < nsm) {
        int worst = 0;
        for (int k = 1; k < n; ++k)
            if (cost[k] / out[k] > cost[worst] / out[worst]) worst = k;
        ++out[worst];
        ++used;
    }
    return QDFN_OK;
}

extern "C" int qdfn_ensemble_create(qdfn_ensemble** out, int n, qdfn_ctx* const* members, const int* blocks) {
    if (!out || !members || n < 1) return fail(QDFN_ERR_INVALID, "null or empty argument");
    *out = nullptr;
    for (int k = 0; k < n; ++k) {
        const qdfn_ctx* c = members[k];
        if (!c) return fail(QDFN_ERR_INVALID, "null member");
        if (c->prec < 0 || c->hmat) return fail(QDFN_ERR_STATE, "members need a dense operator (qdfn_set_dense)");
        if (c->prec != members[0]->prec || kernel_R(c->R) != kernel_R(members[0]->R))
            return fail(QDFN_ERR_INVALID, "members differ in operator precision or instance count");
        if (c->ens) return fail(QDFN_ERR_STATE, "a member already belongs to an ensemble");
        if (c->running) return fail(QDFN_ERR_STATE, "a member has a run in flight");
        for (int j = 0; j < k; ++j)
            if (members[j] == c) return fail(QDFN_ERR_INVALID, "a context is listed twice");
        if (blocks && blocks[k] < 1) return fail(QDFN_ERR_INVALID, "blocks must be >= 1");
    }
    auto* e = new qdfn_ensemble();
    e->m.assign(members, members + n);
    e->prec = members[0]->prec;
    e->Rk = kernel_R(members[0]->R);
    e->share.assign(n, 1);
    e->mark.assign(n, 0);
    int rc = QDFN_OK;
    if (blocks) {
        e->share.assign(blocks, blocks + n);
    } else {
        std::vector<double> cost(n);
        for (int k = 0; k < n; ++k) cost[k] = member_cost(members[k]);
        rc = qdfn_ensemble_shares(n, cost.data(), num_sms(), e->share.data());
    }
    if (!rc && (cudaMallocHost(&e->hparams, sizeof(SimParams) * n) != cudaSuccess ||
                cudaMallocHost(&e->hstat, sizeof(int) * n) != cudaSuccess ||
                cudaMallocHost(&e->hbusy, sizeof(unsigned long long) * n) != cudaSuccess ||
                cudaMalloc(&e->dbusy, sizeof(unsigned long long) * n) != cudaSuccess ||
                cudaMalloc(&e->dparams, sizeof(SimParams) * n) != cudaSuccess ||
                cudaMalloc(&e->dstat, sizeof(int) * n) != cudaSuccess ||
                cudaMalloc(&e->dfill, sizeof(unsigned)) != cudaSuccess))
        rc = fail(QDFN_ERR_NOMEM, "ensemble buffers");
    if (!rc) rc = ensemble_configure(e);
    if (!rc) {   // the state-transfer map: member after member, [6][R][N] then T, dt, step [R]
        std::vector<XferMember> xm(n);
        int64_t off = 0;
        for (int k = 0; k < n; ++k) {
            qdfn_ctx* c = members[k];
            xm[k] = XferMember{c->V, c->T, c->dt, c->step, off, c->N, c->R, kernel_R(c->R)};
            off += 6 * (int64_t)c->R * c->N + 3 * (int64_t)c->R;
        }
        e->stage_words = off;
        if (cudaMalloc(&e->dxfer, sizeof(XferMember) * n) != cudaSuccess ||
            cudaMalloc(&e->dstage, sizeof(double) * (size_t)off) != cudaSuccess)
            rc = fail(QDFN_ERR_NOMEM, "ensemble state buffers");
        else if (cudaMemcpy(e->dxfer, xm.data(), sizeof(XferMember) * n, cudaMemcpyHostToDevice) != cudaSuccess)
            rc = fail(QDFN_ERR_CUDA, "ensemble state map");
    }
    if (rc) {
        for (qdfn_ctx* c : e->m) c->nblocks_override = 0;
        delete e;
        return rc;
    }
    for (int k = 0; k < n; ++k) {
        e->m[k]->ens = e;
        e->mark[k] = member_busy_ns(e->m[k]);
    }
    *out = e;
    return QDFN_OK;
}

extern "C" int qdfn_ensemble_destroy(qdfn_ensemble* e) {
    if (!e) return QDFN_OK;
    if (e->running) cudaStreamSynchronize(e->pending);
    for (qdfn_ctx* c : e->m)
        if (c) {
            c->ens = nullptr;
            c->running = false;
        }
    delete e;
    return QDFN_OK;
}

extern "C" int qdfn_ensemble_get_blocks(const qdfn_ensemble* e, int* blocks) {
    if (!e || !blocks) return fail(QDFN_ERR_INVALID, "null argument");
    for (size_t k = 0; k < e->m.size(); ++k) blocks[k] = e->m[k] ? e->m[k]->nblocks : 0;
    return QDFN_OK;
}

extern "C" int qdfn_ensemble_set_blocks(qdfn_ensemble* e, const int* blocks) {
    int rc = ensemble_check(e);
    if (rc) return rc;
    if (e->running) return fail(QDFN_ERR_STATE, "a run is in flight");
    const int n = (int)e->m.size();
    std::vector<int> s(n);
    if (blocks) {
        for (int k = 0; k < n; ++k) {
            if (blocks[k] < 1) return fail(QDFN_ERR_INVALID, "blocks must be >= 1");
            s[k] = blocks[k];
        }
    } else {
        std::vector<double> cost(n);
        for (int k = 0; k < n; ++k) cost[k] = member_cost(e->m[k]);
        if ((rc = qdfn_ensemble_shares(n, cost.data(), num_sms(), s.data()))) return rc;
    }
    std::vector<int> old = e->share;
    e->share = s;
    if ((rc = ensemble_configure(e))) {
        e->share = old;
        ensemble_configure(e);
        return rc;
    }
    return QDFN_OK;
}

extern "C" int qdfn_ensemble_balance(qdfn_ensemble* e) {
    int rc = ensemble_check(e);
    if (rc) return rc;
    if (e->running) return fail(QDFN_ERR_STATE, "a run is in flight");
    const int n = (int)e->m.size();
    // measured cost of each member since the last balance: its busy time times
    // the blocks it ran on (block-ns); members without a run keep their share
    std::vector<double> cost(n);
    std::vector<uint64_t> now(n);
    bool any = false;
    for (int k = 0; k < n; ++k) {
        now[k] = e->busy_valid ? busy_of(e, k) : member_busy_ns(e->m[k]);
        const double t = (double)(now[k] - e->mark[k]);
        cost[k] = t * e->m[k]->nblocks;
        any = any || t > 0;
    }
    if (!any) return QDFN_OK;
    double mean = 0;
    int cnt = 0;
    for (int k = 0; k < n; ++k)
        if (cost[k] > 0) { mean += cost[k]; ++cnt; }
    mean /= cnt;
    for (int k = 0; k < n; ++k)
        if (!(cost[k] > 0)) cost[k] = mean;
    std::vector<int> s(n);
    int cap = 0;
    if ((rc = ensemble_max_blocks(e, e->smem, &cap))) return rc;
    if ((rc = qdfn_ensemble_shares(n, cost.data(), std::min(cap, num_sms()), s.data()))) return rc;
    std::vector<int> old = e->share;
    e->share = s;
    if ((rc = ensemble_configure(e))) {
        e->share = old;
        ensemble_configure(e);
        return rc;
    }
    e->mark = now;
    return QDFN_OK;
}

extern "C" int qdfn_ensemble_run_async(qdfn_ensemble* e, int64_t nsteps, double timeout_s, void* stream) {
    int rc = ensemble_check(e);
    if (rc) return rc;
    if (e->running) return fail(QDFN_ERR_STATE, "a run is in flight (qdfn_ensemble_sync first)");
    if (nsteps < 0) return fail(QDFN_ERR_INVALID, "nsteps < 0");
    if (nsteps == 0) return QDFN_OK;
    for (size_t k = 0; k < e->m.size(); ++k)   // a member re-sized since (qdfn_set_dense) is re-mapped
        if (e->m[k]->nblocks_override != e->share[k]) {
            if ((rc = ensemble_configure(e))) return rc;
            break;
        }
    const double budget = timeout_s > 0 ? timeout_s : 1e6;
    const uint64_t budget_ns = (uint64_t)(budget * 1e9);
    cudaStream_t st = (cudaStream_t)stream;
    const int n = (int)e->m.size();
    for (int k = 0; k < n; ++k) {
        e->hparams[k] = make_params(e->m[k], budget_ns);
        if (e->fill) {
            e->hparams[k].fill_ctr = e->dfill;
            e->hparams[k].fill_need = (unsigned)n;
        }
    }
    QDFN_CUDA(cudaMemcpyAsync(e->dparams, e->hparams, sizeof(SimParams) * n, cudaMemcpyHostToDevice, st));
    if ((rc = members_reset(e->dparams, n, e->dfill, st))) return rc;
    const MembersKernel k = members_kernel(e->prec, e->Rk);
    const SimParams* dp = e->dparams;
    const int2* dm = e->dmap;
    void* args[] = {&dp, &dm, &nsteps};
    QDFN_CUDA(cudaLaunchCooperativeKernel((const void*)k, dim3(e->total), dim3(kSimThreads), args, e->smem, st));
    if ((rc = members_status(e->dparams, n, e->dstat, e->dbusy, st))) return rc;
    QDFN_CUDA(cudaMemcpyAsync(e->hstat, e->dstat, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    QDFN_CUDA(cudaMemcpyAsync(e->hbusy, e->dbusy, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, st));
    e->busy_valid = false;   // current once the run is synchronised
    e->pending = st;
    e->running = true;
    return QDFN_OK;
}

extern "C" int qdfn_ensemble_sync(qdfn_ensemble* e) {
    if (!e) return fail(QDFN_ERR_INVALID, "null ensemble");
    if (!e->running) return QDFN_OK;
    e->running = false;
    QDFN_CUDA(cudaStreamSynchronize(e->pending));
    e->busy_valid = true;
    for (size_t k = 0; k < e->m.size(); ++k)
        if (e->hstat[k] != 0) return fail(e->hstat[k], "ensemble member " + std::to_string(k) + " stopped");
    return QDFN_OK;
}

extern "C" int qdfn_ensemble_state_bytes(const qdfn_ensemble* e, int64_t* bytes) {
    if (!e || !bytes) return fail(QDFN_ERR_INVALID, "null argument");
    *bytes = e->stage_words * 8;
    return QDFN_OK;
}

extern "C" int qdfn_ensemble_set_state_all(qdfn_ensemble* e, const void* host, void* stream) {
    int rc = ensemble_check(e);
    if (rc) return rc;
    if (!host) return fail(QDFN_ERR_INVALID, "null host buffer");
    if (e->running) return fail(QDFN_ERR_STATE, "a run is in flight (qdfn_ensemble_get_state_all first)");
    cudaStream_t st = (cudaStream_t)stream;
    QDFN_CUDA(cudaMemcpyAsync(e->dstage, host, (size_t)e->stage_words * 8, cudaMemcpyHostToDevice, st));
    return members_xfer(e->dxfer, (int)e->m.size(), e->dstage, 0, st);
}

extern "C" int qdfn_ensemble_get_state_all(qdfn_ensemble* e, void* host, void* stream, int wait) {
    if (!e || !host) return fail(QDFN_ERR_INVALID, "null argument");
    for (size_t k = 0; k < e->m.size(); ++k)
        if (!e->m[k]) return fail(QDFN_ERR_STATE, "member " + std::to_string(k) + " was destroyed");
    cudaStream_t st = (cudaStream_t)stream;
    const bool completes = e->running && e->pending == st;
    if (e->running && !completes) return fail(QDFN_ERR_STATE, "the run in flight is on another stream");
    if (completes && !wait) return fail(QDFN_ERR_INVALID, "reading the state of a run in flight needs wait=1");
    int rc = members_xfer(e->dxfer, (int)e->m.size(), e->dstage, 1, st);
    if (rc) return rc;
    QDFN_CUDA(cudaMemcpyAsync(host, e->dstage, (size_t)e->stage_words * 8, cudaMemcpyDeviceToHost, st));
    if (!wait) return QDFN_OK;
    if (completes) return qdfn_ensemble_sync(e);   // the run's outcome arrived with the state
    QDFN_CUDA(cudaStreamSynchronize(st));
    return QDFN_OK;
}

extern "C" int qdfn_ensemble_set_fill(qdfn_ensemble* e, int on) {
    if (!e) return fail(QDFN_ERR_INVALID, "null ensemble");
    if (e->running) return fail(QDFN_ERR_STATE, "a run is in flight");
    e->fill = on ? 1 : 0;
    return QDFN_OK;
}

extern "C" int qdfn_ensemble_run(qdfn_ensemble* e, int64_t nsteps, double timeout_s) {
    int rc = qdfn_ensemble_run_async(e, nsteps, timeout_s, nullptr);
    if (rc) return rc;
    return qdfn_ensemble_sync(e);
}

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
        rows<<<(unsigned)((tot + 31) / 32), 256>>>(p);   // 32 rows per block
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
            if (B.nr > ((int64_t)1 << 20) * hmat::kSliceRows) return fail(QDFN_ERR_INVALID, "block too tall");
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
    // warp tasks, largest first: pass A one per (low-rank block, group of
    // rows_a rank rows) (cost ns x rows), pass B one per (block, 64-row slice)
    // (cost rows x inner size; a rank-0 block's task writes zero partials)
    const int ga = Rk <= 2 ? hmat::rows_a<1>() : hmat::rows_a<4>();
    std::vector<std::pair<int64_t, int64_t>> ta, tb;   // (cost, code)
    for (int64_t q = 0; q < 2 * nb; ++q) {
        const hmat::Blk& B = blk[q];
        for (int64_t kk = 0; kk < B.rank; kk += ga)
            ta.push_back({B.ns * std::min<int64_t>(ga, B.rank - kk), (q << 8) | kk});
        const int64_t inner = B.rank < 0 ? B.ns : B.rank;
        const int64_t nt = (B.nr + hmat::kSliceRows - 1) / hmat::kSliceRows;
        for (int64_t t = 0; t < nt; ++t)
            tb.push_back({std::min<int64_t>(hmat::kSliceRows, B.nr - t * hmat::kSliceRows) * inner, (q << 20) | t});
    }
    auto by_cost = [](const std::pair<int64_t, int64_t>& x, const std::pair<int64_t, int64_t>& y) {
        return x.first != y.first ? x.first > y.first : x.second < y.second;
    };
    std::sort(ta.begin(), ta.end(), by_cost);
    // pass B: the dense blocks' tasks first (they need nothing from pass A),
    // each part largest first
    std::stable_partition(tb.begin(), tb.end(),
                          [&](const std::pair<int64_t, int64_t>& x) { return blk[x.second >> 20].rank < 0; });
    const int64_t n_dense = (int64_t)std::count_if(
        tb.begin(), tb.end(), [&](const std::pair<int64_t, int64_t>& x) { return blk[x.second >> 20].rank < 0; });
    std::sort(tb.begin(), tb.begin() + n_dense, by_cost);
    std::sort(tb.begin() + n_dense, tb.end(), by_cost);
    std::vector<int64_t> lr, tiles;
    for (auto& x : ta) lr.push_back(x.second);
    for (auto& x : tb) tiles.push_back(x.second);
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
    h.n_tiles_dense = n_dense;
    h.a_done = c->tile_ctr;   // reset in every launch's prologue
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
