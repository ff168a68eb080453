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
}

extern "C" int qdfn_run_async(qdfn_ctx* c, int64_t nsteps, double timeout_s, void* stream) {
    if (!c) return fail(QDFN_ERR_INVALID, "null context");
    if (c->ens && ensemble_running(c->ens)) return fail(QDFN_ERR_STATE, "the context's ensemble has a run in flight");
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
    if (c->ens) return fail(QDFN_ERR_STATE, "the context is an ensemble member (qdfn_ensemble_set_blocks)");
    c->nblocks_override = nblocks;
    return c->prec < 0 ? QDFN_OK : configure_launch(c);
}

extern "C" int qdfn_get_blocks(const qdfn_ctx* c) { return c ? c->nblocks : -1; }

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
    int2* dmap = nullptr;                // device [total]: (member, block within it)
    int* dstat = nullptr;                // device [n] outcome of the last run
    int* hstat = nullptr;                // pinned [n]
    cudaStream_t pending = nullptr;
    bool running = false;
    ~qdfn_ensemble() {
        if (hparams) cudaFreeHost(hparams);
        if (hstat) cudaFreeHost(hstat);
        if (dparams) cudaFree(dparams);
        if (dmap) cudaFree(dmap);
        if (dstat) cudaFree(dstat);
    }
};

namespace {

bool ensemble_running(const qdfn_ensemble* e) { return e->running; }

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
    for (int k = 0; k < n; ++k) {
        qdfn_ctx* c = e->m[k];
        c->nblocks_override = e->share[k];
        int rc = configure_launch(c);
        if (rc) return rc;
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
    if (e->dmap) cudaFree(e->dmap);
    e->dmap = nullptr;
    QDFN_CUDA(cudaMalloc(&e->dmap, sizeof(int2) * map.size()));
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
    double sum = 0;
    for (int k = 0; k < n; ++k) {
        if (!(cost[k] > 0) || !std::isfinite(cost[k])) return fail(QDFN_ERR_INVALID, "costs must be positive");
        sum += cost[k];
    }
    // at least one block each, then the rest by largest remainder of the ideal
    // (proportional) split; ties to the lower index
    std::vector<double> ideal(n);
    int used = 0;
    for (int k = 0; k < n; ++k) {
        ideal[k] = nsm * cost[k] / sum;
        out[k] = std::max(1, (int)std::floor(ideal[k]));
        used += out[k];
    }
    while (used > nsm) {   // the floors of 1 pushed the sum over: trim the largest
        int big = 0;
        for (int k = 1; k < n; ++k)
            if (out[k] > out[big]) big = k;
        --out[big];
        --used;
    }
    std::vector<int> order(n);
    for (int k = 0; k < n; ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return ideal[a] - out[a] > ideal[b] - out[b]; });
    for (int k = 0; k < n && used < nsm; ++k, ++used) ++out[order[k]];
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
                cudaMalloc(&e->dparams, sizeof(SimParams) * n) != cudaSuccess ||
                cudaMalloc(&e->dstat, sizeof(int) * n) != cudaSuccess))
        rc = fail(QDFN_ERR_NOMEM, "ensemble buffers");
    if (!rc) rc = ensemble_configure(e);
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
        now[k] = member_busy_ns(e->m[k]);
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
    for (int k = 0; k < n; ++k) e->hparams[k] = make_params(e->m[k], budget_ns);
    QDFN_CUDA(cudaMemcpyAsync(e->dparams, e->hparams, sizeof(SimParams) * n, cudaMemcpyHostToDevice, st));
    if ((rc = members_reset(e->dparams, n, st))) return rc;
    const MembersKernel k = members_kernel(e->prec, e->Rk);
    const SimParams* dp = e->dparams;
    const int2* dm = e->dmap;
    void* args[] = {&dp, &dm, &nsteps};
    QDFN_CUDA(cudaLaunchCooperativeKernel((const void*)k, dim3(e->total), dim3(kSimThreads), args, e->smem, st));
    if ((rc = members_status(e->dparams, n, e->dstat, st))) return rc;
    QDFN_CUDA(cudaMemcpyAsync(e->hstat, e->dstat, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    e->pending = st;
    e->running = true;
    return QDFN_OK;
}

extern "C" int qdfn_ensemble_sync(qdfn_ensemble* e) {
    if (!e) return fail(QDFN_ERR_INVALID, "null ensemble");
    if (!e->running) return QDFN_OK;
    e->running = false;
    QDFN_CUDA(cudaStreamSynchronize(e->pending));
    for (size_t k = 0; k < e->m.size(); ++k)
        if (e->hstat[k] != 0) return fail(e->hstat[k], "ensemble member " + std::to_string(k) + " stopped");
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
