/*
 * qdfn.h -- C ABI of libqdfn.so, the GB300 (sm_103a) implementation of the
 * Quake-DFN earthquake-cycle hot path.
 *
 * Conventions
 *   - Every function returns int: 0 (QDFN_OK) or a negative QDFN_ERR_* code;
 *     nothing throws across the ABI.  qdfn_last_error() gives the message of the
 *     last failure on the calling thread.
 *   - Functions without a _dev suffix take HOST pointers owned by the caller;
 *     the data are copied during the call.  _dev functions take DEVICE pointers
 *     and a cudaStream_t passed as void*.
 *   - Indices are 0-based.  A matrix argument has a `layout`:
 *       QDFN_LAYOUT_ROW (0): K[r * ld + s]   (row = receiver, C order)
 *       QDFN_LAYOUT_COL (1): K[s * ld + r]   (Julia's column-major K[recv, src])
 *   - One context is driven by one host thread at a time; contexts are
 *     independent of each other.
 *   - Angles are in degrees; lengths in metres; stresses in Pa.
 *
 * Reference interfaces replaced (paths inside limkjae/Quake-DFN):
 *   assembly   scripts/Functions_BuildInputFile.jl:386  StiffnessMatrix_ByParts_Calculation_Rec
 *              scripts/Functions_BuildInputFile.jl:516  BuildMatrixByParts_Even_Rec
 *              scripts/Functions_BuildInputFile.jl:551  StiffnessMatrix_ByParts_Calculation_Tri
 *              scripts/Functions_BuildInputFile.jl:599  BuildMatrixByParts_Even_Tri
 *              scripts/Functions_OKADA3D.jl:464         Okada_DC3D_Vector
 *              scripts/Functions_TDstressHS.jl:2        TDstressHS
 *   simulation scripts/Functions_RSFDFN3DMain_D.jl:2     main   (dense)
 *              scripts/Functions_RSFDFN3DMain_H.jl:2     main_H (H-matrix)
 *              scripts/Functions_Solvers.jl:334          SolveOneTimeStep (+ :26, :185, :2, :465)
 *              scripts/Functions_Hmatrix.jl:631          HmatSolver_Pararllel
 */
#ifndef QDFN_H
#define QDFN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QDFN_OK 0
#define QDFN_ERR_INVALID -1      /* bad argument */
#define QDFN_ERR_CUDA -2         /* CUDA runtime error */
#define QDFN_ERR_NOMEM -3        /* device allocation failed */
#define QDFN_ERR_STATE -4        /* call out of order (e.g. run before set_dense) */
#define QDFN_ERR_DOMAIN -10      /* log/sqrt of a negative number (Julia DomainError) */
#define QDFN_ERR_EMPTY -11       /* minimum over an empty set in the time-step control */
#define QDFN_ERR_RETRIES -12     /* retry loop of one step passed its cap */
#define QDFN_ERR_NO_CONVERGE -13 /* per-patch iteration passed its cap */
#define QDFN_ERR_TIMEOUT -14     /* device-side deadline passed (kernel returned early) */
#define QDFN_ERR_HALF_SPACE -15  /* triangle vertex or receiver above the free surface */

#define QDFN_LAYOUT_ROW 0
#define QDFN_LAYOUT_COL 1

/* storage precision of the elastic operator */
#define QDFN_FP64 0
#define QDFN_FP32 1
#define QDFN_BF16X2 2   /* value = hi + lo, both bfloat16 (4 bytes per entry) */

/* ---- library ------------------------------------------------------------ */
/* Version string of the library. */
const char* qdfn_version(void);
/* Message for a status code. */
const char* qdfn_status_string(int status);
/* Copies the last error message of the calling thread into buf (NUL-terminated). */
int qdfn_last_error(char* buf, size_t n);

/* ---- stiffness assembly -------------------------------------------------- */
/* Rectangular patches, Okada (1992) DC3D.  src/recv are n x 8 row-major records
 *   {centre_x, centre_y, centre_z (depth, positive down), strike length,
 *    dip length, strike, dip, rake}.
 * Ks, Kn: n_recv x n_src in `layout` with leading dimension n_recv (COL) or
 * n_src (ROW).  Replaces StiffnessMatrix_ByParts_Calculation_Rec
 * (Functions_BuildInputFile.jl:386-512) and its part driver (:516-548). */
int qdfn_assemble_rect(int64_t n_src, const double* src, int64_t n_recv, const double* recv,
                       double shear_modulus, double poisson, double* Ks, double* Kn, int layout);
/* Device-pointer form; ld is the leading dimension of Ks/Kn. */
int qdfn_assemble_rect_dev(int64_t n_src, const double* src, int64_t n_recv, const double* recv,
                           double shear_modulus, double poisson, double* Ks, double* Kn,
                           int64_t ld, int layout, void* stream);

/* Triangular patches, Nikkhoo & Walter (2015) TDstressHS.
 * P1,P2,P3: n_src x 3 vertices (z <= 0, up positive, already reordered by
 * RotVerts_UnitVectors), rake: n_src; centre, nhat, shat: n_recv x 3 receiver
 * centroids, unit normals and unit slip vectors.  Replaces
 * StiffnessMatrix_ByParts_Calculation_Tri (Functions_BuildInputFile.jl:551-594). */
int qdfn_assemble_tri(int64_t n_src, const double* P1, const double* P2, const double* P3,
                      const double* rake, int64_t n_recv, const double* centre, const double* nhat,
                      const double* shat, double shear_modulus, double poisson, double* Ks,
                      double* Kn, int layout);
int qdfn_assemble_tri_dev(int64_t n_src, const double* P1, const double* P2, const double* P3,
                          const double* rake, int64_t n_recv, const double* centre,
                          const double* nhat, const double* shat, double shear_modulus,
                          double poisson, double* Ks, double* Kn, int64_t ld, int layout,
                          void* stream);

/* Gathered entries of the triangle stiffness (device pointers): for pair k,
 * Ks[k], Kn[k] = the (receiver recv_idx[k], source src_idx[k]) entries of
 * StiffnessMatrix_ByParts_Calculation_Tri (Functions_BuildInputFile.jl:551-594),
 * indices into the same per-triangle arrays as qdfn_assemble_tri_dev.  The
 * rows and columns that adaptive cross approximation of an H-matrix block asks
 * for (the role of HmatBuild_T's block assembly, :643-723), formed without
 * assembling the block. */
int qdfn_assemble_tri_pairs_dev(int64_t npairs, const int64_t* recv_idx, const int64_t* src_idx,
                                const double* P1, const double* P2, const double* P3, const double* rake,
                                const double* centre, const double* nhat, const double* shat,
                                double shear_modulus, double poisson, double* Ks, double* Kn, void* stream);

/* ---- cycle simulation ------------------------------------------------------ */
typedef struct qdfn_ctx qdfn_ctx;

/* Problem description.  Per-patch arrays have length n_inst * N (instance-major:
 * instance k owns [k*N, (k+1)*N)); instances share the elastic operator and the
 * loading-fault count (friction draws on one geometry).  Fields follow the
 * positional arguments of main() (Functions_RSFDFN3DMain_D.jl:2-8). */
typedef struct qdfn_problem {
    int64_t N;              /* FaultCount */
    int64_t Nload;          /* LoadingFaultCount (the last Nload patches) */
    int32_t n_inst;         /* instances sharing the operator (1..4) */
    int32_t evolution_dr;   /* EvolutionDR: 1 aging law, otherwise slip law */
    const double* a;        /* length n_inst*N each */
    const double* b;
    const double* Dc;
    const double* theta_i;
    const double* V_i;
    const double* f_i;      /* FrictionI */
    const double* sigma0;   /* InitialNormalStress */
    const double* V_const;  /* LoadingRate */
    const double* mass;     /* Mass */
    double G;               /* ShearModulus */
    double rho;             /* RockDensity */
    double sigma_min;       /* MinimumNormalStress */
    double switch_v;        /* SwitchV */
    double dt_cut;          /* DtCut */
    double rupture_dt;      /* RuptureDt */
    double max_dt;          /* MaximumDt */
    double alpha_evo;       /* Alpha_Evo */
    int32_t interp_at_told; /* 0: external stress at TOld+Dt (main); 1: at TOld (main_H) */
    int32_t reserved;
    int64_t record_step;    /* RecordStep (0 = no history) */
    int64_t max_records;    /* capacity of the history buffers, in records */
} qdfn_problem;

/* Creates a context (device allocations) and initialises the state the way
 * main()/main_H() do before their step loop. */
int qdfn_ctx_create(qdfn_ctx** out, const qdfn_problem* p);
int qdfn_ctx_destroy(qdfn_ctx* ctx);

/* Dense operator.  Ks/Kn are N x N in `layout` with leading dimension ld.
 * Forms ElasticLoadingShearMatrix = K_ij/K_ii (zero diagonal) and K_Self =
 * |K_ii| as main() does (Functions_RSFDFN3DMain_D.jl:53-67) and stores both
 * matrices in `precision` (QDFN_FP64, QDFN_FP32, QDFN_BF16X2). */
int qdfn_set_dense(qdfn_ctx* ctx, const double* Ks, const double* Kn, int64_t ld, int layout,
                   int precision);
/* Device-pointer form of qdfn_set_dense (FP64 Ks/Kn already in device memory,
 * e.g. straight from qdfn_assemble_rect_dev); the call waits on `stream`. */
int qdfn_set_dense_dev(qdfn_ctx* ctx, const double* Ks, const double* Kn, int64_t ld, int layout,
                       int precision, void* stream);

/* ---- H-matrix structure on the device ------------------------------------ */
/* The cluster tree and block partition of an H-matrix operator, built on the
 * GPU (replaces GroupAndSort_AllLevel / BuildHierarchy,
 * scripts/Functions_Hmatrix.jl:1-212, whose k-means tree is randomly
 * initialised).  centres: host [N][3] element centres.  Level by level, every
 * node of more than `leaf` elements orders its elements along the longest
 * axis of its box (ties: lower axis, then lower element index) and splits its
 * range in halves (a k-d tree of median splits), and a (receiver node, source
 * node) pair is a low-rank
 * block when its boxes are apart (dist > 0) and max(diameter) <= eta * dist, a
 * dense block when both nodes are leaves, and is split otherwise.
 * qdfn_hstruct_get: perm [N] (element at each position), ranges [n_blocks][4]
 * (source first, source last, receiver first, receiver last, inclusive,
 * positions of the order -- the ElementRange_SR form, 0-based) and
 * admissible [n_blocks] (1 low-rank), blocks ordered by receiver then source
 * start.  Any pointer may be NULL. */
typedef struct qdfn_hstruct qdfn_hstruct;
int qdfn_hstruct_build(qdfn_hstruct** out, int64_t N, const double* centres, int leaf, double eta);
int qdfn_hstruct_sizes(const qdfn_hstruct* h, int64_t* n_blocks, int64_t* n_nodes);
int qdfn_hstruct_get(const qdfn_hstruct* h, int64_t* perm, int64_t* ranges, int32_t* admissible);
int qdfn_hstruct_destroy(qdfn_hstruct* h);

/* H-matrix operator (Functions_Hmatrix.jl).  nb blocks; range is nb x 4
 * {src_begin, src_end, recv_begin, recv_end}, 0-based inclusive (the
 * reference's ElementRange_SR minus one).  For block b and each of the shear (s)
 * and normal (n) matrices: rank < 0 -> dense block D (recv x src, row-major);
 * rank >= 0 -> low-rank U (recv x rank) * Vt (rank x src), both row-major.
 * Diagonal blocks must be dense; K_Self = -K_ii and the diagonal of the shear
 * blocks is zeroed (StiffnessTransitionToLoading, Functions_Hmatrix.jl:459-477). */
int qdfn_set_hmatrix(qdfn_ctx* ctx, int64_t nb, const int64_t* range, const int64_t* rank_s,
                     const double* const* U_s, const double* const* Vt_s,
                     const double* const* D_s, const int64_t* rank_n,
                     const double* const* U_n, const double* const* Vt_n,
                     const double* const* D_n, int precision);

/* External stress history (Input_ExternalStressChange.jld2): nt samples of
 * time t[nt] and nt x N row-major normal, shear and pressure changes, shared by
 * all instances.  Interpolated as InterpolateFromStressChange
 * (Functions_Solvers.jl:465-540). */
int qdfn_set_external_stress(qdfn_ctx* ctx, int64_t nt, const double* t, const double* dsn,
                             const double* dtau, const double* dp);

/* Advances every instance by nsteps time steps.  timeout_s bounds the wall time
 * of the call (0 = no bound); on expiry the device loop stops at its next
 * barrier and QDFN_ERR_TIMEOUT is returned.  A failing instance stops the run
 * and its status is returned. */
int qdfn_run(qdfn_ctx* ctx, int64_t nsteps, double timeout_s);
/* As qdfn_run, enqueued on `stream` without waiting; query with qdfn_sync. */
int qdfn_run_async(qdfn_ctx* ctx, int64_t nsteps, double timeout_s, void* stream);
int qdfn_sync(qdfn_ctx* ctx);

/* Number of device kernels one qdfn_run launches (for launch accounting). */
int qdfn_kernels_per_run(const qdfn_ctx* ctx);

/* Cap the thread blocks (one per SM) a context's runs use; 0 = every SM
 * (default).  The operator tiling is re-sized for the cap.  To run several
 * contexts at once, group them in an ensemble (qdfn_ensemble_*, below): one
 * cooperative launch holds every member, so their blocks are co-resident;
 * separate cooperative launches on different streams carry no such guarantee,
 * and a member whose blocks are not all resident waits at its grid barrier
 * until its time budget ends the run.  qdfn_get_blocks returns the block count
 * of the next run (-1 for a null context).  No counterpart in the reference,
 * which runs one geometry per process. */
int qdfn_set_blocks(qdfn_ctx* ctx, int nblocks);
int qdfn_get_blocks(const qdfn_ctx* ctx);

/* Dense FP32/BF16 operator: column chunks of the NEXT step that a step's
 * operator warps stream during its own solve tail (0..64; default 64, i.e. as
 * many as are ready).  0 turns the early stream off: the operator warps then
 * join the solves once their own tiles are in, which pays where a context is
 * bound by its FP64 patch solves rather than by its operator stream (small
 * ensemble members).  Results are bit-identical for every value; only the
 * schedule changes.  qdfn_get_early_cols returns the setting (-1 for a null
 * context).  No counterpart in the reference. */
int qdfn_set_early_cols(qdfn_ctx* ctx, int cols);
int qdfn_get_early_cols(const qdfn_ctx* ctx);

/* ---- ensembles: many contexts in one persistent launch ------------------- */
/* Batched ensembles of fault networks of uneven size (no counterpart in the
 * reference, which runs one geometry per Julia process; each member is the
 * state of one `main` call, scripts/Functions_RSFDFN3DMain_D.jl:2-324).  An
 * ensemble advances n member contexts -- each with its own dense operator, up
 * to 4 friction draws, state, external stress and adaptive time steps -- in ONE
 * cooperative launch: member k runs on its own contiguous range of blocks (its
 * share of the SMs) with its own grid barrier, so members never wait on one
 * another, and one grid holds them all, so every member's blocks are
 * co-resident by the cooperative launch's guarantee.  All members must hold a
 * dense operator of the same precision and the same instance count class
 * (1, 2 or 3-4).  Members stay ordinary contexts (their state, history and
 * counter calls work between runs); while an ensemble run is in flight, run
 * no member on its own.  Destroy the ensemble before its members (a member
 * destroyed first makes later ensemble runs fail with QDFN_ERR_STATE).
 *
 * blocks: blocks per member (each >= 1), or NULL for a split proportional to
 * an estimate of each member's per-step cost (operator bytes + patch solves).
 * The sum must fit on the GPU at once (one block per SM), so n <= SM count. */
typedef struct qdfn_ensemble qdfn_ensemble;
int qdfn_ensemble_create(qdfn_ensemble** out, int n, qdfn_ctx* const* members, const int* blocks);
int qdfn_ensemble_destroy(qdfn_ensemble* ens);
/* Blocks each member runs on (n ints). */
int qdfn_ensemble_get_blocks(const qdfn_ensemble* ens, int* blocks);
/* Re-divides the SMs (NULL: the cost estimate). */
int qdfn_ensemble_set_blocks(qdfn_ensemble* ens, const int* blocks);
/* Autotuner step: re-divides the SMs in proportion to each member's measured
 * cost since the last balance (its busy time on the device times its blocks),
 * so that members taking the same number of steps finish together.  Call it
 * between runs, e.g. a few times during warm-up.  The column chunking of a
 * member's FP32/BF16 products follows its block count, so a new split can
 * change results in the last bits of the operator sums. */
int qdfn_ensemble_balance(qdfn_ensemble* ens);
/* Advances every instance of every member by nsteps of its own time steps in
 * one launch (timeout_s as for qdfn_run, per member).  _async enqueues on
 * `stream`; qdfn_ensemble_sync waits and returns the first failing member's
 * status. */
int qdfn_ensemble_run(qdfn_ensemble* ens, int64_t nsteps, double timeout_s);
/* Fill mode (off by default): in a run of nsteps, a member that has taken its
 * nsteps keeps stepping until every member has taken at least nsteps, so no SM
 * idles while the slowest member finishes; members then hold nsteps or more
 * steps each (read their step counts back).  The extra steps are ordinary
 * steps of each member's own trajectory. */
int qdfn_ensemble_set_fill(qdfn_ensemble* ens, int on);

/* All members' state in ONE host<->device copy each way (an ensemble's
 * end-to-end step: state up, one ensemble step, state down).  The host buffer
 * (qdfn_ensemble_state_bytes bytes; pinned for asynchronous copies) holds, member
 * after member in the order given at creation, the six fields of
 * qdfn_set_state_all as [6][n_inst][N] doubles (V, D, theta, friction, accel,
 * sigma_old), then T[n_inst], dt[n_inst] and step[n_inst] (int64) as 8-byte
 * words.  set: enqueued on `stream`; no run may be in flight.  get: enqueued on
 * `stream`; with wait = 1 it returns once the state is on the host, and if an
 * ensemble run is in flight on the same stream it completes that run (its
 * outcome is returned, as qdfn_ensemble_sync does).  The per-context calls
 * qdfn_set_state_all / qdfn_get_state_all move the same data member by member;
 * no counterpart in the reference, which runs one geometry per process. */
int qdfn_ensemble_state_bytes(const qdfn_ensemble* ens, int64_t* bytes);
int qdfn_ensemble_set_state_all(qdfn_ensemble* ens, const void* host, void* stream);
int qdfn_ensemble_get_state_all(qdfn_ensemble* ens, void* host, void* stream, int wait);
int qdfn_ensemble_run_async(qdfn_ensemble* ens, int64_t nsteps, double timeout_s, void* stream);
int qdfn_ensemble_sync(qdfn_ensemble* ens);
/* Host-only split rule used above: with member k taking cost[k] / b on b
 * blocks, out[k] >= 1 blocks minimising the longest member time, summing to
 * nsm (cost[k] > 0, n <= nsm). */
int qdfn_ensemble_shares(int n, const double* cost, int nsm, int* out);
/* Cumulative device counters of the context's runs (first n of): ns spent in
 * [0] time-step control, [1] elastic operator, [2] friction solves and retries,
 * [3] state rotation; [4] solve passes (1 + retries per step), [5] steps;
 * [6] low-velocity patch solves, [7] their secant iterations, [8] high-velocity
 * patch solves, [9] their secant iterations (summed over patches, instances
 * (padding instances included) and solve passes); [10] ns of [2] that the
 * first block spent on its own solves and block reduction, [11] ns of [2] it
 * waited at the grid barrier after them; [12]/[13] ns the first block's
 * operator warps / solver warps spent in the overlapped operator-and-solve
 * phase (FP32/BF16 dense operator), [14]/[15] the same for the slowest block of
 * each step, [16] the longest time from a row block being complete to one of
 * its row chunks being solved, [17] the time from a block's start of the
 * overlapped phase to the step's last row block being complete (per-step
 * maxima, summed over steps). */
int qdfn_get_counters(const qdfn_ctx* ctx, int64_t* out, int n);

/* State of one instance (host copies).  Any pointer may be NULL. */
int qdfn_get_state(const qdfn_ctx* ctx, int inst, double* V, double* D, double* theta,
                   double* friction, double* accel, double* sigma_old, double* T, double* dt,
                   int64_t* step);
int qdfn_set_state(qdfn_ctx* ctx, int inst, const double* V, const double* D,
                   const double* theta, const double* friction, const double* accel,
                   const double* sigma_old, double T, double dt, int64_t step);

/* The state of every instance at once: host arrays [n_inst][N] (instance
 * major), scalars [n_inst]; any pointer may be NULL.  The copies are enqueued
 * on `stream` (a cudaStream_t as void*, NULL = default stream); from pinned
 * host memory they do not block the caller.  qdfn_get_state_all with wait = 1
 * synchronises the stream, and when the context's run is in flight on that
 * stream it completes the run like qdfn_sync (same status codes), so a host
 * loop set_state_all -> run_async -> get_state_all costs one synchronisation.
 * No counterpart in the reference (its state stays inside the Julia process);
 * they serve callers that keep the ensemble state on the host between steps. */
int qdfn_set_state_all(qdfn_ctx* ctx, const double* V, const double* D, const double* theta,
                       const double* friction, const double* accel, const double* sigma_old,
                       const double* T, const double* dt, const int64_t* step, void* stream);
int qdfn_get_state_all(qdfn_ctx* ctx, double* V, double* D, double* theta, double* friction,
                       double* accel, double* sigma_old, double* T, double* dt, int64_t* step,
                       void* stream, int wait);

/* History of one instance: records 0..*nrec-1 (History_Time, History_Dt and the
 * record x N arrays History_V/_Disp/_Theta/_NormalStress).  Any pointer may be
 * NULL; nrec receives the number of records written so far. */
int qdfn_get_history(const qdfn_ctx* ctx, int inst, double* T, double* Dt, double* V, double* D,
                     double* theta, double* sigma, int64_t* nrec);

/* Applies the stored operator once: tld = ElasticLoadingShearMatrix * (0 - D)
 * and knd = StiffnessMatrixNormal * D for every instance (D, tld, knd are
 * n_inst x N host arrays).  Exposed for operator-level tests. */
int qdfn_apply_operator(qdfn_ctx* ctx, const double* D, double* tld, double* knd);

/* K_Self of the stored operator (length N). */
int qdfn_get_kself(const qdfn_ctx* ctx, double* kself);

/* ---- adjoint ----------------------------------------------------------------- */
/* Reverse-mode gradient of a loss on the trajectory with respect to the
 * per-patch friction parameters a, b and Dc.  The reference has no derivatives;
 * this differentiates its step map (scripts/Functions_Solvers.jl:185-327 and
 * :26-182, the products at scripts/Functions_RSFDFN3DMain_D.jl:199-202 and the
 * time-step control at :162-201).
 *
 * Runs nsteps steps from the context's current state (one step per launch,
 * checkpointing the state every checkpoint_every steps; 0 = ceil(sqrt(nsteps))),
 * then sweeps them backwards: per step the implicit-function derivative of each
 * patch's converged solve, the transposed products E^T and Kn^T over the stored
 * operator (its precision), and the time step's derivative through the patch
 * that set it.  The context ends at the window's last state, as after qdfn_run.
 *
 * The loss enters through its derivatives: dL_dD_final ([n_inst][N], may be
 * NULL) on the slip after the last step, and n_seeds sparse terms on any state
 * of the window -- seed k adds seed_dV[k] and seed_dD[k] to the adjoint of
 * V and D of patch seed_patch[k] (-1: none) of instance seed_inst[k], and
 * seed_dT[k] to that of its time T, after step seed_step[k] (0 = the starting
 * state, nsteps = the last), e.g. the derivatives of an event onset time
 * interpolated between two steps.  Outputs dL_da, dL_db, dL_dDc are
 * [n_inst][N] host arrays.  Needs a dense operator and Alpha_Evo = 0. */
int qdfn_adjoint_run(qdfn_ctx* ctx, int64_t nsteps, int64_t checkpoint_every, const double* dL_dD_final,
                     int64_t n_seeds, const int64_t* seed_step, const int32_t* seed_inst,
                     const int64_t* seed_patch, const double* seed_dV, const double* seed_dD,
                     const double* seed_dT, double* dL_da, double* dL_db, double* dL_dDc, double timeout_s);

/* ---- allocation-free operator -------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (device memory owned by another allocator such as a Julia CUDA.jl pool or a
 * framework's caching allocator, or loops where allocation is not allowed):
 * the same products as qdfn_apply_operator -- tld = (K_ij/K_ii, zero diagonal)
 * * (0 - D) and knd = Kn * D, FP64 -- computed straight from caller-owned
 * DEVICE matrices Ks, Kn in source-major layout (Julia's column-major
 * K[recv, src]: entry (r, s) at s*ld + r) and device vectors D, tld, knd (length
 * N), enqueued on `stream`.  Allocates nothing: its scratch is a fixed 2 MiB
 * device array holding N <= 16384; larger N is rejected with QDFN_ERR_INVALID.
 * Each call made outside stream capture looks up the array's device address
 * (with the device current) and records it; calls made during capture use the
 * recorded one, so make the first call on each device before any capture.  All
 * calls on a device share the array: calls whose kernels overlap on the GPU
 * (other streams or host threads) race and must not be issued. */
int qdfn_apply_dense_noalloc(int64_t N, const double* Ks, const double* Kn, int64_t ld,
                             const double* D, double* tld, double* knd, void* stream);

/* ---- self-checks ------------------------------------------------------------ */
/* The friction solves divide by Dt, Dc, a and constants through a correctly
 * rounded reciprocal and one remainder correction (3 FP64 operations instead
 * of a full IEEE division), falling back to IEEE division outside
 * [2^-895, 2^896].  This evaluates that division on DEVICE arrays,
 * q[i] = x[i] / d[i], on `stream`, so that tests can compare it with IEEE
 * division.  No counterpart in the reference (Julia's `/`). */
int qdfn_check_division(int64_t n, const double* x, const double* d, double* q, void* stream);

/* ---- input parsing and discretisation (host only) ------------------------ */
/* The reference's RUN2 front end, so a caller goes from the bulk text file to
 * the segment table without Julia.  Tables are row-major doubles.  Two-call
 * pattern: with seg == NULL only the sizes are returned. */
typedef struct qdfn_bulk_info {
    double switch_ss_rn;             /* 1 strike-slip, 2 reverse/normal (LRtoRake) */
    double shear_modulus, poisson_ratio, rock_density;
    double drop_crit, drop_crit_ns_multiplier, minimum_ns;
    int32_t is_triangle;             /* 0: rectangles, 1: triangles */
    int32_t columns;                 /* segment columns: 19 (rectangles) or 20 (triangles) */
    int64_t fault_count;             /* segment rows */
    int64_t loading_fault_count;     /* rows with a constant loading velocity (sorted last) */
} qdfn_bulk_info;

/* Replaces ReadBulkInput (scripts/Functions_BuildInputFile.jl:216-274, with
 * LRtoRake :182-213 and BulkToSegment :82-179): parses the 18-column
 * (rectangle) or 20-column (triangle) bulk file, sorts by the loading column,
 * converts the +-1 slip sense to rake, grids rectangles into patches, and
 * writes `fault_count` rows of `columns` values to seg (cap_rows rows of room).
 * Malformed files return QDFN_ERR_INVALID (the reference raises). */
int qdfn_read_bulk_input(const char* path, qdfn_bulk_info* info, double* seg, int64_t cap_rows);

/* Replaces BulkToSegment (scripts/Functions_BuildInputFile.jl:82-179): nbulk
 * rows of 18 values (rake in degrees) to *nseg rows of 19. */
int qdfn_bulk_to_segment(int64_t nbulk, const double* bulk, double* seg, int64_t cap_rows, int64_t* nseg);

/* Replaces RotVerts_UnitVectors (scripts/Functions_BuildInputFile.jl:338-377):
 * per triangle (n x 3 vertex arrays) swaps P1/P2 where the unit normal's y
 * component is <= 0, then writes the unit normal, strike, dip and slip
 * vectors (rake in degrees). */
int qdfn_rot_verts_unit_vectors(int64_t n, const double* P1in, const double* P2in, const double* P3in,
                                const double* rake, double* P1, double* P2, double* P3, double* un,
                                double* us, double* ud, double* uslip);

#ifdef __cplusplus
}
#endif
#endif /* QDFN_H */
