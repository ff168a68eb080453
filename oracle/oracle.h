// CPU FP64 oracle of the Quake-DFN earthquake-cycle hot path.
//
// TEST INFRASTRUCTURE ONLY: the tests and the smoke check compare the GPU
// results with it, and the bench's CPU baseline leg times it.  The shipped
// CUDA library never includes, links or calls anything here.
//
// PARITY STATUS: the reference (pure Julia) ships no tests, golden vectors or
// fixtures, and Julia is not available to run it, so this restatement is
// pinned by physical known-answer tests (rectangle == two triangles, traction-
// free surface, reciprocity, decay, steady-state friction) rather than by the
// reference's own outputs -- "parity unpinned" in the strict sense.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// ---- Green's functions (per point) ----------------------------------------
// Functions_OKADA3D.jl:464 Okada_DC3D_Vector; out = UX,UY,UZ,UXX,UYX,UZX,UXY,UYY,UZY,UXZ,UYZ,UZZ
void oracle_okada_dc3d(double alpha, double x, double y, double z, double depth, double dip,
                       double al1, double al2, double aw1, double aw2, double disl1,
                       double disl2, double disl3, double out[12], int* iret);
// Functions_TDstressHS.jl:2 TDstressHS; stress/strain = xx,yy,zz,xy,xz,yz
int oracle_tdstress_hs(double x, double y, double z, const double P1[3], const double P2[3],
                       const double P3[3], double Ss, double Ds, double Ts, double mu,
                       double lambda, double stress[6], double strain[6]);

// ---- stiffness assembly ------------------------------------------------------
// Functions_BuildInputFile.jl:386 StiffnessMatrix_ByParts_Calculation_Rec.
// Patch arrays (length n): centre x,y,z (z = depth, positive down), strike length,
// dip length, strike, dip, rake (degrees).  Output K[r*n_src + s] (row = receiver).
void oracle_assemble_rect(int64_t n_src, const double* s_cx, const double* s_cy,
                          const double* s_cz, const double* s_ls, const double* s_ld,
                          const double* s_str, const double* s_dip, const double* s_rake,
                          int64_t n_recv, const double* r_cx, const double* r_cy,
                          const double* r_cz, const double* r_str, const double* r_dip,
                          const double* r_rake, double G, double nu, double* Ks, double* Kn,
                          int nthreads);
// Functions_BuildInputFile.jl:551 StiffnessMatrix_ByParts_Calculation_Tri.
// P1,P2,P3: n_src x 3 (row-major, z <= 0 up-positive); rake (deg);
// receiver centres n_recv x 3, unit normals and unit slip vectors n_recv x 3.
int oracle_assemble_tri(int64_t n_src, const double* P1, const double* P2, const double* P3,
                        const double* rake, int64_t n_recv, const double* centre,
                        const double* nhat, const double* shat, double G, double nu,
                        double* Ks, double* Kn, int nthreads);

// ---- cycle simulator (Functions_RSFDFN3DMain_D.jl / _H.jl) ------------------
typedef struct {
    int64_t N, Nload;
    const double *a, *b, *Dc, *theta_i, *V_i, *f_i, *sigma0, *V_const, *mass;
    double G, rho, sigma_min, switch_v, dt_cut, rupture_dt, max_dt, alpha_evo;
    int evolution_dr;
    int interp_at_told;  // 0: dense path (TOld+Dt), 1: H path (TOld)
    // external stress (optional): n_ext samples, rows of N values (row-major)
    int64_t n_ext;
    const double *ext_t, *ext_n, *ext_s, *ext_p;
} oracle_problem;

typedef struct {
    double T, dt;                 // TOld, Dt carried between steps
    int64_t step;                 // steps completed
    double *V, *D, *theta, *friction, *accel, *sigma_old;  // length N each
} oracle_state;

// Elastic operator: given DispOld, produce TLD (= Elastic_Load_Disp) and
// KnD (= StiffnessMatrixNormal * DispOld).
typedef struct oracle_operator oracle_operator;
// dense: Ks, Kn row-major N x N (row = receiver); builds ELSM = K_ij/K_ii
oracle_operator* oracle_op_dense(int64_t N, const double* Ks, const double* Kn, int nthreads);
// H-matrix: nb blocks; range[4*b..] = src_begin, src_end, recv_begin, recv_end (0-based
// inclusive, the reference's ElementRange_SR minus 1); block b is either dense
// (rank<0, Ds[b] = (recv x src) row-major) or low-rank U (recv x k) * Vt (k x src),
// both row-major.  Shear and normal blocks share the ranges.
oracle_operator* oracle_op_hmat(int64_t N, int64_t nb, const int64_t* range,
                                const int64_t* rank_s, const double* const* Us,
                                const double* const* Vts, const double* const* Ds,
                                const int64_t* rank_n, const double* const* Un,
                                const double* const* Vtn, const double* const* Dn,
                                int nthreads);
void oracle_op_free(oracle_operator* op);
// K_self as the simulator uses it (|K_ii| dense, -K_ii H)
void oracle_op_kself(const oracle_operator* op, double* kself);
void oracle_op_apply(const oracle_operator* op, const double* D, double* tld, double* knd);

// Initialise the state the way main()/main_H() do before their step loop.
void oracle_state_init(const oracle_problem* p, oracle_state* s);
// Advance nsteps steps.  hist_* (may be NULL) receive one row per RecordStep
// (History_Time/Dt/V/Disp/Theta/NormalStress); *n_rec is incremented.
// Returns 0, or a negative status (see codes below).
int oracle_run(const oracle_problem* p, const oracle_operator* op, oracle_state* s,
               int64_t nsteps, int64_t record_step, int64_t max_rec, double* hist_t,
               double* hist_dt, double* hist_V, double* hist_D, double* hist_theta,
               double* hist_sigma, int64_t* n_rec, int nthreads);

#define ORACLE_OK 0
#define ORACLE_ERR_DOMAIN -10        /* log/sqrt of a negative number (Julia DomainError) */
#define ORACLE_ERR_EMPTY -11         /* minimum over an empty collection (Julia ArgumentError) */
#define ORACLE_ERR_RETRIES -12       /* retry loop passed the hard cap */
#define ORACLE_ERR_NO_CONVERGE -13   /* per-patch iteration passed the hard cap */

#ifdef __cplusplus
}
#endif
