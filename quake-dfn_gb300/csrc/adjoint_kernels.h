// Launchers and argument blocks of the adjoint kernels (adjoint.cu), used by
// the adjoint driver in sim.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "qdfn_internal.h"

namespace qdfn {

constexpr int kAdjMaxInst = 4;

// One reverse step's per-patch inputs and outputs ([R][N] unless noted).
struct AdjLocalArgs {
    int64_t N, Ns;
    int R, dr, interp_at_told;
    double eta, sigma_min;
    // the step: state before (prev) and after (cur), its TLD, sigma, solver
    const double *Vprev, *Dprev, *thprev, *Vcur, *tld, *sig;
    const unsigned char* sw;
    const double *dt, *Tprev;          // [R]: the step's dt and the time before it
    // run constants
    const double *pa, *pb, *pDc, *F0, *la, *lth0, *kself /*[N]*/, *mass, *omega, *tau0;
    int64_t n_ext;
    const double *ext_t, *ext_n, *ext_s, *ext_p;
    // adjoints of the step's outputs
    const double *lV, *lD, *lth, *lA;
    // adjoints of its inputs (D_old local part, V_old, theta_old, TLD, sigma)
    double *oDloc, *oVold, *oThold, *oTLD, *oSig;
    double *ga, *gb, *gDc;             // parameter gradients, accumulated
    double *blk_dt, *blk_tx;           // [blocks][R] partial sums
    double* sums;                      // [2R]: d/d(dt), d/d(external-stress time)
    int* err;                          // set when a residual's derivative vanishes
};

// Transposed products over the tile-contiguous operator (rpb rows per block).
struct AdjTransArgs {
    int64_t N, rpb, nrb;
    int64_t gx;                        // column blocks per row block
    const void *E, *Kn;
    const double *x_s, *x_n;           // [R][N]: lambda_TLD (E^T) and lambda_sigma (Kn^T)
    double* part;                      // [nrb][2][R][N]
};

int adj_local(const AdjLocalArgs& a, cudaStream_t st);
int adj_local_blocks(int64_t RN);
int adj_transpose_prepare(int prec, int R, int64_t rpb);
int adj_transpose(int prec, int R, const AdjTransArgs& a, const double* dloc, double* out, cudaStream_t st);
// lV[idx[k]] += vals[k], lD[idx[k]] += vals[n + k], lA[idx[k]] += vals[2n + k] (device arrays)
int adj_add(int n, const int64_t* idx, const double* vals, double* lV, double* lD, double* lA, cudaStream_t st);
int adj_dtctl(int R, int64_t N, int64_t Ns, const double* V, const double* A, const unsigned char* unstable,
              const int* has_unstable, double* out, cudaStream_t st);

}  // namespace qdfn
