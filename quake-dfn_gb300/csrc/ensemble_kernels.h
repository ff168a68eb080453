// Launch helpers of the ensemble kernels (ensemble.cu), used by the ensemble
// host code in sim.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "qdfn_internal.h"

namespace qdfn {

struct SimParams;   // sim_kernel.cuh

// k_sim_members<Format, R>: grid = the members' blocks, args (members, map, nsteps)
using MembersKernel = void (*)(const SimParams*, const int2*, int64_t);
MembersKernel members_kernel(int prec, int R);

// clears every member's error flag and barrier arrivals, and the fill-mode
// counter when dfill is not null (enqueued on st)
int members_reset(const SimParams* dmembers, int n, unsigned* dfill, cudaStream_t st);
// writes every member's outcome (first failing instance status, else the
// launch's error flag, else 0) to dout[n] and its cumulative busy ns (block
// 0's phase counters) to dbusy[n] (enqueued on st)
int members_status(const SimParams* dmembers, int n, int* dout, unsigned long long* dbusy, cudaStream_t st);

// One member's slice of an ensemble state transfer: its six state fields
// (kernel instance stride Rk x N, the first R instances moved), T, dt and step,
// at word `off` of the staging buffer ([6][R][N] doubles, then T[R], dt[R],
// step[R] as 8-byte words)
struct XferMember {
    double* state6;
    double* T;
    double* dt;
    int64_t* step;
    int64_t off, N;
    int R, Rk;
};
// dir 0: staging buffer -> members; 1: members -> staging buffer (enqueued on st)
int members_xfer(const XferMember* dm, int n, double* stage, int dir, cudaStream_t st);

}  // namespace qdfn
