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
// launch's error flag, else 0) to dout[n] (enqueued on st)
int members_status(const SimParams* dmembers, int n, int* dout, cudaStream_t st);

}  // namespace qdfn
