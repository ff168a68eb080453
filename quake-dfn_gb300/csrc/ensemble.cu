// Ensemble launch kernels: k_sim_members (several contexts in one cooperative
// grid, sim_kernel.cuh) instantiated for every operator format and instance
// count, plus the small kernels around it -- clearing every member's error
// flag and barrier arrivals before the launch, gathering every member's
// outcome into one array after it, and moving every member's state to or from
// one staging buffer (the ensemble's one-copy state transfer).  The host side (qdfn_ensemble_*)
// is in sim.cu beside the context it drives.
#include "ensemble_kernels.h"
#include "sim_kernel.cuh"

namespace qdfn {
namespace {

// one thread per member: error flag and barrier arrivals (adjacent words);
// thread 0 also clears the fill-mode counter
__global__ void k_members_reset(const SimParams* __restrict__ members, int n, unsigned* fill) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m == 0 && fill) *fill = 0u;
    if (m >= n) return;
    members[m].gerr[0] = 0;
    *members[m].bar_count = 0u;
}

// one thread per member: the first failing instance's status, else the
// launch's error flag, else 0; and the member's busy ns so far (the
// autotuner's measure, read back with the status instead of member by member)
__global__ void k_members_status(const SimParams* __restrict__ members, int n, int* __restrict__ out,
                                 unsigned long long* __restrict__ busy) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const SimParams& p = members[m];
    int s = 0;
    for (int r = 0; r < p.R && s == 0; ++r) s = p.status[r];
    if (s == 0) s = p.gerr[0];
    out[m] = s;
    busy[m] = p.prof ? p.prof[0] + p.prof[1] + p.prof[2] + p.prof[3] : 0ull;
}

// the state of every member to or from one staging buffer: blockIdx.y is the
// member, the x blocks stride its words (coalesced on both sides)
__global__ void k_members_xfer(const XferMember* __restrict__ dm, double* __restrict__ stage, int dir) {
    const XferMember m = dm[blockIdx.y];
    const int64_t rn = (int64_t)m.R * m.N, words = 6 * rn + 3 * (int64_t)m.R;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < words; w += (int64_t)gridDim.x * blockDim.x) {
        double* dev;
        if (w < 6 * rn) {
            const int64_t f = w / rn;
            dev = m.state6 + f * (int64_t)m.Rk * m.N + (w - f * rn);
        } else {
            const int64_t s = w - 6 * rn;
            const int k = (int)(s / m.R), r = (int)(s - (int64_t)k * m.R);
            dev = k == 0 ? m.T + r : (k == 1 ? m.dt + r : reinterpret_cast<double*>(m.step + r));
        }
        if (dir == 0) *dev = stage[m.off + w];   // (step words move as raw 8-byte patterns)
        else stage[m.off + w] = *dev;
    }
}

template <class M>
MembersKernel pick(int R) {
    switch (R) {
        case 1: return k_sim_members<M, 1>;
        case 2: return k_sim_members<M, 2>;
        default: return k_sim_members<M, 4>;
    }
}

}  // namespace

MembersKernel members_kernel(int prec, int R) {
    if (prec == QDFN_FP64) return pick<FmtF64>(R);
    if (prec == QDFN_FP32) return pick<FmtF32>(R);
    return pick<FmtBF16x2>(R);
}

int members_reset(const SimParams* dmembers, int n, unsigned* dfill, cudaStream_t st) {
    k_members_reset<<<(n + 127) / 128, 128, 0, st>>>(dmembers, n, dfill);
    QDFN_CUDA(cudaGetLastError());
    return QDFN_OK;
}

int members_xfer(const XferMember* dm, int n, double* stage, int dir, cudaStream_t st) {
    if (n <= 0) return QDFN_OK;
    k_members_xfer<<<dim3(32, (unsigned)n), 256, 0, st>>>(dm, stage, dir);
    QDFN_CUDA(cudaGetLastError());
    return QDFN_OK;
}

int members_status(const SimParams* dmembers, int n, int* dout, unsigned long long* dbusy, cudaStream_t st) {
    k_members_status<<<(n + 127) / 128, 128, 0, st>>>(dmembers, n, dout, dbusy);
    QDFN_CUDA(cudaGetLastError());
    return QDFN_OK;
}

}  // namespace qdfn
