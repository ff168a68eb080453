// Device self-checks of the solver's arithmetic helpers, exposed for the
// test suite: the reciprocal-based division the friction solves use in place
// of IEEE division (sim_device.cuh div_by) evaluated on caller arrays.
#include <cuda_runtime.h>

#include "qdfn_internal.h"
#include "sim_device.cuh"

namespace qdfn {
namespace {

__global__ void k_check_division(int64_t n, const double* __restrict__ x, const double* __restrict__ d,
                                 double* __restrict__ q) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    q[i] = sim::div_by(x[i], sim::recip(d[i]));
}

}  // namespace
}  // namespace qdfn

using namespace qdfn;

extern "C" int qdfn_check_division(int64_t n, const double* x, const double* d, double* q, void* stream) {
    if (n < 0) return fail(QDFN_ERR_INVALID, "n < 0");
    if (n == 0) return QDFN_OK;
    if (!x || !d || !q) return fail(QDFN_ERR_INVALID, "null pointer");
    const int64_t blocks = (n + 255) / 256;
    if (blocks > 2147483647LL) return fail(QDFN_ERR_INVALID, "n too large");
    k_check_division<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(n, x, d, q);
    QDFN_CUDA(cudaGetLastError());
    return QDFN_OK;
}
