// Allocation-free variant of the dense elastic operator (the product of
// qdfn_apply_operator), for callers that cannot call cudaMalloc: processes
// whose device memory is owned by another allocator (a Julia CUDA.jl pool, a
// framework's caching allocator, a fixed-budget embedding) or real-time loops
// that forbid allocation.  Its scratch -- the per-column-chunk partial sums --
// lives in a file-scope __device__ array of fixed size, so the call itself
// allocates nothing.
//
// The scratch array is shared by every call on a device and keeps the last
// call's contents; each call overwrites every slot it reads, so nothing needs
// clearing.  Calls whose kernels overlap on the GPU (different streams, or
// different host threads) race on the scratch and must not be issued.
#include <cuda_runtime.h>

#include <mutex>

#include "qdfn_internal.h"

namespace qdfn {
namespace {

constexpr int64_t kNoAllocMaxN = 16384;   // largest N accepted
constexpr int kNoAllocChunks = 8;         // source-column chunks
constexpr int kNoAllocThreads = 256;      // 2 receiver rows per thread
constexpr int kMaxDevices = 64;

// [2 matrices][kNoAllocChunks][kNoAllocMaxN] FP64 partial sums: 2 MiB
__device__ __align__(256) double g_noalloc_scratch[2 * kNoAllocChunks * kNoAllocMaxN];

std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {nullptr};

// partial products of one column chunk for two receiver rows per thread;
// ELSM = K_ij / K_ii (zero diagonal) is formed on the fly exactly as the
// stored operator forms it
__global__ void __launch_bounds__(kNoAllocThreads)
k_noalloc_chunk(int64_t N, const double* __restrict__ Ks, const double* __restrict__ Kn, int64_t ld,
                const double* __restrict__ D, int64_t chunk, double* __restrict__ scratch) {
    const int c = blockIdx.y;
    const int64_t i0 = ((int64_t)blockIdx.x * kNoAllocThreads + threadIdx.x) * 2;
    if (i0 >= N) return;
    const int64_t j0 = (int64_t)c * chunk, j1 = min(N, j0 + chunk);
    const bool two = i0 + 1 < N;
    const double kii0 = Ks[i0 * ld + i0];
    const double kii1 = two ? Ks[(i0 + 1) * ld + i0 + 1] : 1.0;
    double s0 = 0, s1 = 0, n0 = 0, n1 = 0;
    for (int64_t j = j0; j < j1; ++j) {
        const double x = D[j];
        const double a0 = Ks[j * ld + i0];
        const double b0 = Kn[j * ld + i0];
        const double e0 = (j == i0) ? 0.0 : a0 / kii0;
        s0 = fma(e0, x, s0);
        n0 = fma(b0, x, n0);
        if (two) {
            const double a1 = Ks[j * ld + i0 + 1];
            const double b1 = Kn[j * ld + i0 + 1];
            const double e1 = (j == i0 + 1) ? 0.0 : a1 / kii1;
            s1 = fma(e1, x, s1);
            n1 = fma(b1, x, n1);
        }
    }
    scratch[(int64_t)c * kNoAllocMaxN + i0] = s0;
    scratch[(int64_t)(kNoAllocChunks + c) * kNoAllocMaxN + i0] = n0;
    if (two) {
        scratch[(int64_t)c * kNoAllocMaxN + i0 + 1] = s1;
        scratch[(int64_t)(kNoAllocChunks + c) * kNoAllocMaxN + i0 + 1] = n1;
    }
}

// chunk partials summed in chunk order: tld = ELSM (0 - D), knd = Kn D
__global__ void k_noalloc_reduce(int64_t N, int nchunk, const double* __restrict__ scratch,
                                 double* __restrict__ tld, double* __restrict__ knd) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double s = 0, n = 0;
    for (int c = 0; c < nchunk; ++c) {
        s += scratch[(int64_t)c * kNoAllocMaxN + i];
        n += scratch[(int64_t)(kNoAllocChunks + c) * kNoAllocMaxN + i];
    }
    tld[i] = -s;
    knd[i] = n;
}

// Device address of the scratch array on the current device.  The name
// g_noalloc_scratch is a host-side stand-in, not a device address.  A call
// made outside stream capture looks the address up (with the device current)
// and records it for that device; a call made while `st` is being captured
// uses the recorded address, so the first call on a device must come before
// any capture.  Looking it up on every uncaptured call keeps the address right
// after cudaDeviceReset, which may reload the module at another address.
int scratch_address(cudaStream_t st, double** out) {
    int dev = 0;
    QDFN_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(QDFN_ERR_INVALID, "device index out of range");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    QDFN_CUDA(cudaStreamIsCapturing(st, &cap));
    std::lock_guard<std::mutex> lock(g_mu);
    if (cap == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_scratch_addr[dev] = static_cast<double*>(p);
    } else if (!g_scratch_addr[dev]) {
        return fail(QDFN_ERR_STATE, "first call on this device made during stream capture");
    }
    *out = g_scratch_addr[dev];
    return QDFN_OK;
}

}  // namespace
}  // namespace qdfn

using namespace qdfn;

extern "C" int qdfn_apply_dense_noalloc(int64_t N, const double* Ks, const double* Kn, int64_t ld,
                                        const double* D, double* tld, double* knd, void* stream) {
    if (N < 1) return fail(QDFN_ERR_INVALID, "N must be >= 1");
    if (N > kNoAllocMaxN)
        return fail(QDFN_ERR_INVALID, "N = " + std::to_string(N) + " exceeds the allocation-free limit of " +
                                          std::to_string(kNoAllocMaxN) + " patches");
    if (ld < N) return fail(QDFN_ERR_INVALID, "ld < N");
    if (!Ks || !Kn || !D || !tld || !knd) return fail(QDFN_ERR_INVALID, "null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    double* scratch = nullptr;
    int rc = scratch_address(st, &scratch);
    if (rc) return rc;
    const int64_t chunk = (N + kNoAllocChunks - 1) / kNoAllocChunks;
    const int nchunk = (int)((N + chunk - 1) / chunk);
    const int64_t rows_per_blk = (int64_t)kNoAllocThreads * 2;
    dim3 grid((unsigned)((N + rows_per_blk - 1) / rows_per_blk), (unsigned)nchunk);
    k_noalloc_chunk<<<grid, kNoAllocThreads, 0, st>>>(N, Ks, Kn, ld, D, chunk, scratch);
    QDFN_CUDA(cudaGetLastError());
    k_noalloc_reduce<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(N, nchunk, scratch, tld, knd);
    QDFN_CUDA(cudaGetLastError());
    return QDFN_OK;
}
