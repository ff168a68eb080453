// Kernels of the discrete adjoint of the stepped system (qdfn_adjoint_run in
// sim.cu drives them, one reverse step at a time):
//
//   k_adj_local      per (instance, patch): the vector-Jacobian product of the
//                    patch's converged step (adjoint.cuh) -- adjoints of the
//                    step's inputs D_old, V_old, theta_old, TLD, sigma, dtau,
//                    dt, and the parameter gradients a, b, Dc accumulated
//   k_adj_transpose  the transposed stiffness products E^T y and Kn^T z over
//                    the forward operator's tile-contiguous storage: each warp
//                    takes one column segment of a row block (2 KB, read once,
//                    coalesced) against R adjoint vectors staged in shared
//                    memory; FP32/BF16 storage multiplies in FP32 with the
//                    segment sum folded error-free into an (hi, lo) pair, FP64
//                    storage in FP64; one partial per (row block, instance,
//                    column), summed in row-block order by k_adj_combine
//   k_adj_combine    lambda_D(old) = local part - E^T lambda_TLD + Kn^T lambda_sigma
//   k_adj_dtctl      the time-step controller's reductions of a state (max V,
//                    min |V/Accel| and its patch), to route the adjoint of dt
//                    through the patch that set it
// The transposed product is the reverse pass's HBM-bound kernel (the operator
// bytes once per product); the local products are FP64 (dual numbers).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "adjoint.cuh"
#include "adjoint_kernels.h"
#include "qdfn_internal.h"

namespace qdfn {
namespace {

constexpr int kAdjThreads = 256;

// slope d/dt of the piecewise-linear external stress of patch column i at time
// Time (InterpolateFromStressChange, Functions_Solvers.jl:465-540): the ramp
// from zero before the first sample, the segment's slope inside, zero after the
// last sample
__device__ inline void interp_slope(int64_t nt, const double* t, const double* en, const double* es, int64_t N,
                                    int64_t i, double Time, double& sn, double& ss) {
    int64_t idx = 0;
    for (int64_t k = 1; k <= nt; ++k)
        if (Time >= t[k - 1]) idx = k;
    if (idx == 0) {
        sn = en[i] / t[0];
        ss = es[i] / t[0];
    } else if (idx == nt) {
        sn = ss = 0.0;
    } else {
        const double w = t[idx] - t[idx - 1];
        sn = (en[idx * N + i] - en[(idx - 1) * N + i]) / w;
        ss = (es[idx * N + i] - es[(idx - 1) * N + i]) / w;
    }
}

__global__ void __launch_bounds__(kAdjThreads) k_adj_local(AdjLocalArgs a) {
    __shared__ double s_dt[kAdjMaxInst][kAdjThreads / 32], s_tx[kAdjMaxInst][kAdjThreads / 32];
    const int64_t RN = (int64_t)a.R * a.N;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double ldt = 0, ltx = 0;   // this thread's share of d/d(dt) and of d/d(external-stress time)
    int r = -1;
    if (q < RN) {
        r = (int)(q / a.N);
        const int64_t i = q - (int64_t)r * a.N;
        const double dt = a.dt[r];
        const double lV = a.lV[q], lD = a.lD[q], lth = a.lth[q], lA = a.lA[q];
        const double Vold = a.Vprev[q];
        double lDloc = 0, lVold = 0, lThold = 0, lTLD = 0, lSig = 0;
        if (a.sw[q] == 2) {   // loading fault: D += Vc dt, theta kept, V = Vc
            const double Vn = a.Vcur[q];
            lDloc = lD;
            lThold = lth;
            lVold = -lA / dt;
            ldt = lD * Vn - lA * (Vn - Vold) / (dt * dt);
        } else {
            adj::PatchX x;
            x.V = a.Vcur[q];
            x.Dold = a.Dprev[q]; x.Vold = Vold; x.thold = a.thprev[q];
            x.TLD = a.tld[q]; x.sig = a.sig[q]; x.dt = dt;
            x.a = a.pa[q]; x.b = a.pb[q]; x.Dc = a.pDc[q];
            x.F0 = a.F0[q]; x.la = a.la[q]; x.lth = a.lth0[q];
            x.K = a.kself[i]; x.M = a.mass[q]; x.Omega = a.omega[q]; x.eta = a.eta; x.tau0 = a.tau0[q];
            x.high = a.sw[q] == 1; x.dr = a.dr;
            double dtau = 0, dsn = 0, dsp = 0, sn = 0, ss = 0;
            const double tq = a.interp_at_told ? a.Tprev[r] : a.Tprev[r] + dt;
            if (a.n_ext > 0) {
                sim::interp_ext(a.n_ext, a.ext_t, a.ext_n, a.ext_s, a.ext_p, a.N, i, tq, dsn, dtau, dsp);
                interp_slope(a.n_ext, a.ext_t, a.ext_n, a.ext_s, a.N, i, tq, sn, ss);
            }
            x.dtau = dtau;
            double o[adj::kDirs - 1];
            if (adj::local_vjp(x, lV, lD, lth, lA, o)) {
                lDloc = o[adj::dDold - 1];
                lVold = o[adj::dVold - 1];
                lThold = o[adj::dThold - 1];
                lTLD = o[adj::dTLD - 1];
                // sigma = max(sigma_min, Kn D_old + sigma0 + dsn): no derivative where clamped
                lSig = x.sig > a.sigma_min ? o[adj::dSig - 1] : 0.0;
                ldt = o[adj::dDt - 1];
                ltx = o[adj::dDtau - 1] * ss + lSig * sn;
                a.ga[q] += o[adj::dA - 1];
                a.gb[q] += o[adj::dB - 1];
                a.gDc[q] += o[adj::dDc - 1];
            } else {
                atomicExch(a.err, 1);
            }
        }
        a.oDloc[q] = lDloc;
        a.oVold[q] = lVold;
        a.oThold[q] = lThold;
        a.oTLD[q] = lTLD;
        a.oSig[q] = lSig;
    }
    // per-block, per-instance sums of the dt and time adjoints (fixed order)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int rr = 0; rr < a.R; ++rr) {
        double u = (r == rr) ? ldt : 0.0, v = (r == rr) ? ltx : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            u += __shfl_xor_sync(0xffffffffu, u, o);
            v += __shfl_xor_sync(0xffffffffu, v, o);
        }
        if (lane == 0) { s_dt[rr][wid] = u; s_tx[rr][wid] = v; }
    }
    __syncthreads();
    if (threadIdx.x < a.R) {
        double u = 0, v = 0;
        for (int w = 0; w < kAdjThreads / 32; ++w) { u += s_dt[threadIdx.x][w]; v += s_tx[threadIdx.x][w]; }
        a.blk_dt[(int64_t)blockIdx.x * a.R + threadIdx.x] = u;
        a.blk_tx[(int64_t)blockIdx.x * a.R + threadIdx.x] = v;
    }
}

// sums of the per-block partials, in block order: out[r] = dt adjoint, out[R + r] = time adjoint
__global__ void k_adj_sum_blocks(int nblk, int R, const double* __restrict__ bdt, const double* __restrict__ btx,
                                 double* __restrict__ out) {
    const int r = threadIdx.x;
    if (r >= R) return;
    double u = 0, v = 0;
    for (int b = 0; b < nblk; ++b) { u += bdt[(int64_t)b * R + r]; v += btx[(int64_t)b * R + r]; }
    out[r] = u;
    out[R + r] = v;
}

// ---------------------------------------------------------------------------
// transposed products over the tile-contiguous operator
struct TF32 {
    static constexpr int kBytes = 4;
    __device__ static float get(const void* p, int64_t k) { return reinterpret_cast<const float*>(p)[k]; }
};
struct TBF16x2 {
    static constexpr int kBytes = 4;
    __device__ static float get(const void* p, int64_t k) {
        const uint32_t w = reinterpret_cast<const uint32_t*>(p)[k];
        return __uint_as_float(w & 0xFFFF0000u) + __uint_as_float(w << 16);
    }
};

__device__ __forceinline__ void two_sum(float& hi, float& lo, float p) {
    const float s = hi + p;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (p - bp);
    hi = s;
}

// one warp per (row block, column): partial[rb][side][r][j]
template <class F, int R>
__global__ void __launch_bounds__(kAdjThreads) k_adj_transpose_f32(AdjTransArgs a) {
    extern __shared__ float xs[];   // [2 sides][R][rpb]
    const int rb = blockIdx.y;
    const int64_t rpb = a.rpb, N = a.N;
    for (int64_t k = threadIdx.x; k < 2 * R * rpb; k += blockDim.x) {
        const int side = (int)(k / (R * rpb));
        const int r = (int)((k / rpb) % R);
        const int64_t i = rb * rpb + k % rpb;
        const double* src = side == 0 ? a.x_s : a.x_n;
        xs[k] = i < N ? (float)src[(int64_t)r * N + i] : 0.f;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    for (int64_t j = (int64_t)blockIdx.x * nw + wid; j < N; j += (int64_t)gridDim.x * nw) {
        const int64_t base = ((int64_t)rb * N + j) * rpb;
        for (int side = 0; side < 2; ++side) {
            const void* M = side == 0 ? a.E : a.Kn;
            float hi[R], lo[R];
#pragma unroll
            for (int r = 0; r < R; ++r) { hi[r] = 0.f; lo[r] = 0.f; }
            for (int64_t k = lane; k < rpb; k += 32) {
                const float m = F::get(M, base + k);
#pragma unroll
                for (int r = 0; r < R; ++r) hi[r] = fmaf(m, xs[(side * R + r) * rpb + k], hi[r]);
            }
            // warp tree in error-free pairs
#pragma unroll
            for (int r = 0; r < R; ++r)
                for (int o = 16; o > 0; o >>= 1) {
                    const float h2 = __shfl_xor_sync(0xffffffffu, hi[r], o);
                    const float l2 = __shfl_xor_sync(0xffffffffu, lo[r], o);
                    two_sum(hi[r], lo[r], h2);
                    lo[r] += l2;
                }
            if (lane == 0)
#pragma unroll
                for (int r = 0; r < R; ++r)
                    a.part[(((int64_t)rb * 2 + side) * R + r) * N + j] = (double)hi[r] + (double)lo[r];
        }
    }
}

template <int R>
__global__ void __launch_bounds__(kAdjThreads) k_adj_transpose_f64(AdjTransArgs a) {
    extern __shared__ double xd[];   // [2 sides][R][rpb]
    const int rb = blockIdx.y;
    const int64_t rpb = a.rpb, N = a.N;
    for (int64_t k = threadIdx.x; k < 2 * R * rpb; k += blockDim.x) {
        const int side = (int)(k / (R * rpb));
        const int r = (int)((k / rpb) % R);
        const int64_t i = rb * rpb + k % rpb;
        const double* src = side == 0 ? a.x_s : a.x_n;
        xd[k] = i < N ? src[(int64_t)r * N + i] : 0.0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    for (int64_t j = (int64_t)blockIdx.x * nw + wid; j < N; j += (int64_t)gridDim.x * nw) {
        const int64_t base = ((int64_t)rb * N + j) * rpb;
        for (int side = 0; side < 2; ++side) {
            const double* M = reinterpret_cast<const double*>(side == 0 ? a.E : a.Kn);
            double acc[R];
#pragma unroll
            for (int r = 0; r < R; ++r) acc[r] = 0.0;
            for (int64_t k = lane; k < rpb; k += 32) {
                const double m = M[base + k];
#pragma unroll
                for (int r = 0; r < R; ++r) acc[r] = fma(m, xd[(side * R + r) * rpb + k], acc[r]);
            }
#pragma unroll
            for (int r = 0; r < R; ++r)
                for (int o = 16; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
            if (lane == 0)
#pragma unroll
                for (int r = 0; r < R; ++r) a.part[(((int64_t)rb * 2 + side) * R + r) * N + j] = acc[r];
        }
    }
}

// lambda_D_old = local part - sum_rb E^T partials + sum_rb Kn^T partials (row-block order)
__global__ void k_adj_combine(int64_t N, int R, int64_t nrb, const double* __restrict__ part,
                              const double* __restrict__ dloc, double* __restrict__ out) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)R * N) return;
    const int r = (int)(q / N);
    const int64_t j = q - (int64_t)r * N;
    double se = 0, sk = 0;
    for (int64_t rb = 0; rb < nrb; ++rb) {
        se += part[((rb * 2 + 0) * R + r) * N + j];
        sk += part[((rb * 2 + 1) * R + r) * N + j];
    }
    out[q] = dloc[q] - se + sk;
}

// the controller's reductions of a state, one block per instance: out[r*5 ..]
// = {max V, V is NaN, min |V/A| (NaN and 0 left out), any usable, its patch}
__global__ void __launch_bounds__(kAdjThreads) k_adj_dtctl(int64_t N, int64_t Ns, const double* __restrict__ V,
                                                           const double* __restrict__ A,
                                                           const unsigned char* __restrict__ unstable,
                                                           const int* __restrict__ has_unstable,
                                                           double* __restrict__ out) {
    const int r = blockIdx.x;
    __shared__ double s_vmax[kAdjThreads], s_q[kAdjThreads];
    __shared__ long long s_k[kAdjThreads];
    __shared__ int s_nan[kAdjThreads];
    double vmax = -INFINITY, qmin = INFINITY;
    long long kmin = -1;
    int vnan = 0;
    for (int64_t i = threadIdx.x; i < N; i += blockDim.x) {
        const int64_t q = (int64_t)r * N + i;
        const bool ctl = has_unstable[r] ? (unstable[q] != 0) : (i < Ns);
        if (!ctl) continue;
        const double v = V[q];
        if (isnan(v)) vnan = 1;
        else vmax = fmax(vmax, v);
        const double qa = fabs(v / A[q]);
        if (!isnan(qa) && qa != 0 && qa < qmin) { qmin = qa; kmin = i; }
    }
    s_vmax[threadIdx.x] = vmax; s_q[threadIdx.x] = qmin; s_k[threadIdx.x] = kmin; s_nan[threadIdx.x] = vnan;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int t = 1; t < blockDim.x; ++t) {
            vmax = fmax(vmax, s_vmax[t]);
            vnan |= s_nan[t];
            if (s_q[t] < qmin || (s_q[t] == qmin && s_k[t] >= 0 && (kmin < 0 || s_k[t] < kmin))) {
                qmin = s_q[t];
                kmin = s_k[t];
            }
        }
        out[r * 5 + 0] = vmax;
        out[r * 5 + 1] = vnan;
        out[r * 5 + 2] = qmin;
        out[r * 5 + 3] = kmin >= 0 ? 1.0 : 0.0;
        out[r * 5 + 4] = (double)kmin;
    }
}

template <int R>
void launch_transpose_R(int prec, const AdjTransArgs& a, cudaStream_t st) {
    const dim3 grid((unsigned)std::max<int64_t>(1, std::min<int64_t>((a.N + 7) / 8, a.gx)), (unsigned)a.nrb);
    if (prec == QDFN_FP64) {
        const size_t sm = 2 * (size_t)R * a.rpb * sizeof(double);
        k_adj_transpose_f64<R><<<grid, kAdjThreads, sm, st>>>(a);
    } else if (prec == QDFN_FP32) {
        const size_t sm = 2 * (size_t)R * a.rpb * sizeof(float);
        k_adj_transpose_f32<TF32, R><<<grid, kAdjThreads, sm, st>>>(a);
    } else {
        const size_t sm = 2 * (size_t)R * a.rpb * sizeof(float);
        k_adj_transpose_f32<TBF16x2, R><<<grid, kAdjThreads, sm, st>>>(a);
    }
}

// sparse additions to the adjoint state: lV[idx[k]] += v[k], lD[idx[k]] += v[n+k], lA[idx[k]] += v[2n+k]
// (one thread, in order, so repeated indices add up deterministically)
__global__ void k_adj_add(int n, const int64_t* __restrict__ idx, const double* __restrict__ v, double* lV,
                          double* lD, double* lA) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int k = 0; k < n; ++k) {
        const int64_t q = idx[k];
        lV[q] += v[k];
        lD[q] += v[n + k];
        lA[q] += v[2 * n + k];
    }
}

}  // namespace

int adj_add(int n, const int64_t* idx, const double* vals, double* lV, double* lD, double* lA, cudaStream_t st) {
    if (n <= 0) return QDFN_OK;
    k_adj_add<<<1, 1, 0, st>>>(n, idx, vals, lV, lD, lA);
    QDFN_CUDA(cudaGetLastError());
    return QDFN_OK;
}

int adj_local(const AdjLocalArgs& a, cudaStream_t st) {
    const int64_t RN = (int64_t)a.R * a.N;
    const int nblk = (int)((RN + kAdjThreads - 1) / kAdjThreads);
    k_adj_local<<<nblk, kAdjThreads, 0, st>>>(a);
    QDFN_CUDA(cudaGetLastError());
    k_adj_sum_blocks<<<1, 32, 0, st>>>(nblk, a.R, a.blk_dt, a.blk_tx, a.sums);
    QDFN_CUDA(cudaGetLastError());
    return QDFN_OK;
}

int adj_local_blocks(int64_t RN) { return (int)((RN + kAdjThreads - 1) / kAdjThreads); }

int adj_transpose(int prec, int R, const AdjTransArgs& a, const double* dloc, double* out, cudaStream_t st) {
    switch (R) {
        case 1: launch_transpose_R<1>(prec, a, st); break;
        case 2: launch_transpose_R<2>(prec, a, st); break;
        default: launch_transpose_R<4>(prec, a, st); break;
    }
    QDFN_CUDA(cudaGetLastError());
    const int64_t RN = (int64_t)R * a.N;
    k_adj_combine<<<(unsigned)((RN + 255) / 256), 256, 0, st>>>(a.N, R, a.nrb, a.part, dloc, out);
    QDFN_CUDA(cudaGetLastError());
    return QDFN_OK;
}

int adj_transpose_prepare(int prec, int R, int64_t rpb) {
    const size_t sm = 2 * (size_t)R * rpb * (prec == QDFN_FP64 ? sizeof(double) : sizeof(float));
    if (sm > 48 * 1024) {
        cudaError_t e = cudaSuccess;
        auto set = [&](const void* f) {
            if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        };
        if (prec == QDFN_FP64) {
            set((const void*)k_adj_transpose_f64<1>); set((const void*)k_adj_transpose_f64<2>);
            set((const void*)k_adj_transpose_f64<4>);
        } else {
            set((const void*)k_adj_transpose_f32<TF32, 1>); set((const void*)k_adj_transpose_f32<TF32, 2>);
            set((const void*)k_adj_transpose_f32<TF32, 4>); set((const void*)k_adj_transpose_f32<TBF16x2, 1>);
            set((const void*)k_adj_transpose_f32<TBF16x2, 2>); set((const void*)k_adj_transpose_f32<TBF16x2, 4>);
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute (adjoint transpose)");
    }
    return QDFN_OK;
}

int adj_dtctl(int R, int64_t N, int64_t Ns, const double* V, const double* A, const unsigned char* unstable,
              const int* has_unstable, double* out, cudaStream_t st) {
    k_adj_dtctl<<<R, kAdjThreads, 0, st>>>(N, Ns, V, A, unstable, has_unstable, out);
    QDFN_CUDA(cudaGetLastError());
    return QDFN_OK;
}

}  // namespace qdfn
