// Stiffness assembly on the GPU: one thread per (receiver, source) pair, FP64.
//
// Rectangles follow StiffnessMatrix_ByParts_Calculation_Rec
// (scripts/Functions_BuildInputFile.jl:386-512); triangles follow
// StiffnessMatrix_ByParts_Calculation_Tri (:551-594).  The reference's split
// into ~2000x2000 parts (:516-548, :599-638) bounds host memory only; every
// entry depends on its own pair, so the GPU forms the whole matrix (or any
// caller-chosen block of it) in one launch.
//
// Mapping: blockIdx.y walks sources, threads of a block take consecutive
// receivers, so column-major (Julia) output is written coalesced.  The work is
// FP64-pipe bound (no reuse to exploit: each pair evaluates 8 Okada corners or
// 3+3 angular dislocations and 3 free-surface pairs).
#include <cuda_runtime.h>

#include "qdfn_internal.h"
#include "assemble_kernels.h"

namespace qdfn {
namespace {

dim3 asm_grid(int64_t n_src, int64_t n_recv) {
    int64_t gx = (n_recv + kAsmThreads - 1) / kAsmThreads;
    int64_t gy = n_src < 65535 ? n_src : 65535;
    return dim3((unsigned)gx, (unsigned)(gy > 0 ? gy : 1), 1);
}

int check_common(int64_t n_src, int64_t n_recv, int64_t ld, int layout) {
    if (n_src < 0 || n_recv < 0) return fail(QDFN_ERR_INVALID, "negative patch count");
    if (layout != QDFN_LAYOUT_ROW && layout != QDFN_LAYOUT_COL)
        return fail(QDFN_ERR_INVALID, "layout must be QDFN_LAYOUT_ROW or QDFN_LAYOUT_COL");
    if (layout == QDFN_LAYOUT_COL && ld < n_recv) return fail(QDFN_ERR_INVALID, "ld < n_recv");
    if (layout == QDFN_LAYOUT_ROW && ld < n_src) return fail(QDFN_ERR_INVALID, "ld < n_src");
    if ((n_recv + kAsmThreads - 1) / kAsmThreads > 2147483647LL)
        return fail(QDFN_ERR_INVALID, "too many receivers");
    return QDFN_OK;
}

// RAII device buffer
struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, n ? n : 1); }
};

}  // namespace
}  // namespace qdfn

using namespace qdfn;

extern "C" int qdfn_assemble_rect_dev(int64_t n_src, const double* src, int64_t n_recv,
                                      const double* recv, double G, double nu, double* Ks,
                                      double* Kn, int64_t ld, int layout, void* stream) {
    int rc = check_common(n_src, n_recv, ld, layout);
    if (rc) return rc;
    if (n_src == 0 || n_recv == 0) return QDFN_OK;
    if (!src || !recv || !Ks || !Kn) return fail(QDFN_ERR_INVALID, "null pointer");
    launch_assemble_rect(asm_grid(n_src, n_recv), (cudaStream_t)stream, n_src, src, n_recv, recv,
                         G, nu, Ks, Kn, ld, layout);
    QDFN_CUDA(cudaGetLastError());
    return QDFN_OK;
}

extern "C" int qdfn_assemble_rect(int64_t n_src, const double* src, int64_t n_recv,
                                  const double* recv, double G, double nu, double* Ks, double* Kn,
                                  int layout) {
    const int64_t ld = layout == QDFN_LAYOUT_COL ? n_recv : n_src;
    int rc = check_common(n_src, n_recv, ld, layout);
    if (rc) return rc;
    if (n_src == 0 || n_recv == 0) return QDFN_OK;
    if (!src || !recv || !Ks || !Kn) return fail(QDFN_ERR_INVALID, "null pointer");
    DevBuf dsrc, drecv, dks, dkn;
    const size_t nk = (size_t)n_src * n_recv * sizeof(double);
    if (dsrc.alloc(n_src * 8 * sizeof(double)) || drecv.alloc(n_recv * 8 * sizeof(double)) ||
        dks.alloc(nk) || dkn.alloc(nk))
        return fail(QDFN_ERR_NOMEM, "device allocation failed in qdfn_assemble_rect");
    QDFN_CUDA(cudaMemcpy(dsrc.p, src, n_src * 8 * sizeof(double), cudaMemcpyHostToDevice));
    QDFN_CUDA(cudaMemcpy(drecv.p, recv, n_recv * 8 * sizeof(double), cudaMemcpyHostToDevice));
    rc = qdfn_assemble_rect_dev(n_src, (const double*)dsrc.p, n_recv, (const double*)drecv.p, G,
                                nu, (double*)dks.p, (double*)dkn.p, ld, layout, nullptr);
    if (rc) return rc;
    QDFN_CUDA(cudaMemcpy(Ks, dks.p, nk, cudaMemcpyDeviceToHost));
    QDFN_CUDA(cudaMemcpy(Kn, dkn.p, nk, cudaMemcpyDeviceToHost));
    return QDFN_OK;
}

extern "C" int qdfn_assemble_tri_dev(int64_t n_src, const double* P1, const double* P2,
                                     const double* P3, const double* rake, int64_t n_recv,
                                     const double* centre, const double* nhat, const double* shat,
                                     double G, double nu, double* Ks, double* Kn, int64_t ld,
                                     int layout, void* stream) {
    int rc = check_common(n_src, n_recv, ld, layout);
    if (rc) return rc;
    if (n_src == 0 || n_recv == 0) return QDFN_OK;
    if (!P1 || !P2 || !P3 || !rake || !centre || !nhat || !shat || !Ks || !Kn)
        return fail(QDFN_ERR_INVALID, "null pointer");
    launch_assemble_tri(asm_grid(n_src, n_recv), (cudaStream_t)stream, n_src, P1, P2, P3, rake,
                        n_recv, centre, nhat, shat, G, nu, Ks, Kn, ld, layout);
    QDFN_CUDA(cudaGetLastError());
    return QDFN_OK;
}

extern "C" int qdfn_assemble_tri_pairs_dev(int64_t npairs, const int64_t* recv_idx, const int64_t* src_idx,
                                           const double* P1, const double* P2, const double* P3,
                                           const double* rake, const double* centre, const double* nhat,
                                           const double* shat, double G, double nu, double* Ks, double* Kn,
                                           void* stream) {
    if (npairs < 0) return fail(QDFN_ERR_INVALID, "npairs < 0");
    if (npairs == 0) return QDFN_OK;
    if ((npairs + kAsmThreads - 1) / kAsmThreads > 2147483647LL) return fail(QDFN_ERR_INVALID, "too many pairs");
    if (!recv_idx || !src_idx || !P1 || !P2 || !P3 || !rake || !centre || !nhat || !shat || !Ks || !Kn)
        return fail(QDFN_ERR_INVALID, "null pointer");
    launch_assemble_tri_pairs((cudaStream_t)stream, npairs, recv_idx, src_idx, P1, P2, P3, rake, centre, nhat, shat,
                              G, nu, Ks, Kn);
    QDFN_CUDA(cudaGetLastError());
    return QDFN_OK;
}

extern "C" int qdfn_assemble_tri(int64_t n_src, const double* P1, const double* P2,
                                 const double* P3, const double* rake, int64_t n_recv,
                                 const double* centre, const double* nhat, const double* shat,
                                 double G, double nu, double* Ks, double* Kn, int layout) {
    const int64_t ld = layout == QDFN_LAYOUT_COL ? n_recv : n_src;
    int rc = check_common(n_src, n_recv, ld, layout);
    if (rc) return rc;
    if (n_src == 0 || n_recv == 0) return QDFN_OK;
    if (!P1 || !P2 || !P3 || !rake || !centre || !nhat || !shat || !Ks || !Kn)
        return fail(QDFN_ERR_INVALID, "null pointer");
    // TDstressHS raises when any receiver or vertex lies above z = 0 (:99-101)
    for (int64_t r = 0; r < n_recv; ++r)
        if (centre[r * 3 + 2] > 0) return fail(QDFN_ERR_HALF_SPACE, "receiver above the free surface");
    for (int64_t s = 0; s < n_src; ++s)
        if (P1[s * 3 + 2] > 0 || P2[s * 3 + 2] > 0 || P3[s * 3 + 2] > 0)
            return fail(QDFN_ERR_HALF_SPACE, "triangle vertex above the free surface");
    DevBuf d1, d2, d3, drk, dc, dn, dsv, dks, dkn;
    const size_t v3s = (size_t)n_src * 3 * sizeof(double), v3r = (size_t)n_recv * 3 * sizeof(double);
    const size_t nk = (size_t)n_src * n_recv * sizeof(double);
    if (d1.alloc(v3s) || d2.alloc(v3s) || d3.alloc(v3s) || drk.alloc(n_src * sizeof(double)) ||
        dc.alloc(v3r) || dn.alloc(v3r) || dsv.alloc(v3r) || dks.alloc(nk) || dkn.alloc(nk))
        return fail(QDFN_ERR_NOMEM, "device allocation failed in qdfn_assemble_tri");
    QDFN_CUDA(cudaMemcpy(d1.p, P1, v3s, cudaMemcpyHostToDevice));
    QDFN_CUDA(cudaMemcpy(d2.p, P2, v3s, cudaMemcpyHostToDevice));
    QDFN_CUDA(cudaMemcpy(d3.p, P3, v3s, cudaMemcpyHostToDevice));
    QDFN_CUDA(cudaMemcpy(drk.p, rake, n_src * sizeof(double), cudaMemcpyHostToDevice));
    QDFN_CUDA(cudaMemcpy(dc.p, centre, v3r, cudaMemcpyHostToDevice));
    QDFN_CUDA(cudaMemcpy(dn.p, nhat, v3r, cudaMemcpyHostToDevice));
    QDFN_CUDA(cudaMemcpy(dsv.p, shat, v3r, cudaMemcpyHostToDevice));
    rc = qdfn_assemble_tri_dev(n_src, (const double*)d1.p, (const double*)d2.p,
                               (const double*)d3.p, (const double*)drk.p, n_recv,
                               (const double*)dc.p, (const double*)dn.p, (const double*)dsv.p, G,
                               nu, (double*)dks.p, (double*)dkn.p, ld, layout, nullptr);
    if (rc) return rc;
    QDFN_CUDA(cudaMemcpy(Ks, dks.p, nk, cudaMemcpyDeviceToHost));
    QDFN_CUDA(cudaMemcpy(Kn, dkn.p, nk, cudaMemcpyDeviceToHost));
    return QDFN_OK;
}
