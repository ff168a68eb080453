// Launchers of the assembly kernels (one translation unit each, so the two
// large FP64 kernels compile in parallel).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace qdfn {
constexpr int kAsmThreads = 128;
void launch_assemble_rect(dim3 grid, cudaStream_t st, int64_t n_src, const double* src,
                          int64_t n_recv, const double* recv, double G, double nu, double* Ks,
                          double* Kn, int64_t ld, int layout);
void launch_assemble_tri(dim3 grid, cudaStream_t st, int64_t n_src, const double* P1,
                         const double* P2, const double* P3, const double* rake, int64_t n_recv,
                         const double* centre, const double* nhat, const double* shat, double G,
                         double nu, double* Ks, double* Kn, int64_t ld, int layout);
void launch_assemble_tri_pairs(cudaStream_t st, int64_t npairs, const int64_t* ridx, const int64_t* sidx,
                               const double* P1, const double* P2, const double* P3, const double* rake,
                               const double* centre, const double* nhat, const double* shat, double G, double nu,
                               double* Ks, double* Kn);
}  // namespace qdfn
