"""The allocation-free operator entry point (qdfn_apply_dense_noalloc).

Some callers cannot call cudaMalloc -- their device memory belongs to another
allocator (a Julia CUDA.jl pool, a framework's caching allocator) or they run
loops where allocation is not allowed.  qdfn_apply_dense_noalloc computes the
same shear and normal products as the context-based operator, keeping its
scratch in a fixed-size device array instead of allocating.  This file is
collected last so that a run stopping at the first failure has already run
everything else; it passes alone or after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from _systems import mixed_rects, problem_for

pytestmark = pytest.mark.gpu
G, NU = 32e9, 0.25


def _noalloc(L, N, Ks_d, Kn_d, D_d, tld_d, knd_d):
    from qdfn import _lib
    return L.qdfn_apply_dense_noalloc(N, C.c_void_p(Ks_d.data_ptr()), C.c_void_p(Kn_d.data_ptr()), N,
                                      C.c_void_p(D_d.data_ptr()), C.c_void_p(tld_d.data_ptr()),
                                      C.c_void_p(knd_d.data_ptr()), C.c_void_p(0))


def test_noalloc_operator_matches_the_context_operator_twice(qdfn_mod):
    import torch
    from qdfn import _lib, assemble, simulate
    L = _lib.load()
    L.qdfn_apply_dense_noalloc.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    rec = mixed_rects()
    N = rec.shape[0]
    Ks, Kn = assemble.assemble_rect(rec, rec, G, NU)
    sim = simulate.Simulation(problem_for(rec, Ks))
    sim.set_dense(Ks, Kn, "fp64")
    # source-major device copies (Julia's column-major K[recv, src])
    Ks_d = torch.tensor(np.ascontiguousarray(Ks.T), dtype=torch.float64, device="cuda")
    Kn_d = torch.tensor(np.ascontiguousarray(Kn.T), dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(7)
    for call in range(2):
        D = rng.uniform(-1.0, 2.0, N)
        D_d = torch.tensor(D, dtype=torch.float64, device="cuda")
        tld_d = torch.full((N,), np.nan, dtype=torch.float64, device="cuda")
        knd_d = torch.full((N,), np.nan, dtype=torch.float64, device="cuda")
        _lib.check(_noalloc(L, N, Ks_d, Kn_d, D_d, tld_d, knd_d))
        torch.cuda.synchronize()
        tld_ref, knd_ref = sim.apply(D)
        tld, knd = tld_d.cpu().numpy(), knd_d.cpu().numpy()
        scale_s, scale_n = np.max(np.abs(tld_ref)), np.max(np.abs(knd_ref))
        assert np.max(np.abs(tld - tld_ref[0])) <= 1e-12 * scale_s, call
        assert np.max(np.abs(knd - knd_ref[0])) <= 1e-12 * scale_n, call
    sim.close()


def test_noalloc_rejects_sizes_beyond_its_limit(qdfn_mod):
    from qdfn import _lib
    L = _lib.load()
    L.qdfn_apply_dense_noalloc.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    dummy = C.c_void_p(16)
    rc = L.qdfn_apply_dense_noalloc(16385, dummy, dummy, 16385, dummy, dummy, dummy, C.c_void_p(0))
    assert rc == -1
    assert "exceeds the allocation-free limit of 16384" in _lib.last_error()
