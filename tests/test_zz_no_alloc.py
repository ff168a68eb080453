"""The allocation-free operator entry point (qdfn_apply_dense_noalloc).

Some callers cannot call cudaMalloc -- their device memory belongs to another
allocator (a Julia CUDA.jl pool, a framework's caching allocator) or they run
loops where allocation is not allowed.  qdfn_apply_dense_noalloc computes the
same shear and normal products as the context-based operator, keeping its
scratch in a fixed-size device array instead of allocating.  Checked here
against the FP64 oracle's operator (ElasticLoadingShearMatrix = K_ij/K_ii with
a zero diagonal times (0 - D), and Kn D), on two calls in a row, at odd and
chunk-boundary sizes, with a padded leading dimension, and at the 16,384-patch
limit.  This file is collected last so that a run stopping at the first
failure has already run everything else; it passes alone or after the other
tests.
"""
import ctypes as C

import numpy as np
import pytest

from _systems import mixed_rects

pytestmark = pytest.mark.gpu
G, NU = 32e9, 0.25


def _lib_noalloc():
    from qdfn import _lib
    L = _lib.load()
    L.qdfn_apply_dense_noalloc.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    return _lib, L


def _oracle_apply(oracle_mod, Ks, Kn, D):
    """The oracle's dense operator on K[recv, src] (forms ELSM itself)."""
    N = Ks.shape[0]
    one = np.ones(N)
    prob = dict(N=N, Nload=0, a=one * 0.01, b=one * 0.015, Dc=one * 1e-3, theta_i=one * 1e6, V_i=one * 1e-9,
                f_i=one * 0.6, sigma0=one * 1e7, V_const=one * 0.0, mass=one * 1e6, G=G, rho=2670.0, sigma_min=1e6,
                switch_v=1e-2, dt_cut=5.0, rupture_dt=0.1, max_dt=1e7)
    return oracle_mod.Simulation(prob, ("dense", Ks, Kn), nthreads=None).apply(D)


def _check(oracle_mod, Ks, Kn, ld, ncalls=2, seed=7):
    """Two (or more) calls in a row through the C ABI, each against the oracle;
    the device matrices are source-major with leading dimension ld >= N."""
    import torch
    _lib, L = _lib_noalloc()
    N = Ks.shape[0]
    Ks_d = torch.zeros((N, ld), dtype=torch.float64, device="cuda")
    Kn_d = torch.zeros((N, ld), dtype=torch.float64, device="cuda")
    Ks_d[:, :N] = torch.from_numpy(np.ascontiguousarray(Ks.T))   # row s holds column s of K[recv, src]
    Kn_d[:, :N] = torch.from_numpy(np.ascontiguousarray(Kn.T))
    if ld > N:   # padding that must never be read
        Ks_d[:, N:] = float("nan")
        Kn_d[:, N:] = float("nan")
    rng = np.random.default_rng(seed)
    for call in range(ncalls):
        D = rng.uniform(-1.0, 2.0, N)
        D_d = torch.tensor(D, dtype=torch.float64, device="cuda")
        tld_d = torch.full((N,), np.nan, dtype=torch.float64, device="cuda")
        knd_d = torch.full((N,), np.nan, dtype=torch.float64, device="cuda")
        _lib.check(L.qdfn_apply_dense_noalloc(N, Ks_d.data_ptr(), Kn_d.data_ptr(), ld, D_d.data_ptr(),
                                              tld_d.data_ptr(), knd_d.data_ptr(), None))
        torch.cuda.synchronize()
        tld_ref, knd_ref = _oracle_apply(oracle_mod, Ks, Kn, D)
        tld, knd = tld_d.cpu().numpy(), knd_d.cpu().numpy()
        assert np.max(np.abs(tld - tld_ref)) <= 1e-12 * np.max(np.abs(tld_ref)), (N, ld, call)
        assert np.max(np.abs(knd - knd_ref)) <= 1e-12 * np.max(np.abs(knd_ref)), (N, ld, call)


def test_noalloc_operator_matches_the_oracle_twice(qdfn_mod, oracle_mod):
    from qdfn import assemble
    rec = mixed_rects()
    Ks, Kn = assemble.assemble_rect(rec, rec, G, NU)
    _check(oracle_mod, Ks, Kn, rec.shape[0])


@pytest.mark.parametrize("N,pad", [(1, 0), (9, 3), (513, 0), (513, 3), (1000, 5)])
def test_noalloc_odd_sizes_and_padded_leading_dimension(qdfn_mod, oracle_mod, N, pad):
    """Sizes below, at and between the column-chunk boundaries (8 chunks; one
    patch leaves seven empty), and ld = N + pad."""
    rng = np.random.default_rng(N + pad)
    Ks = rng.normal(size=(N, N)) * 1e6
    Ks[np.diag_indices(N)] = -rng.uniform(1e9, 2e9, N)    # K_ii < 0 as for real patches
    Kn = rng.normal(size=(N, N)) * 1e6
    _check(oracle_mod, Ks, Kn, N + pad)


def test_noalloc_at_its_limit(qdfn_mod, oracle_mod):
    """N = 16,384, the largest size the fixed scratch array holds."""
    N = 16384
    rng = np.random.default_rng(3)
    Ks = rng.normal(size=(N, N)) * 1e6
    Ks[np.diag_indices(N)] = -rng.uniform(1e9, 2e9, N)
    Kn = rng.normal(size=(N, N)) * 1e6
    _check(oracle_mod, Ks, Kn, N)


def test_noalloc_rejects_sizes_beyond_its_limit(qdfn_mod):
    _lib, L = _lib_noalloc()
    dummy = C.c_void_p(16)
    rc = L.qdfn_apply_dense_noalloc(16385, dummy, dummy, 16385, dummy, dummy, dummy, C.c_void_p(0))
    assert rc == -1
    assert "exceeds the allocation-free limit of 16384" in _lib.last_error()
