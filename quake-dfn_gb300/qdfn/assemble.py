"""Stiffness assembly through the C ABI (GPU, FP64).

``build_matrix_rect`` / ``build_matrix_tri`` stand in for the reference's
BuildMatrixByParts_Even_Rec / _Tri (scripts/Functions_BuildInputFile.jl:516,
:599): the same K[receiver, source] shear and normal matrices, formed in one
device pass instead of ~2000x2000 host parts.
"""
import numpy as np

from . import _lib
from .geometry import rect_records


def assemble_rect(src, recv, shear_modulus, poisson, layout="row"):
    """src/recv: n x 8 records (see geometry.rect_records).  Returns (Ks, Kn)
    of shape (n_recv, n_src) in C order (layout="row") or as Fortran-ordered
    arrays with the same shape (layout="col", Julia's memory order)."""
    L = _lib.load()
    src = np.ascontiguousarray(src, dtype=np.float64)
    recv = np.ascontiguousarray(recv, dtype=np.float64)
    ns, nr = src.shape[0], recv.shape[0]
    lay = _lib.LAYOUT_COL if layout == "col" else _lib.LAYOUT_ROW
    if lay == _lib.LAYOUT_COL:
        Ks = np.zeros((ns, nr))
        Kn = np.zeros((ns, nr))
    else:
        Ks = np.zeros((nr, ns))
        Kn = np.zeros((nr, ns))
    _lib.check(L.qdfn_assemble_rect(ns, _lib.dp(src), nr, _lib.dp(recv), float(shear_modulus), float(poisson),
                                    _lib.dp(Ks), _lib.dp(Kn), lay))
    if lay == _lib.LAYOUT_COL:
        return Ks.T, Kn.T
    return Ks, Kn


def assemble_tri(P1, P2, P3, rake, centre, nhat, shat, shear_modulus, poisson, layout="row"):
    L = _lib.load()
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    P1, P2, P3, rake, centre, nhat, shat = map(f, (P1, P2, P3, rake, centre, nhat, shat))
    ns, nr = P1.shape[0], centre.shape[0]
    lay = _lib.LAYOUT_COL if layout == "col" else _lib.LAYOUT_ROW
    shape = (ns, nr) if lay == _lib.LAYOUT_COL else (nr, ns)
    Ks, Kn = np.zeros(shape), np.zeros(shape)
    _lib.check(L.qdfn_assemble_tri(ns, _lib.dp(P1), _lib.dp(P2), _lib.dp(P3), _lib.dp(rake), nr, _lib.dp(centre),
                                   _lib.dp(nhat), _lib.dp(shat), float(shear_modulus), float(poisson), _lib.dp(Ks),
                                   _lib.dp(Kn), lay))
    if lay == _lib.LAYOUT_COL:
        return Ks.T, Kn.T
    return Ks, Kn


def build_matrix_rect(seg_dict, shear_modulus, poisson):
    """BuildMatrixByParts_Even_Rec equivalent on a read_segment_input dict."""
    rec = rect_records(seg_dict)
    return assemble_rect(rec, rec, shear_modulus, poisson)


def build_matrix_tri(P1, P2, P3, rake, centre, nhat, shat, shear_modulus, poisson):
    """BuildMatrixByParts_Even_Tri equivalent (vertices already reordered by
    rot_verts_unit_vectors)."""
    return assemble_tri(P1, P2, P3, rake, centre, nhat, shat, shear_modulus, poisson)


def assemble_rect_dev(src, recv, shear_modulus, poisson, Ks, Kn, stream=0, layout="col"):
    """Device-pointer form on torch tensors: src/recv (n x 8, float64, cuda),
    Ks/Kn preallocated float64 cuda tensors.  layout="col" expects Ks of shape
    (n_src, n_recv) contiguous (entry (r, s) at s*n_recv + r)."""
    L = _lib.load()
    lay = _lib.LAYOUT_COL if layout == "col" else _lib.LAYOUT_ROW
    ld = Ks.stride(0)
    _lib.check(L.qdfn_assemble_rect_dev(src.shape[0], src.data_ptr(), recv.shape[0], recv.data_ptr(),
                                        float(shear_modulus), float(poisson), Ks.data_ptr(), Kn.data_ptr(), ld, lay,
                                        stream))


def assemble_tri_dev(P1, P2, P3, rake, centre, nhat, shat, shear_modulus, poisson, Ks, Kn, stream=0, layout="col"):
    """Device-pointer form of assemble_tri on torch tensors: P1/P2/P3
    (n_src x 3), rake (n_src), centre/nhat/shat (n_recv x 3), all contiguous
    float64 CUDA tensors (slices of larger ones included); Ks/Kn preallocated,
    layout="col": shape (n_src, n_recv), entry (r, s) at s*ld + r."""
    L = _lib.load()
    lay = _lib.LAYOUT_COL if layout == "col" else _lib.LAYOUT_ROW
    for t in (P1, P2, P3, rake, centre, nhat, shat):
        if not t.is_contiguous():
            raise ValueError("assemble_tri_dev needs contiguous tensors")
    _lib.check(L.qdfn_assemble_tri_dev(P1.shape[0], P1.data_ptr(), P2.data_ptr(), P3.data_ptr(), rake.data_ptr(),
                                       centre.shape[0], centre.data_ptr(), nhat.data_ptr(), shat.data_ptr(),
                                       float(shear_modulus), float(poisson), Ks.data_ptr(), Kn.data_ptr(),
                                       Ks.stride(0), lay, stream))


def assemble_tri_pairs_dev(ridx, sidx, P1, P2, P3, rake, centre, nhat, shat, shear_modulus, poisson, stream=0):
    """Gathered triangle stiffness entries (qdfn_assemble_tri_pairs_dev): ridx,
    sidx int64 CUDA tensors of receiver and source indices into the per-triangle
    float64 CUDA tensors; returns (Ks, Kn) CUDA tensors of the pairs."""
    import torch
    L = _lib.load()
    n = int(ridx.shape[0])
    Ks = torch.empty(n, dtype=torch.float64, device=ridx.device)
    Kn = torch.empty(n, dtype=torch.float64, device=ridx.device)
    for t in (ridx, sidx, P1, P2, P3, rake, centre, nhat, shat):
        if not t.is_contiguous():
            raise ValueError("assemble_tri_pairs_dev needs contiguous tensors")
    _lib.check(L.qdfn_assemble_tri_pairs_dev(n, ridx.data_ptr(), sidx.data_ptr(), P1.data_ptr(), P2.data_ptr(),
                                             P3.data_ptr(), rake.data_ptr(), centre.data_ptr(), nhat.data_ptr(),
                                             shat.data_ptr(), float(shear_modulus), float(poisson), Ks.data_ptr(),
                                             Kn.data_ptr(), stream))
    return Ks, Kn
