"""The C-ABI library loads and exports every symbol include/qdfn.h declares
(no compute call: these run without a GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "qdfn.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qdfn_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_binding_list(qdfn_mod):
    from qdfn import _lib
    assert declared_symbols() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(qdfn_mod):
    from qdfn import _lib
    L = ctypes.CDLL(_lib.lib_path())
    for name in declared_symbols():
        assert hasattr(L, name), name


def test_version_and_status_strings(qdfn_mod):
    from qdfn import _lib
    L = _lib.load()
    assert b"sm_103a" in L.qdfn_version()
    assert L.qdfn_status_string(-14) == b"device deadline passed"
    assert L.qdfn_status_string(0) == b"ok"


def test_invalid_arguments_are_rejected_on_the_host(qdfn_mod):
    import numpy as np
    from qdfn import _lib
    L = _lib.load()
    rec = np.zeros((1, 8))
    K = np.zeros(1)
    rc = L.qdfn_assemble_rect(-1, _lib.dp(rec), 1, _lib.dp(rec), 1.0, 0.25, _lib.dp(K), _lib.dp(K), 0)
    assert rc == -1
    assert "negative" in _lib.last_error()
    rc = L.qdfn_assemble_rect(1, _lib.dp(rec), 1, _lib.dp(rec), 1.0, 0.25, _lib.dp(K), _lib.dp(K), 7)
    assert rc == -1
    # a receiver above the free surface is refused before any device work
    P = np.array([[0.0, 0.0, -1.0]])
    c = np.array([[0.0, 0.0, 5.0]])
    rc = L.qdfn_assemble_tri(1, _lib.dp(P), _lib.dp(P), _lib.dp(P), _lib.dp(np.zeros(1)), 1, _lib.dp(c),
                             _lib.dp(c), _lib.dp(c), 1.0, 0.25, _lib.dp(K), _lib.dp(K), 0)
    assert rc == -15


def test_new_entry_points_reject_bad_arguments_on_the_host(qdfn_mod):
    """The H-structure, ensemble-state and early-column calls check their
    arguments before any device work (no GPU needed)."""
    import ctypes as C
    import numpy as np
    from qdfn import _lib
    L = _lib.load()
    h = C.c_void_p()
    c = np.zeros((4, 3))
    assert L.qdfn_hstruct_build(None, 4, C.c_void_p(c.ctypes.data), 8, 2.0) == -1
    assert L.qdfn_hstruct_build(C.byref(h), 0, C.c_void_p(c.ctypes.data), 8, 2.0) == -1
    assert L.qdfn_hstruct_build(C.byref(h), 4, C.c_void_p(c.ctypes.data), 0, 2.0) == -1
    assert "leaf" in _lib.last_error()
    assert L.qdfn_hstruct_build(C.byref(h), 4, C.c_void_p(c.ctypes.data), 8, -1.0) == -1
    assert L.qdfn_hstruct_build(C.byref(h), 4, C.c_void_p(c.ctypes.data), 8, float("nan")) == -1
    bad = c.copy()
    bad[2, 1] = np.inf
    assert L.qdfn_hstruct_build(C.byref(h), 4, C.c_void_p(bad.ctypes.data), 8, 2.0) == -1
    assert "finite" in _lib.last_error()
    assert L.qdfn_hstruct_build(C.byref(h), 1 << 30, C.c_void_p(c.ctypes.data), 1, 2.0) == -1
    assert "tree nodes" in _lib.last_error()
    assert L.qdfn_hstruct_sizes(None, None, None) == -1
    assert L.qdfn_hstruct_get(None, None, None, None) == -1
    assert L.qdfn_hstruct_destroy(None) == 0
    n = C.c_int64()
    assert L.qdfn_ensemble_state_bytes(None, C.byref(n)) == -1
    assert L.qdfn_ensemble_set_state_all(None, C.c_void_p(c.ctypes.data), None) == -1
    assert L.qdfn_ensemble_get_state_all(None, C.c_void_p(c.ctypes.data), None, 1) == -1
    assert L.qdfn_set_early_cols(None, 4) == -1
    assert L.qdfn_get_early_cols(None) == -1


def test_context_rejects_bad_problems(qdfn_mod):
    import ctypes as C
    import numpy as np
    from qdfn import _lib
    L = _lib.load()
    pr = _lib.Problem()
    pr.N = 0
    h = C.c_void_p()
    assert L.qdfn_ctx_create(C.byref(h), C.byref(pr)) == -1
    pr.N = 4
    pr.n_inst = 9
    assert L.qdfn_ctx_create(C.byref(h), C.byref(pr)) == -1
