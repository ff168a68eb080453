"""ctypes binding of the CPU FP64 oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/`` and
``__graft_entry__.smoke()``, which compare the GPU results with it, and by the
CPU-baseline leg of ``bench.py``, which times it; the shipped library never
imports it.

Parity status: the reference publishes no golden vectors and cannot run here
(it is Julia), so the oracle is pinned by physical known-answer tests -- strictly
"parity unpinned" against the reference's own outputs.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int64)


def build(quiet=True):
    """Compile liboracle.so with the Makefile beside this file."""
    out = subprocess.run(["make", "-s", "-j8", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.oracle_okada_dc3d.argtypes = [C.c_double] * 13 + [_dp, C.POINTER(C.c_int)]
        L.oracle_tdstress_hs.argtypes = [C.c_double] * 3 + [_dp] * 3 + [C.c_double] * 5 + [_dp, _dp]
        L.oracle_tdstress_hs.restype = C.c_int
        L.oracle_assemble_rect.argtypes = [C.c_int64] + [_dp] * 8 + [C.c_int64] + [_dp] * 6 + [C.c_double] * 2 + [_dp, _dp, C.c_int]
        L.oracle_assemble_tri.argtypes = [C.c_int64] + [_dp] * 4 + [C.c_int64] + [_dp] * 3 + [C.c_double] * 2 + [_dp, _dp, C.c_int]
        L.oracle_assemble_tri.restype = C.c_int
        L.oracle_op_dense.argtypes = [C.c_int64, _dp, _dp, C.c_int]
        L.oracle_op_dense.restype = C.c_void_p
        L.oracle_op_hmat.argtypes = [C.c_int64, C.c_int64, _ip, _ip, C.POINTER(_dp), C.POINTER(_dp), C.POINTER(_dp),
                                     _ip, C.POINTER(_dp), C.POINTER(_dp), C.POINTER(_dp), C.c_int]
        L.oracle_op_hmat.restype = C.c_void_p
        L.oracle_op_free.argtypes = [C.c_void_p]
        L.oracle_op_kself.argtypes = [C.c_void_p, _dp]
        L.oracle_op_apply.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.oracle_state_init.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64,
                                 _dp, _dp, _dp, _dp, _dp, _dp, _ip, C.c_int]
        L.oracle_run.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def okada_dc3d(alpha, x, y, z, depth, dip, al1, al2, aw1, aw2, d1, d2, d3):
    out = np.zeros(12)
    iret = C.c_int(0)
    lib().oracle_okada_dc3d(alpha, x, y, z, depth, dip, al1, al2, aw1, aw2, d1, d2, d3, _p(out), C.byref(iret))
    return out, iret.value


def tdstress_hs(x, y, z, P1, P2, P3, Ss, Ds, Ts, mu, lam):
    st = np.zeros(6)
    sn = np.zeros(6)
    P1, P2, P3 = _f64(P1), _f64(P2), _f64(P3)
    rc = lib().oracle_tdstress_hs(x, y, z, _p(P1), _p(P2), _p(P3), Ss, Ds, Ts, mu, lam, _p(st), _p(sn))
    if rc != 0:
        raise ValueError("Half-space solution: Z coordinates must be negative!")
    return st, sn


def assemble_rect(src, recv, G, nu, nthreads=None):
    """src/recv: dicts of 1-D arrays cx, cy, cz, ls, ld, strike, dip, rake.
    Returns (Ks, Kn) with shape (n_recv, n_src)."""
    nthreads = nthreads or os.cpu_count()
    s = {k: _f64(v) for k, v in src.items()}
    r = {k: _f64(v) for k, v in recv.items()}
    ns, nr = len(s["cx"]), len(r["cx"])
    Ks = np.zeros((nr, ns))
    Kn = np.zeros((nr, ns))
    lib().oracle_assemble_rect(ns, _p(s["cx"]), _p(s["cy"]), _p(s["cz"]), _p(s["ls"]), _p(s["ld"]),
                               _p(s["strike"]), _p(s["dip"]), _p(s["rake"]), nr, _p(r["cx"]), _p(r["cy"]),
                               _p(r["cz"]), _p(r["strike"]), _p(r["dip"]), _p(r["rake"]), G, nu, _p(Ks), _p(Kn),
                               nthreads)
    return Ks, Kn


def assemble_tri(P1, P2, P3, rake, centre, nhat, shat, G, nu, nthreads=None):
    nthreads = nthreads or os.cpu_count()
    P1, P2, P3, rake = _f64(P1), _f64(P2), _f64(P3), _f64(rake)
    centre, nhat, shat = _f64(centre), _f64(nhat), _f64(shat)
    ns, nr = P1.shape[0], centre.shape[0]
    Ks = np.zeros((nr, ns))
    Kn = np.zeros((nr, ns))
    rc = lib().oracle_assemble_tri(ns, _p(P1), _p(P2), _p(P3), _p(rake), nr, _p(centre), _p(nhat), _p(shat),
                                   G, nu, _p(Ks), _p(Kn), nthreads)
    if rc != 0:
        raise ValueError("Half-space solution: Z coordinates must be negative!")
    return Ks, Kn


class _Problem(C.Structure):
    _fields_ = [("N", C.c_int64), ("Nload", C.c_int64)] + \
               [(n, _dp) for n in ("a", "b", "Dc", "theta_i", "V_i", "f_i", "sigma0", "V_const", "mass")] + \
               [(n, C.c_double) for n in ("G", "rho", "sigma_min", "switch_v", "dt_cut", "rupture_dt", "max_dt",
                                          "alpha_evo")] + \
               [("evolution_dr", C.c_int), ("interp_at_told", C.c_int), ("n_ext", C.c_int64)] + \
               [(n, _dp) for n in ("ext_t", "ext_n", "ext_s", "ext_p")]


class _State(C.Structure):
    _fields_ = [("T", C.c_double), ("dt", C.c_double), ("step", C.c_int64)] + \
               [(n, _dp) for n in ("V", "D", "theta", "friction", "accel", "sigma_old")]


STATUS = {0: "ok", -10: "domain error (log/sqrt of a negative number)", -11: "minimum over an empty collection",
          -12: "retry cap exceeded", -13: "per-patch iteration cap exceeded"}


class Simulation:
    """Oracle cycle simulation.  ``problem`` is a dict with the per-patch arrays
    (a, b, Dc, theta_i, V_i, f_i, sigma0, V_const, mass) and the scalars
    (N, Nload, G, rho, sigma_min, switch_v, dt_cut, rupture_dt, max_dt,
    alpha_evo, evolution_dr, interp_at_told) and optional ext_* arrays.
    ``operator`` is ("dense", Ks, Kn) or ("hmat", blocks)."""

    def __init__(self, problem, operator, nthreads=None):
        L = lib()
        self.nthreads = nthreads or os.cpu_count()
        self.N = N = int(problem["N"])
        self._keep = {}
        pr = _Problem()
        pr.N, pr.Nload = N, int(problem["Nload"])
        for n in ("a", "b", "Dc", "theta_i", "V_i", "f_i", "sigma0", "V_const", "mass"):
            arr = _f64(problem[n])
            assert arr.shape == (N,), n
            self._keep[n] = arr
            setattr(pr, n, _p(arr))
        for n in ("G", "rho", "sigma_min", "switch_v", "dt_cut", "rupture_dt", "max_dt"):
            setattr(pr, n, float(problem[n]))
        pr.alpha_evo = float(problem.get("alpha_evo", 0.0))
        pr.evolution_dr = int(problem.get("evolution_dr", 1))
        pr.interp_at_told = int(problem.get("interp_at_told", 0))
        if problem.get("ext_t") is not None:
            for n in ("ext_t", "ext_n", "ext_s", "ext_p"):
                arr = _f64(problem[n])
                self._keep[n] = arr
                setattr(pr, n, _p(arr))
            pr.n_ext = len(self._keep["ext_t"])
        else:
            pr.n_ext = 0
        self._pr = pr
        kind = operator[0]
        self._owner = True
        if kind == "dense":
            Ks, Kn = _f64(operator[1]), _f64(operator[2])
            self._op = L.oracle_op_dense(N, _p(Ks), _p(Kn), self.nthreads)
        elif kind == "hmat":
            self._op = self._make_hmat(N, operator[1])
        elif kind == "shared":  # reuse another Simulation's operator (friction draws)
            self._op = operator[1]._op
            self._keep["shared"] = operator[1]
            self._owner = False
        else:
            raise ValueError(kind)
        self.state = {n: np.zeros(N) for n in ("V", "D", "theta", "friction", "accel", "sigma_old")}
        st = _State()
        for n, arr in self.state.items():
            setattr(st, n, _p(arr))
        self._st = st
        L.oracle_state_init(C.byref(pr), C.byref(st))

    def _make_hmat(self, N, blocks):
        L = lib()
        nb = len(blocks["range"])
        rng = np.ascontiguousarray(np.asarray(blocks["range"], dtype=np.int64).reshape(nb, 4))
        keep = [rng]

        def plist(arrs):
            ptrs = (_dp * nb)()
            for b, a in enumerate(arrs):
                if a is None:
                    ptrs[b] = _dp()
                else:
                    a = _f64(a)
                    keep.append(a)
                    ptrs[b] = _p(a)
            return ptrs

        def side(prefix):
            ranks = np.array([-1 if blocks[prefix + "D"][b] is not None else blocks[prefix + "U"][b].shape[1]
                              for b in range(nb)], dtype=np.int64)
            keep.append(ranks)
            U = plist(blocks[prefix + "U"])
            Vt = plist(blocks[prefix + "Vt"])
            D = plist(blocks[prefix + "D"])
            keep.extend([U, Vt, D])
            return ranks, U, Vt, D

        rs, Us, Vts, Ds = side("s")
        rn, Un, Vtn, Dn = side("n")
        self._keep["hmat"] = keep
        return L.oracle_op_hmat(N, nb, rng.ctypes.data_as(_ip), rs.ctypes.data_as(_ip), Us, Vts, Ds,
                                rn.ctypes.data_as(_ip), Un, Vtn, Dn, self.nthreads)

    def __del__(self):
        try:
            if self._owner:
                lib().oracle_op_free(self._op)
        except Exception:
            pass

    def set_scalars(self, T, dt, step):
        """Time, carried Dt and step count (state arrays are edited in place)."""
        self._st.T, self._st.dt, self._st.step = float(T), float(dt), int(step)

    @property
    def T(self):
        return self._st.T

    @property
    def dt(self):
        return self._st.dt

    @property
    def step(self):
        return self._st.step

    def kself(self):
        out = np.zeros(self.N)
        lib().oracle_op_kself(self._op, _p(out))
        return out

    def apply(self, D):
        D = _f64(D)
        tld, knd = np.zeros(self.N), np.zeros(self.N)
        lib().oracle_op_apply(self._op, _p(D), _p(tld), _p(knd))
        return tld, knd

    def run(self, nsteps, record_step=0, max_rec=0):
        N = self.N
        ht = np.zeros(max(max_rec, 1))
        hdt = np.zeros(max(max_rec, 1))
        hV = np.zeros((max(max_rec, 1), N))
        hD = np.zeros_like(hV)
        hth = np.zeros_like(hV)
        hs = np.zeros_like(hV)
        nrec = C.c_int64(0)
        rc = lib().oracle_run(C.byref(self._pr), self._op, C.byref(self._st), int(nsteps), int(record_step),
                              int(max_rec), _p(ht), _p(hdt), _p(hV), _p(hD), _p(hth), _p(hs), C.byref(nrec),
                              self.nthreads)
        if rc != 0:
            raise RuntimeError("oracle run failed: %s" % STATUS.get(rc, rc))
        n = nrec.value
        return dict(T=ht[:n], Dt=hdt[:n], V=hV[:n], D=hD[:n], theta=hth[:n], sigma=hs[:n])
