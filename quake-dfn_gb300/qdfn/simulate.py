"""Cycle simulation through the C ABI, with the reference's entry points.

``main`` and ``main_H`` keep the positional signatures of
scripts/Functions_RSFDFN3DMain_D.jl:2-8 and scripts/Functions_RSFDFN3DMain_H.jl:2-8
and write the same history keys (History_V, History_Disp, History_Time,
History_Theta, History_NormalStress; Main_D :287-289), to ``.npz`` because
JLD2/HDF5 is not available on this side of the boundary.  ``Simulation`` is the
object API underneath (one qdfn context).
"""
import ctypes as C
import os

import numpy as np

from . import _lib


def _f64(a, n=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel())
    if n is not None and a.shape[0] != n:
        raise ValueError("expected %d values, got %d" % (n, a.shape[0]))
    return a


def _addr(buf):
    """Address of a host buffer: numpy array or an object with data_ptr()."""
    if buf is None:
        return None
    if hasattr(buf, "data_ptr"):
        return C.c_void_p(buf.data_ptr())
    if not (buf.flags.c_contiguous and buf.flags.writeable):
        raise ValueError("host buffers must be C-contiguous and writeable")
    return C.c_void_p(buf.ctypes.data)


class Simulation:
    """One qdfn context: ``n_inst`` instances (friction draws) sharing an operator.

    problem: dict with N, Nload, per-patch arrays a, b, Dc, theta_i, V_i, f_i,
    sigma0, V_const, mass (length N, or n_inst*N instance-major) and scalars G,
    rho, sigma_min, switch_v, dt_cut, rupture_dt, max_dt, alpha_evo,
    evolution_dr, interp_at_told.
    """

    PER_PATCH = ("a", "b", "Dc", "theta_i", "V_i", "f_i", "sigma0", "V_const", "mass")

    def __init__(self, problem, n_inst=1, record_step=0, max_records=0):
        self.L = _lib.load()
        self.N = N = int(problem["N"])
        self.n_inst = int(n_inst)
        self._keep = {}
        pr = _lib.Problem()
        pr.N, pr.Nload = N, int(problem["Nload"])
        pr.n_inst = self.n_inst
        pr.evolution_dr = int(problem.get("evolution_dr", 1))
        for n in self.PER_PATCH:
            a = _f64(problem[n])
            if a.shape[0] == N and self.n_inst > 1:
                a = np.tile(a, self.n_inst)
            if a.shape[0] != N * self.n_inst:
                raise ValueError("%s: expected %d values" % (n, N * self.n_inst))
            self._keep[n] = a
            setattr(pr, n, _lib.dp(a))
        for n in ("G", "rho", "sigma_min", "switch_v", "dt_cut", "rupture_dt", "max_dt"):
            setattr(pr, n, float(problem[n]))
        pr.alpha_evo = float(problem.get("alpha_evo", 0.0))
        pr.interp_at_told = int(problem.get("interp_at_told", 0))
        pr.record_step = int(record_step)
        pr.max_records = int(max_records)
        self.max_records = int(max_records)
        self._pr = pr
        h = C.c_void_p()
        _lib.check(self.L.qdfn_ctx_create(C.byref(h), C.byref(pr)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.L.qdfn_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- operator -----------------------------------------------------------
    def set_dense(self, Ks, Kn, precision="fp64"):
        """Ks/Kn: (N, N) arrays K[receiver, source] (C or Fortran order)."""
        prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        Ks = np.asarray(Ks, dtype=np.float64)
        Kn = np.asarray(Kn, dtype=np.float64)
        if Ks.flags.f_contiguous and not Ks.flags.c_contiguous:
            lay, Ks_buf, Kn_buf = _lib.LAYOUT_COL, Ks.T, np.asfortranarray(Kn).T
        else:
            lay, Ks_buf, Kn_buf = _lib.LAYOUT_ROW, np.ascontiguousarray(Ks), np.ascontiguousarray(Kn)
        Ks_buf = np.ascontiguousarray(Ks_buf)
        Kn_buf = np.ascontiguousarray(Kn_buf)
        _lib.check(self.L.qdfn_set_dense(self._h, _lib.dp(Ks_buf), _lib.dp(Kn_buf), self.N, lay, prec))

    def set_dense_device(self, Ks, Kn, precision="fp64", layout="col", stream=0):
        """Ks/Kn: float64 CUDA tensors already holding K.  layout="col": shape
        (N_src, N_recv) contiguous, entry (r, s) at s*N + r (what
        assemble_rect_dev writes); "row": shape (N_recv, N_src)."""
        prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        lay = _lib.LAYOUT_COL if layout == "col" else _lib.LAYOUT_ROW
        _lib.check(self.L.qdfn_set_dense_dev(self._h, Ks.data_ptr(), Kn.data_ptr(), Ks.stride(0), lay, prec,
                                             C.c_void_p(stream)))

    def set_external_stress(self, t, normal, shear, pressure):
        t = _f64(t)
        nt = t.shape[0]
        n = _f64(normal, nt * self.N)
        s = _f64(shear, nt * self.N)
        p = _f64(pressure, nt * self.N)
        self._keep["ext"] = (t, n, s, p)
        _lib.check(self.L.qdfn_set_external_stress(self._h, nt, _lib.dp(t), _lib.dp(n), _lib.dp(s), _lib.dp(p)))

    # -- stepping -----------------------------------------------------------
    def run(self, nsteps, timeout_s=0.0):
        _lib.check(self.L.qdfn_run(self._h, int(nsteps), float(timeout_s)))

    def run_async(self, nsteps, stream=0, timeout_s=0.0):
        _lib.check(self.L.qdfn_run_async(self._h, int(nsteps), float(timeout_s), C.c_void_p(stream)))

    def sync(self):
        _lib.check(self.L.qdfn_sync(self._h))

    def kernels_per_run(self):
        return self.L.qdfn_kernels_per_run(self._h)

    def set_blocks(self, nblocks):
        """Cap the SMs (thread blocks) this context's runs use (0 = all)."""
        _lib.check(self.L.qdfn_set_blocks(self._h, int(nblocks)))

    def blocks(self):
        return self.L.qdfn_get_blocks(self._h)

    def set_early_cols(self, cols):
        """Next-step column chunks streamed in a step's solve tail (0..64; 0:
        the operator warps join the solves instead).  Schedule only."""
        _lib.check(self.L.qdfn_set_early_cols(self._h, int(cols)))

    def early_cols(self):
        return self.L.qdfn_get_early_cols(self._h)

    def counters(self):
        """Cumulative device counters: ns in time control / operator / solves /
        rotation, solve passes, steps, low-/high-velocity patch solves and their
        secant iterations."""
        out = np.zeros(18, dtype=np.int64)
        _lib.check(self.L.qdfn_get_counters(self._h, out.ctypes.data_as(C.POINTER(C.c_int64)), 18))
        keys = ("ns_control", "ns_operator", "ns_solve", "ns_rotate", "solve_passes", "steps",
                "lowv_solves", "lowv_iterations", "highv_solves", "highv_iterations",
                "ns_solve_own", "ns_solve_wait", "ns_operator_warps", "ns_solver_warps",
                "ns_operator_warps_slowest", "ns_solver_warps_slowest",
                "ns_chunk_solve_longest", "ns_last_row_block")
        return {k: int(out[i]) for i, k in enumerate(keys)}

    # -- state --------------------------------------------------------------
    def state(self, inst=0):
        N = self.N
        out = {k: np.zeros(N) for k in ("V", "D", "theta", "friction", "accel", "sigma_old")}
        T, dt, step = C.c_double(), C.c_double(), C.c_int64()
        _lib.check(self.L.qdfn_get_state(self._h, inst, *(_lib.dp(out[k]) for k in
                                                            ("V", "D", "theta", "friction", "accel", "sigma_old")),
                                         C.byref(T), C.byref(dt), C.byref(step)))
        out.update(T=T.value, dt=dt.value, step=step.value)
        return out

    def set_state(self, inst, st):
        arrs = [_f64(st[k], self.N) for k in ("V", "D", "theta", "friction", "accel", "sigma_old")]
        _lib.check(self.L.qdfn_set_state(self._h, inst, *(_lib.dp(a) for a in arrs), float(st["T"]),
                                         float(st["dt"]), int(st["step"])))

    STATE_FIELDS = ("V", "D", "theta", "friction", "accel", "sigma_old")

    def set_state_all(self, arrays, T, dt, step, stream=0):
        """Enqueue the state of every instance: arrays maps each STATE_FIELDS
        name to a host buffer of n_inst*N float64 (numpy array, or any object
        with a data_ptr(), e.g. a pinned CPU tensor); T, dt, step: n_inst
        values (float64, float64, int64 buffers).  Asynchronous on `stream`."""
        ptrs = [_addr(arrays[k]) if k in arrays else None for k in self.STATE_FIELDS]
        _lib.check(self.L.qdfn_set_state_all(self._h, *ptrs, _addr(T), _addr(dt), _addr(step), C.c_void_p(stream)))

    def get_state_all(self, arrays, T, dt, step, stream=0, wait=True):
        """Enqueue the copy of every instance's state into host buffers (as in
        set_state_all); wait=True synchronises and completes a run in flight on
        `stream` (raising its error like sync())."""
        ptrs = [_addr(arrays[k]) if k in arrays else None for k in self.STATE_FIELDS]
        _lib.check(self.L.qdfn_get_state_all(self._h, *ptrs, _addr(T), _addr(dt), _addr(step),
                                             C.c_void_p(stream), 1 if wait else 0))

    def history(self, inst=0):
        n = C.c_int64()
        _lib.check(self.L.qdfn_get_history(self._h, inst, None, None, None, None, None, None, C.byref(n)))
        n = n.value
        T, Dt = np.zeros(n), np.zeros(n)
        V, D, th, sg = (np.zeros((n, self.N)) for _ in range(4))
        if n:
            _lib.check(self.L.qdfn_get_history(self._h, inst, _lib.dp(T), _lib.dp(Dt), _lib.dp(V), _lib.dp(D),
                                               _lib.dp(th), _lib.dp(sg), C.byref(C.c_int64())))
        return dict(T=T, Dt=Dt, V=V, D=D, theta=th, sigma=sg)

    def apply(self, D):
        """(tld, knd) = (ELSM (0 - D), Kn D) for every instance; D is
        (n_inst, N) or (N,) when n_inst == 1."""
        D = _f64(D, self.N * self.n_inst)
        tld, knd = np.zeros_like(D), np.zeros_like(D)
        _lib.check(self.L.qdfn_apply_operator(self._h, _lib.dp(D), _lib.dp(tld), _lib.dp(knd)))
        return tld.reshape(self.n_inst, self.N), knd.reshape(self.n_inst, self.N)

    def kself(self):
        out = np.zeros(self.N)
        _lib.check(self.L.qdfn_get_kself(self._h, _lib.dp(out)))
        return out


def _load_external_stress(N):
    """The reference picks up Input_ExternalStressChange.jld2 from the working
    directory (Main_D :13-38); here the same keys are read from an .npz."""
    path = "Input_ExternalStressChange.npz"
    if not os.path.isfile(path):
        print("No External Stress Change Detected")
        return None
    z = np.load(path)
    if z["ExternalStress_Normal"].shape[1] != N:
        print("External Stress Change Dosen't match the fault Count. Will not be applied")
        return None
    print("External Stress Change Will be Applied")
    return dict(t=z["ExternalStress_TimeArray"], normal=z["ExternalStress_Normal"],
                shear=z["ExternalStress_Shear"], pressure=z["Pressure"])


def _padded(a, rows):
    """History array padded with zero rows to the reference's TotalRecord rows
    (Main_D :133-141 allocates zeros(TotalRecord, N) and fills record by record)."""
    a = np.asarray(a)
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    out = np.zeros((rows, a.shape[1]))
    n = min(rows, a.shape[0])
    out[:n] = a[:n]
    return out


def _run_and_save(sim, TotalStep, RecordStep, SaveStep, SaveResultFileName, verbose):
    """Runs TotalStep steps in SaveStep chunks and saves the history after every
    chunk that ends on a multiple of SaveStep, as Main_D :286-290 does (with
    SaveStep <= 0: one chunk, saved at its end).  The saved arrays have
    TotalRecord = round(TotalStep / RecordStep) rows, zero past the records
    written so far, like the reference's; History_Dt is saved beside them."""
    done = 0
    chunk = int(SaveStep) if SaveStep and SaveStep > 0 else int(TotalStep)
    rows = int(round(TotalStep / RecordStep)) if RecordStep else 0
    while done < TotalStep:
        n = min(chunk, TotalStep - done)
        sim.run(n)
        done += n
        h = sim.history(0)
        if SaveResultFileName and (done % chunk == 0 or not (SaveStep and SaveStep > 0)):
            np.savez(SaveResultFileName, History_V=_padded(h["V"], rows), History_Disp=_padded(h["D"], rows),
                     History_Time=_padded(h["T"], rows), History_Theta=_padded(h["theta"], rows),
                     History_NormalStress=_padded(h["sigma"], rows), History_Dt=_padded(h["Dt"], rows))
        if verbose:
            st = sim.state(0)
            print("%.5f %.5f   %.3e   %.3e" % (done / TotalStep, st["T"] / 86400, np.max(st["V"]), st["dt"]))
    return sim.history(0)


def main(StiffnessMatrixShear, StiffnessMatrixNormal, NormalStiffnessZero,
         ShearModulus, FaultCount, LoadingFaultCount, Mass,
         a, b, Dc, ThetaI, Vini, FrictionI,
         InitialNormalStress, LoadingRate,
         TotalStep, RecordStep, SwitchV, DtCut, RuptureDt, MaximumDt, SaveResultFileName, RockDensity,
         FaultCenter, FaultLengthStrike, FaultLengthDip, FaultStrikeAngle, FaultDipAngle, FaultRakeAngle, SaveStep,
         MinimumNormalStress, Alpha_Evo, EvolutionDR, *, external_stress=False, precision="fp64", verbose=False):
    """Dense-matrix cycle simulation (Functions_RSFDFN3DMain_D.jl main).
    Returns the history dict and writes SaveResultFileName (.npz) every
    SaveStep steps.  external_stress: None to disable, a dict (t, normal,
    shear, pressure), or False (default) to look for
    Input_ExternalStressChange.npz in the working directory as the reference
    does for its .jld2."""
    N = int(FaultCount)
    problem = dict(N=N, Nload=int(LoadingFaultCount), a=a, b=b, Dc=Dc, theta_i=ThetaI, V_i=Vini, f_i=FrictionI,
                   sigma0=InitialNormalStress, V_const=LoadingRate, mass=Mass, G=ShearModulus, rho=RockDensity,
                   sigma_min=MinimumNormalStress, switch_v=SwitchV, dt_cut=DtCut, rupture_dt=RuptureDt,
                   max_dt=MaximumDt, alpha_evo=Alpha_Evo, evolution_dr=EvolutionDR, interp_at_told=0)
    TotalRecord = int(round(TotalStep / RecordStep))
    sim = Simulation(problem, record_step=RecordStep, max_records=TotalRecord)
    Kn = np.zeros((N, N)) if NormalStiffnessZero == 1 else StiffnessMatrixNormal
    sim.set_dense(StiffnessMatrixShear, Kn, precision=precision)
    ext = _load_external_stress(N) if external_stress is False else external_stress
    if ext is not None:
        sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    hist = _run_and_save(sim, int(TotalStep), int(RecordStep), SaveStep, SaveResultFileName, verbose)
    sim.close()
    return hist


def main_H(ShearModulus, FaultCount, LoadingFaultCount, Mass, NormalStiffnessZero,
           a, b, Dc, ThetaI, Vini, FrictionI,
           InitialNormalStress, LoadingRate,
           TotalStep, RecordStep, SwitchV, DtCut, RuptureDt, MaximumDt, SaveResultFileName, RockDensity,
           FaultCenter, FaultLengthStrike, FaultLengthDip, FaultStrikeAngle, FaultDipAngle, FaultRakeAngle, SaveStep,
           MinimumNormalStress, Alpha_Evo,
           Ranks_Shear, Ranks_Normal, ElementRange_SR, NormalStiffness_H, ShearStiffness_H, ThreadCount, EvolutionDR,
           Admissible, *, external_stress=False, precision="fp64", verbose=False):
    """H-matrix cycle simulation (Functions_RSFDFN3DMain_H.jl main_H).
    ElementRange_SR is 1-based as in the reference; each block of
    ShearStiffness_H / NormalStiffness_H is a dense (recv x src) array or a
    (U, Vt) pair."""
    from .hmatrix import set_hmatrix_from_reference
    N = int(FaultCount)
    problem = dict(N=N, Nload=int(LoadingFaultCount), a=a, b=b, Dc=Dc, theta_i=ThetaI, V_i=Vini, f_i=FrictionI,
                   sigma0=InitialNormalStress, V_const=LoadingRate, mass=Mass, G=ShearModulus, rho=RockDensity,
                   sigma_min=MinimumNormalStress, switch_v=SwitchV, dt_cut=DtCut, rupture_dt=RuptureDt,
                   max_dt=MaximumDt, alpha_evo=Alpha_Evo, evolution_dr=EvolutionDR, interp_at_told=1)
    TotalRecord = int(round(TotalStep / RecordStep))
    sim = Simulation(problem, record_step=RecordStep, max_records=TotalRecord)
    set_hmatrix_from_reference(sim, ElementRange_SR, ShearStiffness_H, NormalStiffness_H,
                               zero_normal=(NormalStiffnessZero == 1), precision=precision)
    ext = _load_external_stress(N) if external_stress is False else external_stress
    if ext is not None:
        sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    hist = _run_and_save(sim, int(TotalStep), int(RecordStep), SaveStep, SaveResultFileName, verbose)
    sim.close()
    return hist
