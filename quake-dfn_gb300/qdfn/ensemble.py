"""Batched ensembles of fault networks of uneven size in one persistent launch.

Each geometry with its friction draws (up to 4 per geometry, sharing the
operator) is one qdfn context.  ``qdfn_ensemble_create`` groups the contexts so
that ONE cooperative launch advances all of them: member k runs on its own
contiguous range of thread blocks (its share of the SMs) with its own grid
barrier and its own adaptive time steps, and the members never wait on one
another.  The shares start from a cost estimate (operator bytes plus patch
solves) and ``balance`` -- the autotuner -- re-divides the SMs by each member's
measured device time, so that members taking the same number of steps finish
together.  (The reference runs one geometry per Julia process;
scripts/Functions_RSFDFN3DMain_D.jl:146-322 is the loop each member runs.)
"""
import ctypes as C

import numpy as np

from . import _lib, simulate


def _ptr(buf):
    """Address of a host buffer: a numpy array or a CPU tensor."""
    return buf.data_ptr() if hasattr(buf, "data_ptr") else buf.ctypes.data


def sm_shares(cost, n_sms):
    """Blocks per member: at least one each, minimising the longest member
    time cost/blocks, summing to ``n_sms`` -- the library's split rule
    (qdfn_ensemble_shares, host code, no GPU needed)."""
    cost = np.ascontiguousarray(np.asarray(cost, dtype=np.float64))
    out = np.zeros(cost.shape[0], dtype=np.int32)
    _lib.check(_lib.load().qdfn_ensemble_shares(int(cost.shape[0]), C.c_void_p(cost.ctypes.data), int(n_sms),
                                                C.c_void_p(out.ctypes.data)))
    return out.astype(np.int64)


class Ensemble:
    """members: list of dicts with keys ``problem`` (as for simulate.Simulation,
    per-patch arrays of length n_inst*N), ``n_inst``, ``Ks``/``Kn`` (host
    arrays, or float64 CUDA tensors in column layout), optional ``ext`` (dict
    t/normal/shear/pressure), ``record_step``/``max_records``.  precision as
    for Simulation.set_dense.  blocks: per-member block counts, or None for the
    library's cost estimate."""

    def __init__(self, members, precision="fp32", blocks=None):
        self.L = _lib.load()
        self.members = []
        for m in members:
            sim = simulate.Simulation(m["problem"], n_inst=m.get("n_inst", 1),
                                      record_step=m.get("record_step", 0), max_records=m.get("max_records", 0))
            if hasattr(m["Ks"], "data_ptr"):
                sim.set_dense_device(m["Ks"], m["Kn"], precision, layout=m.get("layout", "col"))
            else:
                sim.set_dense(m["Ks"], m["Kn"], precision)
            if m.get("ext") is not None:
                e = m["ext"]
                sim.set_external_stress(e["t"], e["normal"], e["shear"], e["pressure"])
            self.members.append(sim)
        n = len(self.members)
        handles = (C.c_void_p * n)(*[s._h.value for s in self.members])
        bl = None
        if blocks is not None:
            bl = np.ascontiguousarray(np.asarray(blocks, dtype=np.int32))
            if bl.shape[0] != n:
                raise ValueError("blocks: expected %d values" % n)
        h = C.c_void_p()
        _lib.check(self.L.qdfn_ensemble_create(C.byref(h), n, handles,
                                               None if bl is None else C.c_void_p(bl.ctypes.data)))
        self._h = h

    @property
    def blocks(self):
        out = np.zeros(len(self.members), dtype=np.int32)
        _lib.check(self.L.qdfn_ensemble_get_blocks(self._h, C.c_void_p(out.ctypes.data)))
        return out

    def set_blocks(self, blocks=None):
        bl = None if blocks is None else np.ascontiguousarray(np.asarray(blocks, dtype=np.int32))
        _lib.check(self.L.qdfn_ensemble_set_blocks(self._h, None if bl is None else C.c_void_p(bl.ctypes.data)))

    def balance(self):
        """Autotuner step: re-divide the SMs by the members' measured cost since
        the last balance."""
        _lib.check(self.L.qdfn_ensemble_balance(self._h))

    def autotune(self, steps, rounds=3, timeout_s=0.0):
        """Runs `steps` steps in `rounds` parts with a balance after each (these
        steps advance the ensemble: use them as warm-up).  Returns the shares
        after each round."""
        hist = [self.blocks.copy()]
        per = max(1, int(steps) // max(1, int(rounds)))
        done = 0
        while done < steps:
            n = min(per, steps - done)
            self.run(n, timeout_s=timeout_s)
            done += n
            self.balance()
            hist.append(self.blocks.copy())
        return hist

    # -- the whole ensemble's state in one copy each way -------------------
    def state_words(self):
        """8-byte words of the ensemble's state record (qdfn_ensemble_state_bytes / 8)."""
        n = C.c_int64()
        _lib.check(self.L.qdfn_ensemble_state_bytes(self._h, C.byref(n)))
        return int(n.value) // 8

    def pack_states(self, states, out=None):
        """The state record from per-member, per-instance state dicts (as
        Simulation.state returns): member after member, [6][n_inst][N] (V, D,
        theta, friction, accel, sigma_old), then T, dt, step [n_inst].  `out`:
        a float64 buffer (numpy array or CPU tensor) of state_words() words."""
        buf = np.empty(self.state_words()) if out is None else out
        a = buf.numpy() if hasattr(buf, "numpy") else buf
        o = 0
        for sim, sts in zip(self.members, states):
            R, N = sim.n_inst, sim.N
            for k in simulate.Simulation.STATE_FIELDS:
                a[o:o + R * N] = np.concatenate([st[k] for st in sts])
                o += R * N
            a[o:o + R] = [st["T"] for st in sts]
            a[o + R:o + 2 * R] = [st["dt"] for st in sts]
            a[o + 2 * R:o + 3 * R].view(np.int64)[:] = [st["step"] for st in sts]
            o += 3 * R
        return buf

    def unpack_states(self, buf):
        """Per-member lists of per-instance state dicts from a state record."""
        a = buf.numpy() if hasattr(buf, "numpy") else np.asarray(buf)
        out, o = [], 0
        for sim in self.members:
            R, N = sim.n_inst, sim.N
            f = {}
            for k in simulate.Simulation.STATE_FIELDS:
                f[k] = a[o:o + R * N].reshape(R, N).copy()
                o += R * N
            T, dt, step = a[o:o + R], a[o + R:o + 2 * R], a[o + 2 * R:o + 3 * R].view(np.int64)
            o += 3 * R
            out.append([dict({k: f[k][r] for k in f}, T=float(T[r]), dt=float(dt[r]), step=int(step[r]))
                        for r in range(R)])
        return out

    def set_state_all(self, buf, stream=None):
        """Every member's state from one host buffer (state record; pinned for
        an asynchronous copy), one copy (qdfn_ensemble_set_state_all)."""
        _lib.check(self.L.qdfn_ensemble_set_state_all(self._h, C.c_void_p(_ptr(buf)),
                                                      C.c_void_p(stream) if stream else None))

    def get_state_all(self, buf, stream=None, wait=True):
        """Every member's state into one host buffer, one copy; with wait it
        also completes a run in flight on the same stream."""
        _lib.check(self.L.qdfn_ensemble_get_state_all(self._h, C.c_void_p(_ptr(buf)),
                                                      C.c_void_p(stream) if stream else None, 1 if wait else 0))

    def set_fill(self, on=True):
        """Fill mode: members that have taken the run's nsteps keep stepping
        until every member has, so that no SM idles (qdfn_ensemble_set_fill)."""
        _lib.check(self.L.qdfn_ensemble_set_fill(self._h, 1 if on else 0))

    def steps(self):
        """Step count of every instance of every member."""
        return np.asarray([sim.state(r)["step"] for sim in self.members for r in range(sim.n_inst)])

    def run_async(self, nsteps, timeout_s=0.0, stream=None):
        _lib.check(self.L.qdfn_ensemble_run_async(self._h, int(nsteps), float(timeout_s),
                                                  C.c_void_p(stream) if stream else None))

    def sync(self):
        _lib.check(self.L.qdfn_ensemble_sync(self._h))

    def run(self, nsteps, timeout_s=0.0):
        _lib.check(self.L.qdfn_ensemble_run(self._h, int(nsteps), float(timeout_s)))

    def sim_years(self):
        """Simulated time of every instance of every member, in years."""
        out = []
        for sim in self.members:
            out.extend(sim.state(r)["T"] / (365.25 * 86400.0) for r in range(sim.n_inst))
        return np.asarray(out)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.L.qdfn_ensemble_destroy(self._h)
            self._h = None
        for s in self.members:
            s.close()
        self.members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
