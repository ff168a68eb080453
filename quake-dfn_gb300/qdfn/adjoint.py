"""Gradients of trajectory losses with respect to the per-patch friction
parameters a, b and Dc, through the library's discrete adjoint
(qdfn_adjoint_run).

``gradient`` is the plain call; ``onset_seeds`` turns an event onset time --
the interpolated time at which a patch's slip rate first crosses a threshold,
the start of an event fragment of scripts/Functions_Plot.jl:430-510 -- into the
adjoint's per-step seeds; ``CycleLoss`` is a torch.autograd.Function (the
counterpart of the ChainRulesCore rrule a Julia caller would write, see
INTEGRATION.md) whose forward runs the cycle and whose backward runs the
adjoint.
"""
import ctypes as C

import numpy as np

from . import _lib


def _dev(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def gradient(sim, nsteps, dL_dD_final=None, seeds=None, checkpoint_every=0, timeout_s=0.0):
    """Runs `nsteps` steps of `sim` from its current state and returns the
    gradient of the loss whose derivatives are given -- dL_dD_final
    ((n_inst, N) or (N,)) on the last slip, and `seeds`, a list of
    (step, inst, patch, dL_dV, dL_dD, dL_dT) -- as a dict of (n_inst, N)
    arrays a, b, Dc.  The simulation ends at the window's last state."""
    L = _lib.load()
    R, N = sim.n_inst, sim.N
    dD = None
    if dL_dD_final is not None:
        dD = np.ascontiguousarray(np.asarray(dL_dD_final, dtype=np.float64).reshape(R, N))
    seeds = seeds or []
    ns = len(seeds)
    st = np.array([s[0] for s in seeds], dtype=np.int64)
    si = np.array([s[1] for s in seeds], dtype=np.int32)
    sp = np.array([s[2] for s in seeds], dtype=np.int64)
    sv = np.array([s[3] for s in seeds], dtype=np.float64)
    sd = np.array([s[4] for s in seeds], dtype=np.float64)
    stt = np.array([s[5] for s in seeds], dtype=np.float64)
    ga, gb, gdc = (np.zeros((R, N)) for _ in range(3))
    arrs = [st, si, sp, sv, sd, stt]
    ptrs = [_dev(a) if ns else None for a in arrs]
    _lib.check(L.qdfn_adjoint_run(sim._h, int(nsteps), int(checkpoint_every), _dev(dD), ns, *ptrs,
                                  _dev(ga), _dev(gb), _dev(gdc), float(timeout_s)))
    return dict(a=ga, b=gb, Dc=gdc)


def onset_times(T, V, ns, v_crit=1e-2, count=5):
    """Event onsets of a one-instance history recorded every step (T: (n,),
    V: (n, N); row k is the state after step k + 1, and T0/V0 the starting
    ones prepended by the caller): the first `count` times at which the maximum
    slip rate over the first `ns` patches rises through v_crit, each linearly
    interpolated between the two steps around it.  Returns a list of (time,
    step, patch, fraction)."""
    out = []
    vmax = np.max(V[:, :ns], axis=1)
    above = vmax > v_crit
    for n in range(1, len(T)):
        if above[n] and not above[n - 1]:
            k = int(np.argmax(V[n, :ns]))
            v0, v1 = V[n - 1, k], V[n, k]
            f = (v_crit - v0) / (v1 - v0) if v1 != v0 else 1.0
            out.append((T[n - 1] + f * (T[n] - T[n - 1]), n, k, f))
            if len(out) == count:
                break
    return out


def onset_seeds(T, V, onset, dL_dt, inst=0, v_crit=1e-2):
    """Seeds of one interpolated onset (from onset_times) for the adjoint:
    t_e = T[n-1] + f (T[n] - T[n-1]) with f = (v_crit - V[n-1,k]) / (V[n,k] - V[n-1,k]),
    differentiated in T[n-1], T[n], V[n-1,k] and V[n,k] and scaled by dL/dt_e.
    History row n is the state after step n (row 0 the starting state)."""
    _, n, k, f = onset
    v0, v1 = V[n - 1, k], V[n, k]
    dT = T[n] - T[n - 1]
    den = (v1 - v0) ** 2
    return [(n - 1, inst, k, dL_dt * dT * (v_crit - v1) / den, 0.0, dL_dt * (1.0 - f)),
            (n, inst, k, -dL_dt * dT * (v_crit - v0) / den, 0.0, dL_dt * f)]


def _torch_function():
    import torch

    class CycleLoss(torch.autograd.Function):
        """D_final = cycle(a, b, Dc): forward runs `nsteps` steps of a fresh
        simulation built by make_sim(a, b, Dc) (float64 CPU tensors, (n_inst,
        N)); backward builds it again and runs the adjoint with the incoming
        dL/dD_final."""

        @staticmethod
        def forward(ctx, a, b, Dc, make_sim, nsteps):
            sim = make_sim(a.detach().numpy(), b.detach().numpy(), Dc.detach().numpy())
            sim.run(nsteps)
            D = np.stack([sim.state(r)["D"] for r in range(sim.n_inst)])
            sim.close()
            ctx.make_sim, ctx.nsteps = make_sim, nsteps
            ctx.save_for_backward(a, b, Dc)
            return torch.from_numpy(D)

        @staticmethod
        def backward(ctx, gD):
            a, b, Dc = ctx.saved_tensors
            sim = ctx.make_sim(a.detach().numpy(), b.detach().numpy(), Dc.detach().numpy())
            g = gradient(sim, ctx.nsteps, dL_dD_final=gD.detach().numpy())
            sim.close()
            return (torch.from_numpy(g["a"]), torch.from_numpy(g["b"]), torch.from_numpy(g["Dc"]), None, None)

    return CycleLoss


def __getattr__(name):
    if name == "CycleLoss":
        return _torch_function()
    raise AttributeError(name)
