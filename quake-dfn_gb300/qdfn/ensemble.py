"""Batched ensembles of geometries of uneven size on one GPU.

Each geometry (with its friction draws, up to 4 per geometry sharing the
operator) is one qdfn context.  The contexts split the SMs in proportion to
their work -- operator bytes per step plus the per-patch solves -- through
``qdfn_set_blocks``, and their persistent runs are launched on separate streams,
so every geometry advances at once on its own share of the GPU with its own
adaptive time steps.  The contexts share nothing and never wait on one
another.  (The reference runs one geometry per Julia process.)
"""
import numpy as np

from . import simulate


def sm_shares(work, n_sms):
    """Blocks per member: at least one each, proportional to `work`, summing
    to at most n_sms (members beyond n_sms cannot all be resident at once)."""
    work = np.asarray(work, dtype=np.float64)
    m = work.shape[0]
    if m > n_sms:
        raise ValueError("%d members need at least %d SMs" % (m, m))
    share = np.maximum(1, np.floor(n_sms * work / work.sum()).astype(np.int64))
    while share.sum() > n_sms:                       # trim the largest
        share[np.argmax(share)] -= 1
    spare = n_sms - int(share.sum())                 # hand out the rest by largest deficit
    if spare > 0:
        deficit = n_sms * work / work.sum() - share
        for k in np.argsort(-deficit)[:spare]:
            share[k] += 1
    return share


class Ensemble:
    """members: list of dicts with keys ``problem`` (as for simulate.Simulation,
    per-patch arrays of length n_inst*N), ``n_inst``, ``Ks``/``Kn`` (host
    arrays or float64 CUDA tensors in column layout, see set_dense_device),
    optional ``ext`` (dict t/normal/shear/pressure).  precision as for
    Simulation.set_dense."""

    def __init__(self, members, precision="fp32", n_sms=None):
        import torch
        self.members = []
        self.streams = []
        work = []
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
            N, R = sim.N, sim.n_inst
            work.append(float(N) * N * 2 * (8 if precision == "fp64" else 4) + 2000.0 * N * R)
            self.members.append(sim)
            self.streams.append(torch.cuda.Stream())
        if n_sms is None:
            n_sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        self.blocks = sm_shares(work, n_sms)
        for sim, b in zip(self.members, self.blocks):
            sim.set_blocks(int(b))

    def run_async(self, nsteps, timeout_s=0.0):
        for sim, st in zip(self.members, self.streams):
            sim.run_async(nsteps, stream=st.cuda_stream, timeout_s=timeout_s)

    def sync(self):
        """Waits for every member; raises the first member's error."""
        err = None
        for sim in self.members:
            try:
                sim.sync()
            except Exception as e:   # keep draining the others
                err = err or e
        if err is not None:
            raise err

    def run(self, nsteps, timeout_s=0.0):
        self.run_async(nsteps, timeout_s)
        self.sync()

    def sim_years(self):
        """Simulated time of every instance of every member, in years."""
        out = []
        for sim in self.members:
            out.extend(sim.state(r)["T"] / (365.25 * 86400.0) for r in range(sim.n_inst))
        return np.asarray(out)
