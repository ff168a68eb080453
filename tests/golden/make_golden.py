"""Writes tests/golden/c1_single_fault_oracle.npz.

The reference (Julia) ships no tests, golden vectors or fixtures and cannot run
here, so this fixture is produced by the FP64 CPU oracle (oracle/, a C++
restatement of the reference algorithm, itself pinned by the known-answer
tests in tests/test_oracle_kat.py).  Workload: the plain-method single fault --
a vertical strike-slip fault 20 km x 10 km, top at 0.5 km, 40 x 20 = 800 Okada
patches of 500 m, G = 32 GPa, nu = 0.25, aging law, a = 0.010 / b = 0.015 in
the core and a = 0.020 in a 2 km border ring, Dc = 1 mm, 40 MPa, V_i = 1e-9 m/s,
0.01 MPa/yr background shear stressing -- synthetic, seeded inputs of the
shapes the benchmark configuration names.

Stored: time and step size of every 2nd of the first 400 steps, the state after
step 120, and the event fragments (slip rate above 1e-2 m/s between records,
qdfn.events) of the 400-step history.  The first event nucleates near step 150;
from there a 1e-15 relative perturbation of the operator grows to ~1e-7 in slip
(measured with this oracle), so the GPU FP64 path is compared with the state
at step 120 to 1e-9 and with the later history more loosely, its event onsets
to 1e-9 (they move by ~1e-14 under the same perturbation).

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "quake-dfn_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

NSTEPS, RECORD, NSTATE = 400, 2, 120
OUT = os.path.join(HERE, "c1_single_fault_oracle.npz")


def c1_problem(oracle_mod):
    from qdfn import synth
    sysd = synth.single_fault()
    rec = sysd["records"]
    cols = dict(cx=rec[:, 0], cy=rec[:, 1], cz=rec[:, 2], ls=rec[:, 3], ld=rec[:, 4], strike=rec[:, 5],
                dip=rec[:, 6], rake=rec[:, 7])
    Ks, Kn = oracle_mod.assemble_rect(cols, cols, sysd["G"], sysd["nu"])
    prob = synth.problem_dict(sysd, np.diag(Ks))
    ext = synth.external_ramp(sysd["N"], sysd["stressing_rate"], 1e12)
    oprob = dict(prob, ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
    return sysd, Ks, Kn, prob, ext, oprob


def run_oracle(oracle_mod, nsteps=NSTEPS, record=RECORD, nstate=NSTATE):
    from qdfn import events
    sysd, Ks, Kn, prob, ext, oprob = c1_problem(oracle_mod)
    o = oracle_mod.Simulation(oprob, ("dense", Ks, Kn))
    h1 = o.run(nstate, record_step=record, max_rec=nstate // record)
    st = {k: o.state[k].copy() for k in ("V", "D", "theta")}
    T_state = o.T
    h2 = o.run(nsteps - nstate, record_step=record, max_rec=(nsteps - nstate) // record)
    hT = np.concatenate([h1["T"], h2["T"]])
    hDt = np.concatenate([h1["Dt"], h2["Dt"]])
    hD = np.concatenate([h1["D"], h2["D"]])
    rec = sysd["records"]
    ft, floc, fm, fn = events.event_fragments(hT, hD, rec[:, :3], events.patch_area_rect(rec[:, 3], rec[:, 4]),
                                             sysd["G"])
    return dict(T=hT, Dt=hDt, V=st["V"], D=st["D"], theta=st["theta"], T_state=np.float64(T_state),
                step=np.int64(o.step), frag_t=ft, frag_moment=fm, frag_count=np.int64(fn))


def main():
    import oracle as oracle_mod
    oracle_mod.build()
    out = run_oracle(oracle_mod)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, {k: np.shape(v) for k, v in out.items()})


if __name__ == "__main__":
    main()
