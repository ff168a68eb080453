"""Benchmark: ensemble simulated-years per wall-clock hour of the earthquake-cycle
step loop on GB300.

Workload (default): the 30-fault random network (seed 2, 100 m patches,
12,813 rectangular patches; shapes of the reference's fault-network config),
four friction draws on that geometry advanced together as one ensemble, elastic
operator stored in FP32 (mixed precision) with FP64 state, friction inversion
and time control.  Synthetic, seeded input: the reference ships no benchmark
data.  A bench "step" is one adaptive time step of every ensemble member.

  value     device-resident: one persistent launch advances the ensemble K steps
            (inputs already in HBM), CUDA events on the launch stream
  e2e       the same K steps through the C ABI with host buffers: every step
            uploads the ensemble state from pinned host memory
            (qdfn_set_state), runs one step (qdfn_run) and reads the state back
            (qdfn_get_state)
  fp64_gpu  the same window with the operator in FP64, one instance per launch
            (the plain FP64 GPU path), and the slip error of the mixed run
            against it
  cpu_baseline  the FP64 CPU oracle (restatement of the reference algorithm)
            on a bounded sample of the same window, all host threads

--impl reference times that CPU oracle on the whole window (the reference is
Julia, which is not available; the oracle restates its algorithm in C++).
Under torchrun each rank runs an independent replica (the path does not shard:
"replicas only"); value sums the ranks' simulated years over the slowest rank.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "quake-dfn_gb300"))

YEAR = 365.25 * 24 * 3600.0
TIMEOUT = 300.0   # bound on every device run (s): the kernel returns QDFN_ERR_TIMEOUT past it


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=100)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "bf16x2", "fp64"])
    ap.add_argument("--inst", type=int, default=4)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--faults", type=int, default=30)
    ap.add_argument("--cpu-sample-s", type=float, default=20.0)
    ap.add_argument("--ref-instances", type=int, default=1,
                    help="ensemble members the CPU reference arm times (a bounded sample)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="ensemble", choices=["network", "ensemble", "tri_h", "adjoint"],
                    help="ensemble (default, C4): 64 fault networks of 800-6,000 patches x 4 friction draws in "
                         "one persistent launch; network (C2): the 30-fault network x 4 draws")
    ap.add_argument("--geometries", type=int, default=64)
    ap.add_argument("--tri-edge", type=float, default=80.0,
                    help="tri_h: triangle edge in m (80: ~50,000 triangles; 160: ~12,500)")
    ap.add_argument("--tree", default="pca", choices=["pca", "device"],
                    help="tri_h: H-matrix cluster tree and partition -- host principal-axis bisection, or built "
                         "on the device (qdfn_hstruct_build)")
    ap.add_argument("--cpu-members", type=int, default=4,
                    help="ensemble members (at size quantiles) in the CPU oracle sample and the reference arm")
    ap.add_argument("--plain-members", type=int, default=16,
                    help="ensemble members (at size quantiles, one draw each) run through the plain FP64 GPU path, "
                         "one instance per launch (0: skip)")
    ap.add_argument("--rebalance-every", type=int, default=15,
                    help="ensemble: steps per launch in the timed window, the SMs re-divided between launches "
                         "(0: one launch)")
    ap.add_argument("--no-fill", dest="fill", action="store_false",
                    help="skip the fill-mode measurement of the ensemble window")
    ap.add_argument("--horizon", type=int, default=1000,
                    help="steps of the mixed-vs-FP64 accuracy horizon (from t = 0)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, dev):
    """The largest x over the ranks of the default process group (every rank
    gets it): the job's time is the slowest rank's."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, dev):
    """The sum of x over the ranks (every rank gets it): the job's work is all
    ranks' work."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t)
    return float(t.item())


def workload(args):
    from qdfn import synth
    sysd = synth.fault_network(seed=args.seed, n_faults=args.faults)
    draws = synth.friction_draws(sysd, args.inst, seed=1)
    return sysd, draws


def problem(sysd, draws, kdiag, n_inst):
    from qdfn import synth
    return synth.problem_dict(sysd, kdiag, n_inst=n_inst, draws=draws)


def ext_ramp(sysd):
    from qdfn import synth
    return synth.external_ramp(sysd["N"], sysd["stressing_rate"], 1e12)


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if sm:
            out.update(sm_mhz=float(np.median(sm)), sm_max_mhz=float(np.max(smax)), reasons=sorted(reasons),
                       samples=len(sm))
        return out


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per simulation step of the kernel from a committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "k_sim_network_fp32_r4.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return None
    return None


# ---------------------------------------------------------------------------
def total_sim_time(sim, n):
    return np.array([sim.state(r)["T"] for r in range(n)])


def run_ours(args):
    import torch
    from qdfn import _lib, assemble, simulate

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    sysd, draws = workload(args)
    N, R = sysd["N"], args.inst

    # stiffness on the device (FP64 Okada), column-major like Julia's K[recv, src]
    rec = torch.tensor(sysd["records"], dtype=torch.float64, device=dev)
    Ks = torch.empty((N, N), dtype=torch.float64, device=dev)
    Kn = torch.empty((N, N), dtype=torch.float64, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    assemble.assemble_rect_dev(rec, rec, sysd["G"], sysd["nu"], Ks, Kn, stream=stream.cuda_stream, layout="col")
    e1.record(stream)
    torch.cuda.synchronize()
    asm_ms = e0.elapsed_time(e1)
    kdiag = torch.diagonal(Ks).cpu().numpy()
    prob = problem(sysd, draws, kdiag, R)
    ext = ext_ramp(sysd)

    sim = simulate.Simulation(prob, n_inst=R)
    sim.set_dense_device(Ks, Kn, args.precision, layout="col", stream=stream.cuda_stream)
    sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    sim64 = None
    if not args.no_fp64:
        p1 = problem(sysd, {k: v[:N] for k, v in draws.items()}, kdiag, 1)
        sim64 = simulate.Simulation(p1, n_inst=1)
        sim64.set_dense_device(Ks, Kn, "fp64", layout="col", stream=stream.cuda_stream)
        sim64.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    Ks_host = Kn_host = None
    if rank == 0 and not args.no_cpu:
        Ks_host = Ks.cpu().numpy()  # (src, recv) memory = K[recv, src] column-major -> transpose view
        Kn_host = Kn.cpu().numpy()

    # warm-up (untimed): the first W steps of the trajectory
    sim.run(args.warmup, timeout_s=TIMEOUT)
    if sim64 is not None:
        sim64.run(args.warmup, timeout_s=TIMEOUT)
    start_states = [sim.state(r) for r in range(R)]
    T0 = np.array([s["T"] for s in start_states])

    # ---- timed: one persistent launch over K steps
    clocks = ClockSampler(local)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    cnt0 = sim.counters()
    sim.run_async(args.steps, stream=stream.cuda_stream, timeout_s=TIMEOUT)
    ev1.record(stream)
    torch.cuda.synchronize()
    sim.sync()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    cnt1 = sim.counters()
    phases = {k: cnt1[k] - cnt0[k] for k in cnt1}
    if ws > 1:
        ms = max_over_ranks(ms, dev)
        torch.distributed.barrier()
    T1 = total_sim_time(sim, R)
    sim_years = float(np.sum(T1 - T0)) / YEAR
    end_state0 = sim.state(0)
    if ws > 1:
        sim_years_all = sum_over_ranks(sim_years, dev)
    else:
        sim_years_all = sim_years
    value = sim_years_all / (ms / 1e3 / 3600.0)

    # ---- roofline of the persistent kernel (dominant, and the only kernel of the run)
    esz = {"fp32": 4, "bf16x2": 4, "fp64": 8}[args.precision]
    mat_bytes = 2 * N * N * esz      # shear + normal operator, padding rows not counted
    vec_bytes = R * N * 8 * 14       # state read/write + matvec partials, per step
    alg_bytes = args.steps * (mat_bytes + vec_bytes)
    achieved = alg_bytes / (ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    prof = profiled_traffic()
    traffic = None
    if prof and prof.get("N") == N and prof.get("precision") == args.precision and prof.get("inst") == R:
        traffic = float(prof["dram_bytes_per_step"]) * args.steps

    # ---- FP64 GPU path on the same window (draw 0 alone)
    fp64 = None
    if sim64 is not None:
        s0 = sim64.state(0)
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        sim64.run_async(args.steps, stream=stream.cuda_stream, timeout_s=TIMEOUT)
        f1.record(stream)
        torch.cuda.synchronize()
        sim64.sync()
        ms64 = f0.elapsed_time(f1)
        s1 = sim64.state(0)
        yrs64 = (s1["T"] - s0["T"]) / YEAR
        slip_err = float(np.max(np.abs(end_state0["D"] - s1["D"])) / max(np.max(np.abs(s1["D"])), 1e-300))
        fp64 = {"value": yrs64 / (ms64 / 1e3 / 3600.0), "ms_per_step": ms64 / args.steps, "instances": 1,
                "slip_rel_err_vs_fp64": slip_err, "mixed_over_fp64": (value / max(ws, 1)) / (yrs64 / (ms64 / 3.6e6))}

    # ---- accuracy horizon: mixed ensemble vs the FP64 path from t = 0,
    # compared every 100 steps (this network is chaotic: even a 1e-15
    # perturbation of the FP64 operator grows to ~1e-6 slip error within ~2000
    # steps, so the 1e-6 bar holds over a horizon, reported here)
    horizon = None
    if sim64 is not None:
        pm = problem(sysd, draws, kdiag, R)
        p1 = problem(sysd, {k: v[:N] for k, v in draws.items()}, kdiag, 1)
        am = simulate.Simulation(pm, n_inst=R)
        am.set_dense_device(Ks, Kn, args.precision, layout="col", stream=stream.cuda_stream)
        a64 = simulate.Simulation(p1, n_inst=1)
        a64.set_dense_device(Ks, Kn, "fp64", layout="col", stream=stream.cuda_stream)
        for a in (am, a64):
            a.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
        errs = []
        done = 0
        total = args.warmup + args.steps
        while done < total:
            n = min(100, total - done)
            am.run(n, timeout_s=TIMEOUT)
            a64.run(n, timeout_s=TIMEOUT)
            done += n
            d0, d1 = am.state(0)["D"], a64.state(0)["D"]
            errs.append((done, float(np.max(np.abs(d0 - d1)) / max(np.max(np.abs(d1)), 1e-300))))
        within = [st for st, e in errs if e <= 1e-6]
        first_bad = next((st for st, e in errs if e > 1e-6), None)
        horizon = {"checked_every": 100, "steps_within_1e-6": (first_bad - 100) if first_bad else total,
                   "first_step_above_1e-6": first_bad,
                   "err_at": {str(st): e for st, e in errs[::4] + [errs[-1]]}}
        am.close()
        a64.close()
    del Ks, Kn
    torch.cuda.empty_cache()

    # ---- e2e through the C ABI with host buffers, same window: every step the
    # whole ensemble state goes up from pinned host memory, one step runs, the
    # state comes back (qdfn_set_state_all -> qdfn_run_async -> qdfn_get_state_all,
    # one synchronisation per step)
    e2e = None
    if not args.no_e2e:
        for r in range(R):
            sim.set_state(r, start_states[r])
        names = simulate.Simulation.STATE_FIELDS
        # one pinned block [field][instance][patch]: the library moves it in one copy per direction
        pin6 = torch.empty((len(names), R, N), dtype=torch.float64).pin_memory()
        pin = {k: pin6[f] for f, k in enumerate(names)}
        for k in names:
            pin[k].copy_(torch.from_numpy(np.stack([np.ascontiguousarray(start_states[r][k]) for r in range(R)])))
        Tdt = torch.tensor([[start_states[r]["T"] for r in range(R)], [start_states[r]["dt"] for r in range(R)]],
                           dtype=torch.float64).pin_memory()
        Tp, dtp = Tdt[0], Tdt[1]
        stp = torch.tensor([start_states[r]["step"] for r in range(R)], dtype=torch.int64).pin_memory()
        sptr = stream.cuda_stream
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            sim.set_state_all(pin, Tp, dtp, stp, stream=sptr)
            sim.run_async(1, stream=sptr, timeout_s=TIMEOUT)
            sim.get_state_all(pin, Tp, dtp, stp, stream=sptr, wait=True)
        t_e2e = time.perf_counter() - t0
        yrs = float(sum(Tp[r].item() - start_states[r]["T"] for r in range(R))) / YEAR
        per_inst = 6 * N * 8 + 3 * 8
        e2e = {"value": (yrs * max(ws, 1)) / (t_e2e / 3600.0), "unit": "sim-years/hour",
               "h2d_bytes_per_step": R * per_inst, "d2h_bytes_per_step": R * per_inst}

    # ---- CPU baseline: oracle on a bounded sample of the window
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_sample(args, sysd, draws, kdiag, Ks_host, Kn_host, start_states, ext)

    if rank == 0:
        line = {
            "metric": "ensemble sim-years/hour, mixed-prec vs FP64 on GPU at <=1e-6 rel slip error",
            "value": value, "unit": "sim-years/hour", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32-operator/fp64-state" if args.precision != "fp64" else "fp64",
            "data": "synthetic (seeded fault network; the reference ships no benchmark data)",
            "config": {"workload": "fault network, %d faults seed %d, %d rectangular patches, %d friction draws "
                                   "(ensemble), operator %s, external stressing 0.01 MPa/yr"
                                   % (args.faults, args.seed, N, R, args.precision),
                       "patches": N, "instances": R, "precision": args.precision, "parallelism": "replicas",
                       "l2": "operator %.2f GB per step > 129 MB L2 (no flush needed)" % (mat_bytes / 1e9),
                       "sim_years_in_window": sim_years_all},
            "gpu_launches": sim.kernels_per_run(),
            "e2e": e2e,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "note": "k_sim persistent kernel, algorithmic bytes = K x (2 N^2 x %d B operator + "
                                 "state vectors); peak %s" % (esz, peak_kind)},
            "cpu_baseline": cpu,
            "fp64_gpu": fp64,
            "accuracy_horizon": horizon,
            "assembly": {"pairs": N * N, "ms": asm_ms, "pairs_per_s": N * N / (asm_ms / 1e3)},
            "phases_ms_per_step": {"time_control": phases["ns_control"] / 1e6 / args.steps,
                                   "operator_with_overlapped_solves": phases["ns_operator"] / 1e6 / args.steps,
                                   "block0_operator_warps": phases["ns_operator_warps"] / 1e6 / args.steps,
                                   "block0_solver_warps": phases["ns_solver_warps"] / 1e6 / args.steps,
                                   "slowest_block_operator_warps":
                                       phases["ns_operator_warps_slowest"] / 1e6 / args.steps,
                                   "slowest_block_solver_warps": phases["ns_solver_warps_slowest"] / 1e6 / args.steps,
                                   "longest_chunk_solve": phases["ns_chunk_solve_longest"] / 1e6 / args.steps,
                                   "last_row_block_complete": phases["ns_last_row_block"] / 1e6 / args.steps,
                                   "solve_reduce_and_retries": phases["ns_solve"] / 1e6 / args.steps,
                                   "block0_retry_solves": phases["ns_solve_own"] / 1e6 / args.steps,
                                   "block0_barrier_wait": phases["ns_solve_wait"] / 1e6 / args.steps,
                                   "rotation": phases["ns_rotate"] / 1e6 / args.steps,
                                   "solve_passes_per_step": phases["solve_passes"] / max(phases["steps"], 1),
                                   "lowv_solves_per_step": phases["lowv_solves"] / max(phases["steps"], 1),
                                   "lowv_iterations_per_solve":
                                       phases["lowv_iterations"] / max(phases["lowv_solves"], 1),
                                   "highv_solves_per_step": phases["highv_solves"] / max(phases["steps"], 1),
                                   "highv_iterations_per_solve":
                                       phases["highv_iterations"] / max(phases["highv_solves"], 1)},
            "clocks": clk,
        }
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def cpu_sample(args, sysd, draws, kdiag, Ks_cm, Kn_cm, start_states, ext):
    """Oracle (FP64, OpenMP on all host cores) from the window's start state for
    a bounded number of steps; sim-years/hour of the ensemble on that sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    N, R = sysd["N"], args.inst
    Ks = Ks_cm.T  # device buffer was (src, recv): K[recv, src] = buf[src, recv]
    Kn = Kn_cm.T
    nth = os.cpu_count()
    sims = []
    shared = None
    for r in range(R):
        p = problem(sysd, {k: v[r * N:(r + 1) * N] for k, v in draws.items()}, kdiag, 1)
        p.update(ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
        s = oracle.Simulation(p, ("dense", Ks, Kn) if shared is None else ("shared", shared), nthreads=nth)
        shared = s if shared is None else shared
        st = start_states[r]
        for k in ("V", "D", "theta", "friction", "accel", "sigma_old"):
            s.state[k][:] = st[k]
        s.set_scalars(st["T"], st["dt"], st["step"])
        sims.append(s)
    T0 = np.array([s.T for s in sims])
    t0 = time.perf_counter()
    for s in sims:
        s.run(1)
    per_step = time.perf_counter() - t0
    k = int(max(1, min(args.steps - 1, args.cpu_sample_s / max(per_step, 1e-6))))
    for s in sims:
        s.run(k)
    wall = time.perf_counter() - t0
    yrs = float(np.sum(np.array([s.T for s in sims]) - T0)) / YEAR
    return {"value": yrs / (wall / 3600.0), "unit": "sim-years/hour", "cores": nth, "kind": "port",
            "sample": "first %d steps of the timed window, %d instances, FP64 CPU oracle (C++ restatement of "
                      "the reference algorithm)" % (k + 1, R), "ms_per_step": wall / (k + 1) * 1e3}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.lib()
    sysd, draws = workload(args)
    N, R = sysd["N"], args.inst
    rec = sysd["records"]
    cols = dict(cx=rec[:, 0], cy=rec[:, 1], cz=rec[:, 2], ls=rec[:, 3], ld=rec[:, 4], strike=rec[:, 5],
                dip=rec[:, 6], rake=rec[:, 7])
    nth = os.cpu_count()
    Ks, Kn = oracle.assemble_rect(cols, cols, sysd["G"], sysd["nu"], nthreads=nth)
    kdiag = np.diag(Ks).copy()
    ext = ext_ramp(sysd)
    # bounded sample: the first `ref_instances` ensemble members (instances are
    # independent, so the ensemble rate is their summed simulated time over
    # their summed wall time)
    nr = max(1, min(R, args.ref_instances))
    sims = []
    shared = None
    for r in range(nr):
        p = problem(sysd, {k: v[r * N:(r + 1) * N] for k, v in draws.items()}, kdiag, 1)
        p.update(ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
        s = oracle.Simulation(p, ("dense", Ks, Kn) if shared is None else ("shared", shared), nthreads=nth)
        shared = s if shared is None else shared
        sims.append(s)
    del Ks, Kn
    for s in sims:
        s.run(args.warmup)
    T0 = np.array([s.T for s in sims])
    t0 = time.perf_counter()
    for s in sims:
        s.run(args.steps)
    wall = time.perf_counter() - t0
    yrs = float(np.sum(np.array([s.T for s in sims]) - T0)) / YEAR
    value = yrs / (wall / 3600.0)
    R = nr
    line = {"impl": "reference",
            "metric": "ensemble sim-years/hour, mixed-prec vs FP64 on GPU at <=1e-6 rel slip error",
            "value": value, "unit": "sim-years/hour", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded fault network)",
            "config": {"workload": "fault network, %d faults seed %d, %d rectangular patches, %d friction draws "
                                   "(ensemble), external stressing 0.01 MPa/yr" % (args.faults, args.seed, N, R),
                       "patches": N, "instances": R, "parallelism": "cpu-threads"},
            "cpu_baseline": {"value": value, "unit": "sim-years/hour", "cores": nth, "kind": "port",
                             "sample": "the whole window (%d warm-up + %d timed steps) of %d of the %d ensemble "
                                       "members, FP64 C++ restatement of the reference algorithm (Julia is not "
                                       "available)" % (args.warmup, args.steps, R, args.inst)},
            "e2e": {"value": value, "unit": "sim-years/hour", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def ensemble_geometries(n_geo, seed=11):
    """Geometries drawn as the network (strike, dip, lengths, depths, friction)
    with 3-40 faults each; the patch size is set per geometry so that it holds
    800-6,000 patches (drawn log-uniformly)."""
    from qdfn import synth
    rng = np.random.default_rng(seed)
    out = []
    for g in range(n_geo):
        nf = int(rng.integers(3, 41))
        target = float(np.exp(rng.uniform(np.log(800), np.log(6000))))
        probe = synth.fault_network(seed=1000 + g, n_faults=nf, patch=200.0)
        patch = 200.0 * np.sqrt(probe["N"] / target)
        sysd = synth.fault_network(seed=1000 + g, n_faults=nf, patch=float(patch))
        out.append(sysd)
    return out


def _member_sample(sizes, k):
    """k member indices at evenly spaced size quantiles (smallest to largest),
    so that a bounded CPU sample spans the ensemble's size range."""
    order = np.argsort(sizes, kind="stable")
    pick = sorted(set(int(order[int(round(q * (len(order) - 1)))]) for q in np.linspace(0.0, 1.0, k)))
    return pick


def _snapshot(ens):
    return [[sim.state(r) for r in range(sim.n_inst)] for sim in ens.members]


def _restore(ens, snap):
    for sim, sts in zip(ens.members, snap):
        for r, st in enumerate(sts):
            sim.set_state(r, st)


def _ens_slip_err(a, b):
    """Per-instance relative slip error max|D_a - D_b| / max|D_b|, a vs b."""
    out = []
    for sa, sb in zip(a.members, b.members):
        for r in range(sa.n_inst):
            da, db = sa.state(r)["D"], sb.state(r)["D"]
            out.append(float(np.max(np.abs(da - db)) / max(np.max(np.abs(db)), 1e-300)))
    return np.asarray(out)


def fp64_peak_tflops(dev):
    """FP64 matrix-multiply throughput of this GPU through the vendor library
    (torch.matmul on float64, 4096^3, best of 3) -- the measured FP64 peak the
    FP64-bound kernels are compared with."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best / 1e3) / 1e12


def profiled(name):
    """A committed ncu summary (profiles/<name>.json) or None."""
    p = os.path.join(ROOT, "profiles", name + ".json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return None
    return None


def build_ensemble(args, dev, rank=0):
    """The C4 ensemble: geometries with 3-40 faults and 800-6,000 patches,
    each with `inst` friction draws; FP64 stiffness assembled on the GPU.
    Returns the member dicts (device FP64 K), per-geometry host data and the
    assembly time."""
    import torch
    from qdfn import assemble, synth
    geos = ensemble_geometries(args.geometries, seed=11 + 1000 * rank)
    members, info = [], []
    asm_ms, pairs = 0.0, 0
    for g, sysd in enumerate(geos):
        N = sysd["N"]
        rec = torch.tensor(sysd["records"], dtype=torch.float64, device=dev)
        Ks = torch.empty((N, N), dtype=torch.float64, device=dev)
        Kn = torch.empty((N, N), dtype=torch.float64, device=dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        assemble.assemble_rect_dev(rec, rec, sysd["G"], sysd["nu"], Ks, Kn, layout="col")
        e1.record()
        torch.cuda.synchronize()
        asm_ms += e0.elapsed_time(e1)
        pairs += N * N
        kdiag = torch.diagonal(Ks).cpu().numpy()
        draws = synth.friction_draws(sysd, args.inst, seed=g + 1)
        prob = synth.problem_dict(sysd, kdiag, n_inst=args.inst, draws=draws)
        ext = synth.external_ramp(N, sysd["stressing_rate"], 1e12)
        members.append(dict(problem=prob, n_inst=args.inst, Ks=Ks, Kn=Kn, ext=ext))
        info.append(dict(sysd=sysd, draws=draws, kdiag=kdiag, ext=ext, N=N))
    return members, info, asm_ms, pairs


def _oracle_member(oracle, info_g, inst, Ks, Kn, nthreads):
    N = info_g["N"]
    p = problem(info_g["sysd"], {k: v[inst * N:(inst + 1) * N] for k, v in info_g["draws"].items()},
                info_g["kdiag"], 1)
    ext = info_g["ext"]
    p.update(ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
    return oracle.Simulation(p, ("dense", Ks, Kn), nthreads=nthreads)


def ensemble_cpu_sample(args, info, hostK, start, budget_s):
    """FP64 CPU oracle (all host threads) on instance 0 of the sampled members,
    each from its state at the timed window's start, for a share of
    `budget_s`; sim-years/hour = their summed simulated time over their summed
    wall time."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    nth = os.cpu_count()
    yrs, wall, done = 0.0, 0.0, []
    for g, (Ks, Kn) in hostK.items():
        s = _oracle_member(oracle, info[g], 0, Ks, Kn, nth)
        st = start[g][0]
        for k in ("V", "D", "theta", "friction", "accel", "sigma_old"):
            s.state[k][:] = st[k]
        s.set_scalars(st["T"], st["dt"], st["step"])
        t0 = time.perf_counter()
        s.run(1)
        one = time.perf_counter() - t0
        k = int(max(1, min(args.steps - 1, (budget_s / len(hostK)) / max(one, 1e-6))))
        s.run(k)
        w = time.perf_counter() - t0
        yrs += (s.T - st["T"]) / YEAR
        wall += w
        done.append((g, info[g]["N"], k + 1))
    return {"value": yrs / (wall / 3600.0), "unit": "sim-years/hour", "cores": nth, "kind": "port",
            "sample": "instance 0 of members %s (%s patches) for %s steps from the timed window's start, FP64 "
                      "CPU oracle (C++ restatement of the reference algorithm), all host threads"
                      % ([d[0] for d in done], [d[1] for d in done], [d[2] for d in done]),
            "wall_s": wall}


def plain_fp64_sample(args, info, plainK, start, ens, stream):
    """The plain FP64 GPU path -- the drop-in `main` as a user runs it, one
    instance per context and launch, FP64 operator, every SM -- on one draw of
    each sampled member (draw g mod R of member g), each from its state at the
    timed window's start over the same K steps.  The sample spans the members'
    size quantiles, so the ensemble's plain-path rate is estimated as the
    sample's summed simulated years over its summed device time."""
    import torch
    from qdfn import simulate
    yrs, ms_tot, rows = 0.0, 0.0, []
    for g, (Ks, Kn) in plainK.items():
        N = info[g]["N"]
        r = g % args.inst
        p = problem(info[g]["sysd"], {k: v[r * N:(r + 1) * N] for k, v in info[g]["draws"].items()},
                    info[g]["kdiag"], 1)
        sim = simulate.Simulation(p)
        sim.set_dense_device(Ks, Kn, "fp64", layout="col")
        ext = info[g]["ext"]
        sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
        st = start[g][r]
        sim.set_state(0, st)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.run_async(args.steps, stream=stream.cuda_stream, timeout_s=TIMEOUT)
        e1.record(stream)
        torch.cuda.synchronize()
        sim.sync()
        ms = e0.elapsed_time(e1)
        y = (sim.state(0)["T"] - st["T"]) / YEAR
        ym = (ens.members[g].state(r)["T"] - st["T"]) / YEAR   # the mixed ensemble's run of the same instance
        sim.close()
        yrs += y
        ms_tot += ms
        rows.append({"member": g, "patches": N, "draw": r, "ms_per_step": ms / args.steps, "sim_years": y,
                     "mixed_sim_years": ym})
    return {"value": yrs / (ms_tot / 1e3 / 3600.0), "unit": "sim-years/hour", "instances_sampled": len(rows),
            "method": "one draw of each of %d members at size quantiles, each alone on the GPU (FP64 operator, "
                      "one instance per launch) over the timed window's K steps; rate = summed simulated years "
                      "over summed device time" % len(rows),
            "samples": rows}


def run_ensemble(args):
    """C4, the headline: 64 fault networks of uneven size x 4 friction draws
    (256 instances) advanced by ONE persistent launch (qdfn_ensemble_*),
    operator in FP32 with FP64 state; beside it the same ensemble with the
    FP64 operator (the plain FP64 GPU path), the accuracy horizon of the mixed
    run against it, the end-to-end rate through the C ABI with host buffers,
    and the FP64 CPU oracle on a sample of the same members."""
    import torch
    from qdfn import ensemble
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    members, info, asm_ms, pairs = build_ensemble(args, dev, rank)
    sizes = [g["N"] for g in info]
    R = args.inst
    sample = _member_sample(sizes, args.cpu_members)
    hostK = {}
    if rank == 0 and not args.no_cpu:
        for g in sample:   # (src, recv) buffers: K[recv, src] is their transpose
            hostK[g] = (members[g]["Ks"].cpu().numpy().T, members[g]["Kn"].cpu().numpy().T)
    ens = ensemble.Ensemble(members, precision=args.precision)
    ens64 = None if args.no_fp64 else ensemble.Ensemble(members, precision="fp64")
    plain_sample = [] if (args.no_fp64 or args.plain_members <= 0) else _member_sample(sizes, args.plain_members)
    plainK = {g: (members[g]["Ks"], members[g]["Kn"]) for g in plain_sample}
    del members
    torch.cuda.empty_cache()
    s0 = _snapshot(ens)

    # ---- accuracy horizon: mixed vs FP64 from t = 0, every 100 steps.  A
    # member counts as interseismic until its FP64 run first has a patch past
    # twice the starting slip rate (at a check) or on the high-velocity
    # solver; a nucleation's runaway amplifies any perturbation (a 1e-15
    # perturbation of the FP64 operator alone grows to ~1e-7 through an
    # event), so the 1e-6 contract is stated over each member's interseismic
    # horizon.
    horizon = None
    if ens64 is not None:
        total = min(args.warmup + args.steps, args.horizon)
        errs, done = [], 0
        hi0 = [sim.counters()["highv_solves"] for sim in ens64.members]
        v0 = [max(float(np.max(st["V"])) for st in sts) for sts in s0]
        pre = np.ones(len(ens64.members), dtype=bool)
        while done < total:
            n = min(100, total - done)
            ens.run(n, timeout_s=TIMEOUT)
            ens64.run(n, timeout_s=TIMEOUT)
            done += n
            e = _ens_slip_err(ens, ens64).reshape(len(ens.members), R)
            hi = [sim.counters()["highv_solves"] for sim in ens64.members]
            pre &= np.array([h == h0 for h, h0 in zip(hi, hi0)])
            pre &= np.array([max(float(np.max(sim.state(r)["V"])) for r in range(sim.n_inst)) <= 2 * v0[m]
                             for m, sim in enumerate(ens64.members)])
            ep = e[pre]
            errs.append((done, float(e.max()), float(np.median(e)), int(pre.sum() * R),
                         float(ep.max()) if ep.size else None))
        ok = [st for st, _, _, npre, mp in errs if npre > 0 and mp <= 1e-6]
        bad = [st for st, _, _, npre, mp in errs if npre > 0 and mp > 1e-6]
        horizon = {"checked_every": 100, "instances": int(len(sizes) * R), "against": "FP64 GPU ensemble",
                   "interseismic_max_rel_slip_err": max((mp for *_, mp in errs if mp is not None), default=None),
                   "interseismic_all_within_1e-6": not bad,
                   "last_step_with_interseismic_instances": max(ok + bad) if ok + bad else None,
                   "at_step": {str(st): {"max_all": mx, "median_all": md, "interseismic_instances": npre,
                                         "max_interseismic": mp} for st, mx, md, npre, mp in errs}}
        _restore(ens, s0)
        _restore(ens64, s0)

    # ---- warm-up with the autotuner (SM shares re-divided by measured member time)
    shares0 = [int(b) for b in ens.blocks]
    ens.autotune(args.warmup, rounds=3, timeout_s=TIMEOUT)
    y0 = ens.sim_years()
    start = _snapshot(ens)

    # ---- timed: one persistent launch over K steps of every member
    clocks = ClockSampler(local)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    cnt0 = [sim.counters() for sim in ens.members]

    def chunked(e):
        """K steps as launches of `rebalance_every` steps with the autotuner's
        re-division of the SMs between them (a member that enters an event
        gets more SMs for its slow steps); CUDA events bracket all of it, host
        gaps included.  Returns (ms, launches)."""
        per = args.rebalance_every if args.rebalance_every > 0 else args.steps
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        done, nl = 0, 0
        while done < args.steps:
            n = min(per, args.steps - done)
            e.run_async(n, timeout_s=TIMEOUT, stream=stream.cuda_stream)
            nl += 1
            done += n
            if done < args.steps:
                e.sync()
                e.balance()
        g1.record(stream)
        torch.cuda.synchronize()
        e.sync()
        return g0.elapsed_time(g1), nl

    ms, nlaunch = chunked(ens)
    clk = clocks.stop()
    if ws > 1:
        ms = max_over_ranks(ms, dev)
        torch.distributed.barrier()
    yrs = float(np.sum(ens.sim_years() - y0))
    yrs_all = sum_over_ranks(yrs, dev) if ws > 1 else yrs
    value = yrs_all / (ms / 1e3 / 3600.0)
    steps_done = [sim.state(r)["step"] - start[m][r]["step"] for m, sim in enumerate(ens.members)
                  for r in range(sim.n_inst)]

    # ---- roofline of the persistent kernel (the one long launch of the window)
    esz = {"fp32": 4, "bf16x2": 4, "fp64": 8}[args.precision]
    mat_bytes = sum(2 * n * n * esz for n in sizes)
    vec_bytes = sum(R * n * 8 * 14 for n in sizes)
    alg_bytes = args.steps * (mat_bytes + vec_bytes)
    achieved = alg_bytes / (ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    prof = profiled("k_sim_members_c4_fp32")
    traffic = None
    if prof and prof.get("instances") == len(sizes) * R and prof.get("total_patches") == sum(sizes):
        traffic = float(prof["dram_bytes_per_step"]) * args.steps
    elif prof and prof.get("traffic_over_algorithmic"):
        # captured on a smaller ensemble of the same generator: traffic scales
        # with the members' algorithmic bytes
        traffic = float(prof["traffic_over_algorithmic"]) * alg_bytes
    cnt = [sim.counters() for sim in ens.members]
    solves = sum(c1["lowv_solves"] + c1["highv_solves"] - c0["lowv_solves"] - c0["highv_solves"]
                 for c0, c1 in zip(cnt0, cnt))
    fp64_tf = fp64_peak_tflops(dev) if rank == 0 else None
    # the unit the ensemble is bound by: FP64 instructions of the friction
    # solves per second (the committed capture's instructions per patch solve
    # x the window's solves per second) against the measured FP64 rate (one
    # DFMA per two flops of the FP64 GEMM)
    fp64_pipe = None
    if prof and prof.get("fp64_warp_inst_per_patch_solve") and fp64_tf:
        inst = solves / max(ms / 1e3, 1e-9) * 32.0 * float(prof["fp64_warp_inst_per_patch_solve"])
        fp64_pipe = {"achieved": inst / 1e12, "peak": fp64_tf / 2.0, "unit": "T FP64 lane-instructions/s",
                     "frac": inst / 1e12 / (fp64_tf / 2.0),
                     "note": "patch solves/s x %.1f FP64 warp instructions per solve (ncu, "
                             "profiles/k_sim_members_c4_fp32.md) x 32 lanes, against half the measured FP64 "
                             "GEMM flop rate; ncu: FP64 pipe %.1f %% busy over the captured launch"
                             % (float(prof["fp64_warp_inst_per_patch_solve"]), float(prof.get("fp64_pipe_active_pct", 0)))}

    def fill_window(e, snap):
        """The same window in fill mode: members that have taken K steps keep
        stepping until every member has (no SM idles); sim-years/hour of all
        steps taken.  The ensemble is left where the window began."""
        after = _snapshot(e)
        _restore(e, snap)
        e.set_fill(True)
        st0 = e.steps()
        z0 = e.sim_years()
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        e.run_async(args.steps, timeout_s=TIMEOUT, stream=stream.cuda_stream)
        g1.record(stream)
        torch.cuda.synchronize()
        e.sync()
        e.set_fill(False)
        fms = g0.elapsed_time(g1)
        fy = float(np.sum(e.sim_years() - z0))
        taken = e.steps() - st0
        _restore(e, after)
        return {"value": fy / (fms / 1e3 / 3600.0), "unit": "sim-years/hour", "ms": fms,
                "steps_per_instance": [int(taken.min()), int(taken.max())]}

    fill = fill_window(ens, start) if args.fill else None

    # ---- FP64 GPU path on the same ensemble and window
    fp64 = None
    if ens64 is not None:
        ens64.autotune(args.warmup, rounds=3, timeout_s=TIMEOUT)
        start64 = _snapshot(ens64)
        z0 = ens64.sim_years()
        torch.cuda.synchronize()
        ms64, _ = chunked(ens64)
        yrs64 = float(np.sum(ens64.sim_years() - z0))
        fill64 = fill_window(ens64, start64) if args.fill else None
        # the FP64 operator products are FP64-FMA bound: 2 matrices x R draws
        # x 2 flops per stored entry and step
        fl64 = args.steps * sum(2 * n * n * R * 2 for n in sizes)
        fp64 = {"value": yrs64 / (ms64 / 1e3 / 3600.0), "unit": "sim-years/hour", "ms_per_step": ms64 / args.steps,
                "instances": int(len(sizes) * R),
                "mixed_over_fp64": (yrs / (ms / 3.6e6)) / (yrs64 / (ms64 / 3.6e6)),
                "fill_mode": fill64,
                "mixed_over_fp64_fill_mode": (fill["value"] / fill64["value"]) if fill and fill64 else None,
                "roofline": {"bound": "fp64", "achieved": fl64 / (ms64 / 1e3) / 1e12, "unit": "TFLOP/s",
                             "peak": fp64_tf, "frac": (fl64 / (ms64 / 1e3) / 1e12) / fp64_tf if fp64_tf else None,
                             "note": "operator FP64 FMAs (2 matrices x R x 2 flop per entry and step) over the "
                                     "launch; peak = torch.matmul float64 4096^3 measured in this run"}}
        ens64.close()
        ens64 = None
        torch.cuda.empty_cache()
        if plain_sample:
            fp64["plain_path"] = plain_fp64_sample(args, info, plainK, start, ens, stream)
            fp64["mixed_over_plain_fp64"] = value / fp64["plain_path"]["value"]
    plainK = None

    # ---- e2e through the C ABI with host buffers: every step the whole
    # ensemble's state goes up from pinned host memory in one copy
    # (qdfn_ensemble_set_state_all), one ensemble step runs (one launch), the
    # state comes back in one copy (qdfn_ensemble_get_state_all, which also
    # completes the run: one synchronisation per step)
    e2e = None
    if not args.no_e2e:
        _restore(ens, start)
        buf = torch.empty(ens.state_words(), dtype=torch.float64).pin_memory()
        ens.pack_states(start, out=buf)
        sptr = stream.cuda_stream
        nbytes = ens.state_words() * 8
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.steps):
            ens.set_state_all(buf, stream=sptr)
            ens.run_async(1, timeout_s=TIMEOUT, stream=sptr)
            ens.get_state_all(buf, stream=sptr, wait=True)
            if args.rebalance_every > 0 and (k + 1) % args.rebalance_every == 0 and k + 1 < args.steps:
                ens.balance()
        t_e2e = time.perf_counter() - t0
        if ws > 1:
            t_e2e = max_over_ranks(t_e2e, dev)
        fin = ens.unpack_states(buf)
        ye = sum(fin[m][r]["T"] - start[m][r]["T"] for m, sim in enumerate(ens.members)
                 for r in range(sim.n_inst)) / YEAR
        if ws > 1:
            ye = sum_over_ranks(ye, dev)
        e2e = {"value": ye / (t_e2e / 3600.0), "unit": "sim-years/hour", "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes,
               "note": "one ensemble step per launch, the whole state up and down every step in one copy each "
                       "way (no step streams ahead across a launch boundary); the SMs re-divided every "
                       "rebalance_every steps as in the device-resident window"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = ensemble_cpu_sample(args, info, hostK, start, args.cpu_sample_s)

    if rank == 0:
        tot = sum(sizes)
        line = {
            "metric": "ensemble sim-years/hour, mixed-prec vs FP64 on GPU at <=1e-6 rel slip error",
            "value": value, "unit": "sim-years/hour", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32-operator/fp64-state" if args.precision != "fp64" else "fp64",
            "data": "synthetic (seeded fault networks with the reference's fault-network distributions; the "
                    "reference ships no benchmark data)",
            "config": {"workload": "C4 batched ensemble: %d fault networks of %d-%d patches (%d total, 3-40 faults "
                                   "each) x %d friction draws = %d instances, one persistent launch, operator %s"
                                   % (len(sizes), min(sizes), max(sizes), tot, R, len(sizes) * R, args.precision),
                       "instances": len(sizes) * R, "geometries": len(sizes), "total_patches": tot,
                       "precision": args.precision, "parallelism": "replicas",
                       "l2": "operator %.2f GB per ensemble step > 129 MB L2 (no flush needed)" % (mat_bytes / 1e9),
                       "sm_shares_initial": shares0, "sm_shares_tuned": [int(b) for b in ens.blocks],
                       "launches": nlaunch, "rebalance_every": args.rebalance_every,
                       "steps_per_instance": [int(min(steps_done)), int(max(steps_done))],
                       "sim_years_in_window": yrs_all},
            "gpu_launches": 3 * nlaunch,
            "e2e": e2e,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "note": "k_sim_members (one launch, every member's K steps), algorithmic bytes = K x "
                                 "sum over members (2 N^2 x %d B operator + state vectors); peak %s. The small "
                                 "members are bound by their FP64 friction solves, not by HBM: %.3g patch solves "
                                 "per second. traffic = DRAM bytes of the K-step window: the algorithmic bytes x "
                                 "the DRAM/algorithmic ratio of the committed ncu capture of a smaller ensemble of "
                                 "the same generator (profiles/k_sim_members_c4_fp32.md)"
                                 % (esz, peak_kind, solves / max(ms / 1e3, 1e-9))},
            "fp64_pipe": fp64_pipe,
            "cpu_baseline": cpu,
            "fp64_gpu": fp64,
            "fill_mode": dict(fill, note="the same window with members that have taken K steps stepping on "
                                         "until every member has (qdfn_ensemble_set_fill): no SM idles while the "
                                         "slowest member finishes") if fill else None,
            "accuracy_horizon": horizon,
            "assembly": {"pairs": pairs, "ms": asm_ms, "pairs_per_s": pairs / (asm_ms / 1e3),
                         "fp64_peak_tflops_measured": fp64_tf},
            "clocks": clk,
        }
        asm_prof = profiled("k_assemble_rect_fp64")
        if asm_prof and fp64_tf:
            fl = float(asm_prof["fp64_flop_per_pair"]) * pairs / (asm_ms / 1e3) / 1e12
            line["assembly"].update(fp64_flop_per_pair=asm_prof["fp64_flop_per_pair"], fp64_tflops=fl,
                                    fp64_frac=fl / fp64_tf)
        print(json.dumps(line))
    ens.close()
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def run_reference_ensemble(args):
    """Reference arm for C4: the FP64 CPU oracle (the reference's algorithm
    restated in C++; the Julia reference itself cannot run here) on instance 0
    of sampled members of the same ensemble (same seeds and draws), over the
    whole window, all host threads."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from qdfn import synth
    geos = ensemble_geometries(args.geometries)
    sizes = [g["N"] for g in geos]
    nth = os.cpu_count()
    yrs, wall, done = 0.0, 0.0, []
    for g in _member_sample(sizes, args.cpu_members):
        sysd = geos[g]
        rec = sysd["records"]
        cols = dict(cx=rec[:, 0], cy=rec[:, 1], cz=rec[:, 2], ls=rec[:, 3], ld=rec[:, 4], strike=rec[:, 5],
                    dip=rec[:, 6], rake=rec[:, 7])
        Ks, Kn = oracle.assemble_rect(cols, cols, sysd["G"], sysd["nu"], nthreads=nth)
        kdiag = np.diag(Ks).copy()
        draws = synth.friction_draws(sysd, args.inst, seed=g + 1)
        ext = synth.external_ramp(sysd["N"], sysd["stressing_rate"], 1e12)
        s = _oracle_member(oracle, dict(sysd=sysd, draws=draws, kdiag=kdiag, ext=ext, N=sysd["N"]), 0, Ks, Kn, nth)
        del Ks, Kn
        s.run(args.warmup)
        T0 = s.T
        t0 = time.perf_counter()
        s.run(args.steps)
        wall += time.perf_counter() - t0
        yrs += (s.T - T0) / YEAR
        done.append((g, sysd["N"]))
    value = yrs / (wall / 3600.0)
    sample = ("instance 0 of members %s (%s patches) of the C4 ensemble (same seeds and draws), the whole window "
              "(%d warm-up + %d timed steps), FP64 C++ restatement of the reference algorithm (Julia is not "
              "available), all host threads" % ([d[0] for d in done], [d[1] for d in done], args.warmup, args.steps))
    line = {"impl": "reference",
            "metric": "ensemble sim-years/hour, mixed-prec vs FP64 on GPU at <=1e-6 rel slip error",
            "value": value, "unit": "sim-years/hour", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": wall / args.steps / len(done) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded fault networks)",
            "config": {"workload": "C4 batched ensemble: %d fault networks of %d-%d patches x %d friction draws "
                                   "(sampled members, see cpu_baseline.sample)"
                                   % (len(sizes), min(sizes), max(sizes), args.inst),
                       "instances": len(sizes) * args.inst, "parallelism": "cpu-threads"},
            "cpu_baseline": {"value": value, "unit": "sim-years/hour", "cores": nth, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "sim-years/hour", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_tri_h(args):
    """C3: 5 curved faults meshed into ~50,000 triangles (TDstressHS), H-matrix
    operator (cluster-tree leaf 64, admissibility eta = 2, ACA 1e-6), low-rank
    and near-field blocks stored in FP32 (or --precision fp64), one instance,
    main_H semantics.  value = simulated years per hour over K steps of one
    persistent launch; roofline = the stored block bytes streamed per step."""
    import torch
    from qdfn import geometry, hmatrix, simulate, synth
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    net = synth.curved_fault_network(seed=args.seed, edge=args.tri_edge)
    seg = net["seg"]
    P1, P2, P3, un, _, _, us = geometry.rot_verts_unit_vectors_abi(seg, seg[:, 9])
    cen = (P1 + P2 + P3) / 3
    t0 = time.perf_counter()
    H, perm = hmatrix.build_tri(P1, P2, P3, seg[:, 9], cen, un, us, net["G"], net["nu"], leaf=64, eta=2.0, tol=1e-6,
                                tree=args.tree)
    build_s = time.perf_counter() - t0
    N = net["N"]
    kdiag = np.zeros(N)
    for b, (s0, s1, r0, r1) in enumerate(H.ranges):
        if s0 == r0 and s1 == r1 and H.dense_s[b] is not None:
            kdiag[r0:r1 + 1] = np.diag(H.dense_s[b])
    sysd = {k: (v[perm] if isinstance(v, np.ndarray) and v.shape == (N,) else v) for k, v in net.items()}
    prob = synth.problem_dict(sysd, kdiag)
    prob["interp_at_told"] = 1
    ext = synth.external_ramp(N, net["stressing_rate"], 1e12)
    esz = {"fp32": 4, "bf16x2": 4, "fp64": 8}[args.precision]
    stored = H.stored_entries()
    prec = "fp64" if args.precision == "fp64" else "fp32"

    def make(prec):
        sim = simulate.Simulation(prob)
        hmatrix.set_hmatrix(sim, H, prec)
        sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
        return sim

    def timed(sim):
        sim.run(args.warmup, timeout_s=TIMEOUT)
        T0 = sim.state(0)["T"]
        c0 = sim.counters()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.run_async(args.steps, stream=stream.cuda_stream, timeout_s=TIMEOUT)
        e1.record(stream)
        torch.cuda.synchronize()
        sim.sync()
        ms = e0.elapsed_time(e1)
        c1 = sim.counters()
        ph = {k: (c1[k] - c0[k]) / 1e6 / args.steps for k in ("ns_control", "ns_operator", "ns_solve", "ns_rotate",
                                                              "ns_solve_own", "ns_solve_wait")}
        ph["solve_passes_per_step"] = (c1["solve_passes"] - c0["solve_passes"]) / args.steps
        return ms, (sim.state(0)["T"] - T0) / YEAR, ph

    sim = make(prec)
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    ms, yrs, phases = timed(sim)
    clk = clocks.stop()
    sim.close()
    fp64 = None
    if not args.no_fp64 and prec != "fp64":
        s64 = make("fp64")
        ms64, yrs64, _ = timed(s64)
        s64.close()
        fp64 = {"value": yrs64 / (ms64 / 1e3 / 3600.0), "ms_per_step": ms64 / args.steps,
                "mixed_over_fp64": (yrs / ms) / (yrs64 / ms64)}
    peak, peak_kind = measured_peaks()
    alg = args.steps * stored * esz
    achieved = alg / (ms / 1e3) / 1e9
    prof = profiled("k_sim_hmat_c3_fp32") if prec == "fp32" else None
    traffic = float(prof["traffic_over_algorithmic"]) * alg if prof else None
    nlr = sum(1 for U in H.U_s + H.U_n if U is not None)
    ranks = [U.shape[1] for U in H.U_s + H.U_n if U is not None]
    line = {"metric": "sim-years/hour, triangle-mesh network with H-matrix operator", "value": yrs / (ms / 1e3 / 3600.0),
            "unit": "sim-years/hour", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "%s-operator/fp64-state" % prec, "data": "synthetic (seeded curved fault meshes)",
            "config": {"workload": "C3: 5 curved faults, %d triangles (TDstressHS, edge %g m), H-matrix leaf 64, "
                                   "eta 2, ACA 1e-6, blocks %s" % (N, args.tri_edge, prec),
                       "patches": N, "blocks": int(H.nblocks), "low_rank_blocks": nlr,
                       "max_rank": int(max(ranks)) if ranks else 0, "mean_rank": float(np.mean(ranks)) if ranks else 0,
                       "stored_entries": int(stored), "compression_vs_dense": float(stored / (2.0 * N * N)),
                       "h_build_s": build_s, "tree": args.tree},
            "gpu_launches": 1,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic,
                         "note": "k_sim<H> persistent kernel, algorithmic bytes = K x stored block bytes "
                                 "(%d entries x %d B); peak %s; traffic = those bytes x the DRAM/algorithmic "
                                 "ratio of the committed ncu capture of a 12,500-triangle mesh of the same "
                                 "generator (profiles/k_sim_hmat_c3_fp32.md)" % (stored, esz, peak_kind)},
            "fp64_gpu": fp64, "clocks": clk,
            "phases_ms_per_step": {k.replace("ns_", ""): v for k, v in phases.items()}}
    print(json.dumps(line))


def run_adjoint(args):
    """C5: gradient of a trajectory loss with respect to every patch's a, b and
    Dc on the fault network (seed 2, 30 faults, 12,813 patches, one friction
    draw), operator in FP32 (--precision fp64 for the all-FP64 adjoint): the
    forward window of K steps (one step per launch, sqrt(K) checkpoints) and the
    reverse sweep through qdfn_adjoint_run.  Loss: squared misfit of the final
    slip against a run with 1 %-perturbed a, b, Dc.  Reports the wall time of
    forward + reverse against the plain forward (one persistent launch)."""
    import torch
    from qdfn import adjoint, assemble, simulate
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    sysd, _ = workload(args)
    N = sysd["N"]
    rec = torch.tensor(sysd["records"], dtype=torch.float64, device=dev)
    Ks = torch.empty((N, N), dtype=torch.float64, device=dev)
    Kn = torch.empty((N, N), dtype=torch.float64, device=dev)
    assemble.assemble_rect_dev(rec, rec, sysd["G"], sysd["nu"], Ks, Kn, layout="col")
    kdiag = torch.diagonal(Ks).cpu().numpy()
    prob = problem(sysd, None, kdiag, 1)
    ext = ext_ramp(sysd)
    rng = np.random.default_rng(11)
    pert = dict(prob)
    for k in ("a", "b", "Dc"):
        pert[k] = prob[k] * (1 + 0.01 * rng.standard_normal(N))

    def make(p):
        sim = simulate.Simulation(p)
        sim.set_dense_device(Ks, Kn, args.precision, layout="col")
        sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
        return sim

    tgt = make(pert)
    tgt.run(args.steps, timeout_s=TIMEOUT)
    Dstar = tgt.state(0)["D"]
    tgt.close()
    fwd = make(prob)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fwd.run(args.steps, timeout_s=TIMEOUT)
    t_fwd = time.perf_counter() - t0
    D = fwd.state(0)["D"]
    yrs = fwd.state(0)["T"] / YEAR
    fwd.close()
    sim = make(prob)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g = adjoint.gradient(sim, args.steps, dL_dD_final=2 * (D - Dstar), timeout_s=TIMEOUT)
    t_adj = time.perf_counter() - t0
    sim.close()
    line = {"metric": "adjoint wall time (forward + reverse), fault network", "value": t_adj, "unit": "s",
            "n_gpus": 1, "steps": args.steps, "warmup": 0, "ms_per_step": t_adj / args.steps * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "%s-operator/fp64-state" % args.precision, "data": "synthetic (seeded fault network)",
            "config": {"workload": "C5: fault network seed %d, %d rectangular patches, %d adaptive steps, gradients "
                                   "of final-slip misfit w.r.t. a, b, Dc (every patch)" % (args.seed, N, args.steps),
                       "patches": N, "checkpoints": int(np.ceil(np.sqrt(args.steps)))},
            "forward_only_s": t_fwd, "adjoint_over_forward": t_adj / t_fwd, "sim_years_in_window": yrs,
            "gradient_norms": {k: float(np.linalg.norm(v)) for k, v in g.items()}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference_ensemble(args) if args.workload == "ensemble" else run_reference(args)
    elif args.workload == "ensemble":
        run_ensemble(args)
    elif args.workload == "tri_h":
        run_tri_h(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
