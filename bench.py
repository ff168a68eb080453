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
    ap.add_argument("--workload", default="network", choices=["network", "ensemble"],
                    help="network: the 30-fault network (default); ensemble: 64 geometries of "
                         "800-6,000 patches x 4 friction draws advanced together")
    ap.add_argument("--geometries", type=int, default=64)
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


def run_ensemble(args):
    """Batched ensemble: every geometry with its friction draws is one
    context on a share of the SMs, all advanced together (qdfn.ensemble)."""
    import torch
    from qdfn import assemble, ensemble, synth
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    geos = ensemble_geometries(args.geometries)
    members = []
    for g, sysd in enumerate(geos):
        N = sysd["N"]
        rec = torch.tensor(sysd["records"], dtype=torch.float64, device=dev)
        Ks = torch.empty((N, N), dtype=torch.float64, device=dev)
        Kn = torch.empty((N, N), dtype=torch.float64, device=dev)
        assemble.assemble_rect_dev(rec, rec, sysd["G"], sysd["nu"], Ks, Kn, layout="col")
        kdiag = torch.diagonal(Ks).cpu().numpy()
        draws = synth.friction_draws(sysd, args.inst, seed=g + 1)
        prob = synth.problem_dict(sysd, kdiag, n_inst=args.inst, draws=draws)
        ext = synth.external_ramp(N, sysd["stressing_rate"], 1e12)
        members.append(dict(problem=prob, n_inst=args.inst, Ks=Ks, Kn=Kn, ext=ext))
    ens = ensemble.Ensemble(members, precision=args.precision)
    del members
    torch.cuda.empty_cache()
    ens.run(args.warmup, timeout_s=TIMEOUT)
    y0 = ens.sim_years()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    t0 = time.perf_counter()
    ens.run(args.steps, timeout_s=TIMEOUT)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    yrs = float(np.sum(ens.sim_years() - y0))
    sizes = [m.N for m in ens.members]
    line = {"metric": "ensemble sim-years/hour (batched geometries)", "value": yrs / (wall / 3600.0),
            "unit": "sim-years/hour", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": wall * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "%s-operator/fp64-state" % args.precision, "data": "synthetic",
            "config": {"workload": "%d geometries of %d-%d patches (%d total) x %d friction draws, one context "
                                   "per geometry on its share of the SMs, all advanced together"
                                   % (len(sizes), min(sizes), max(sizes), sum(sizes), args.inst),
                       "instances": len(sizes) * args.inst, "precision": args.precision,
                       "sm_shares": [int(b) for b in ens.blocks]},
            "gpu_launches": len(sizes), "clocks": clk,
            "note": "wall clock over all members' concurrent launches (each member takes its own adaptive steps)"}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "ensemble":
        run_ensemble(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
