"""Benchmark: cell-updates/s of the RK3 advance on one periodic box.

Workload (default): 128^3 cells + 4 ghost cells a side, FP64 plain form, the CNS_NoSpec
initial field with a seeded +-1e-3 perturbation of rho, u, v, w; a step is one full RK3
step (new_advance, cpu/advance.cpp:13-154) of that box.  The mixed FP32/FP64 form is timed on
the same box in the same run and its error against the FP64 result is reported.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank advances its own replica box on its own GPU (the box does
not shard: replicas only); the host-side barrier and the max over ranks go through
torch.distributed (gloo).  Rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic FP64 work of one cell-update (one cell, one full RK3 step) in the reference's
# formulation (each +, -, *, / one flop): 3 x (ctoprim 16 + hypterm 358 + diffterm 415)
# + RK combines 15 + 30 + 30 + Courant 8 = 2450.
FLOPS_PER_CELL_UPDATE = 2450
# Of that, per cell and launch: k_deriv does the nine first derivatives (9 x 12) and the
# dissipation terms of diffterm's energy component (24) = 132; k_assemble the rest of a stage.
FLOPS_DERIV = 132
FLOPS_ASSEMBLE_PER_STEP = FLOPS_PER_CELL_UPDATE - 3 * FLOPS_DERIV  # 2054 over 3 launches
# Compulsory HBM traffic of one cell-update with the FP64 state: stage 1 reads U^n and writes
# U^1 (80 B); stages 2 and 3 read U^(k), U^n and write U^(k+1) (120 B each).
BYTES_PER_CELL_UPDATE = 320


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--size", dest="n", type=int, default=128, help="cells per axis of the periodic box")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample length")
    p.add_argument("--case", choices=["fp64", "mixed", "e2e"], default=None,
                   help="profiling case: only upload + warmup + steps of one form (for ncu), then exit; "
                        "e2e: warmup + steps calls of cns_new_advance on a page-locked host array")
    p.add_argument("--kernel", choices=["ws", "tma", "direct"], default=None,
                   help="--case: the assembly kernel (default: the library's choice; ws is mixed-only)")
    p.add_argument("--workload", choices=["box", "batch", "mixed256", "serve", "cpu"], default="box",
                   help="box: the headline 128^3 line (default); batch: 256 uneven boxes; "
                        "mixed256: FP64 vs mixed at --size (use 256); serve: the request stream; "
                        "cpu: the CPU baseline table (the oracle port on the host cores)")
    p.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    p.add_argument("--boxes", type=int, default=256)
    p.add_argument("--rate", type=float, default=3.0, help="serve: requests per second")
    p.add_argument("--requests", type=int, default=48)
    p.add_argument("--budget-gb", type=float, default=120.0)
    p.add_argument("--big", type=int, default=512, help="serve: the single box run alone beside the stream")
    p.add_argument("--big-steps", type=int, default=3)
    return p.parse_args()


# ---- distributed plumbing (host side only) ---------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---- clocks -------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            out, _ = self.proc.communicate(timeout=10)
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def box_workload(n):
    """The name of the single-box workload, the same on both arms."""
    return f"periodic box {n}^3 + 4 ghosts, FP64 RK3 step, sinusoidal field with a 1e-3 perturbation (seed 1)"


def pinned_like(shape):
    """A pinned host float64 array when torch is importable (plumbing only), else pageable."""
    try:
        import torch
        t = torch.empty(shape, dtype=torch.float64, pin_memory=True)
        return t.numpy(), True, t
    except Exception:
        return np.empty(shape, dtype=np.float64), False, None


def measured_traffic(kernel: str, n: int):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, scaled by cells."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            t = json.load(f)
        per_cell = t[kernel]["dram_bytes_per_cell"]
        return per_cell * n ** 3, t[kernel].get("source")
    except Exception:
        return None, None


# ---- CPU baseline: the oracle (the reference's algorithm restated in C) on the host cores ----
def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the platform string)."""
    import platform
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def cpu_baseline(n: int, seconds: float):
    """The reference algorithm (the oracle port, the reference's cpu/ operation order) on the
    host cores: one single-threaded process per core, each advancing its own n^3 box, for about
    `seconds` (oracle_processes); beside it one core alone at 32^3 and n^3, and all cores as one
    OpenMP process on one box."""
    from cns_nospec_gb300 import initdata as I
    from oracle import oracle as O
    O.build(ref=os.path.isdir(O.REF_SRC))
    cores = os.cpu_count() or 1
    nproc = host_processes(n)
    value, steps, wall = oracle_processes(n, 100, 1, seconds, nproc)
    # one core, as the reference's own cpu/ path runs (its OpenMP pragmas are commented out)
    one = {}
    O.set_threads(1)
    for m, budget in ((32, 1.0), (n, 3.0)):
        V = I.initial_state(m, perturb=1e-3, seed=1)
        k, t1 = 0, time.perf_counter()
        while True:
            V, _ = O.advance(V, 1, I.box_dx(m), I.CFL, I.ETA, I.ALAM, which="port")
            k += 1
            e1 = time.perf_counter() - t1
            if e1 >= budget or k >= 50:
                break
        one[str(m)] = m ** 3 * k / e1
    threads = O.set_threads(cores)
    U = I.initial_state(n, perturb=1e-3, seed=1)
    k, t1 = 0, time.perf_counter()
    while True:
        U, _ = O.advance(U, 1, I.box_dx(n), I.CFL, I.ETA, I.ALAM, which="port")
        k += 1
        e1 = time.perf_counter() - t1
        if e1 >= 4.0 or k >= 20:
            break
    return {"value": value, "unit": "cell-updates/s", "cores": nproc, "cpu_model": cpu_model(), "kind": "port",
            "sample": f"{nproc} single-threaded processes, {steps} RK3 steps in all of their own {n}^3 boxes, "
                      f"{wall:.1f} s", "one_core_by_n": one,
            "openmp_one_process": {"value": n ** 3 * k / e1, "threads": threads, "steps": k}}


def _oracle_process(n, steps, warmup, seconds, which, barrier, out):
    """One single-threaded run of the reference algorithm (a child process of oracle_processes):
    `warmup` untimed steps, a barrier with the other processes, then up to `steps` timed steps or
    `seconds` of them.  Puts the steps done and the wall-clock start and end of the timed part."""
    from cns_nospec_gb300 import initdata as I
    from oracle import oracle as O
    O.set_threads(1)
    U = I.initial_state(n, perturb=1e-3, seed=1)
    dx = I.box_dx(n)
    for _ in range(warmup):
        U, _ = O.advance(U, 1, dx, I.CFL, I.ETA, I.ALAM, which=which)
    barrier.wait(timeout=600)
    k, t0 = 0, time.time()
    while k < steps:
        U, _ = O.advance(U, 1, dx, I.CFL, I.ETA, I.ALAM, which=which)
        k += 1
        if time.time() - t0 >= seconds:
            break
    out.put((k, t0, time.time()))


def host_processes(n: int) -> int:
    """Processes for oracle_processes: one per host core, but no more than a quarter of the
    host's memory holds (an n^3 oracle step needs about 25 doubles per ghost-inclusive cell)."""
    cores = os.cpu_count() or 1
    try:
        mem = os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")
    except (ValueError, OSError, AttributeError):
        return cores
    per = 25 * 8 * (n + 8) ** 3
    return max(1, min(cores, int(mem // 4 // per)))


def oracle_processes(n, steps, warmup, seconds, nproc, which="port"):
    """The reference algorithm on every host core the way its single-threaded cpu/ code uses
    them: `nproc` independent processes (spawned), each advancing its own copy of the n^3 box,
    their timed parts started together.  Throughput = all processes' cell-updates / (last end -
    first start)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    barrier, out = ctx.Barrier(nproc), ctx.Queue()
    procs = [ctx.Process(target=_oracle_process, args=(n, steps, warmup, seconds, which, barrier, out))
             for _ in range(nproc)]
    for p in procs:
        p.start()
    import queue
    res, t0 = [], time.time()
    try:
        while len(res) < nproc:
            try:
                res.append(out.get(timeout=5))
            except queue.Empty:
                if any(p.exitcode not in (None, 0) for p in procs) or time.time() - t0 > 900:
                    raise RuntimeError("an oracle process failed or did not finish")
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.terminate()
    done = sum(r[0] for r in res)
    wall = max(r[2] for r in res) - min(r[1] for r in res)
    return n ** 3 * done / wall, done, wall


def run_cpu_table(args):
    """The CPU baseline in full: the oracle port (the reference's cpu/ algorithm, same operation
    order) on one core at 32^3 (10 steps), 128^3 and 256^3 (3 steps); on all host cores as one
    OpenMP process; and as one single-threaded process per core, each advancing its own 128^3
    box (oracle_processes)."""
    from cns_nospec_gb300 import initdata as I
    from oracle import oracle as O
    O.build(ref=False)
    cores = os.cpu_count() or 1
    one = {}
    O.set_threads(1)
    for n, steps in ((32, 10), (128, 3), (256, 3)):
        U = I.initial_state(n, perturb=1e-3, seed=1)
        t0 = time.perf_counter()
        O.advance(U, steps, I.box_dx(n), I.CFL, I.ETA, I.ALAM, which="port")
        one[str(n)] = n ** 3 * steps / (time.perf_counter() - t0)
    threads = {}
    O.set_threads(cores)
    for n, steps in ((128, 10), (256, 3)):
        U = I.initial_state(n, perturb=1e-3, seed=1)
        t0 = time.perf_counter()
        O.advance(U, steps, I.box_dx(n), I.CFL, I.ETA, I.ALAM, which="port")
        threads[str(n)] = n ** 3 * steps / (time.perf_counter() - t0)
    agg, done, wall = oracle_processes(128, 3, 0, 1e9, host_processes(128))
    return {"workload": "CPU baseline: the oracle port of the reference's cpu/ path, sinusoidal field with a 1e-3 "
                        "perturbation (seed 1)", "unit": "cell-updates/s", "cores": cores, "cpu_model": cpu_model(),
            "one_core_by_n": one, "openmp_all_cores_by_n": threads,
            "processes_128": {"processes": host_processes(128), "steps_each": 3, "aggregate": agg, "wall_s": wall}}


def run_reference(args, dist):
    """--impl reference: the reference algorithm on the host cores, same workload.  Where the
    reference tree exists its own cpu/ objects run (oracle/_ref); elsewhere (the GPU machine, where
    it is absent and x86 objects do not travel) the oracle port, which gives the same bits.
    Its cpu/ path is single-threaded, so it uses the cores as one process per core, each
    advancing its own copy of the box (oracle_processes): `warmup` untimed steps, then `steps`
    timed steps, bounded to about a minute."""
    if dist.rank != 0:
        return None
    from oracle import oracle as O
    O.build(ref=os.path.isdir(O.REF_SRC))
    use_ref = O.have_ref() and os.path.isdir(O.REF_SRC)
    which = "ref" if use_ref else "port"
    n = args.n
    cores = host_processes(n)
    warm = min(args.warmup, 1)
    v, done, wall = oracle_processes(n, args.steps, warm, 60.0, cores, which=which)
    steps = max(1, done // cores)
    kind = "reference" if use_ref else "port"
    sample = f"{cores} single-threaded processes x {steps} RK3 steps of their own {n}^3 box, {wall:.1f} s"
    return {"metric": "cell-updates/s", "value": v, "unit": "cell-updates/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": steps, "warmup": warm, "ms_per_step": 1e3 * wall / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": box_workload(n), "n": n, "host_processes": cores},
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": cores, "cpu_model": cpu_model(), "kind": kind,
                             "sample": sample},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_ours(args, dist):
    import cns_nospec_gb300 as C
    from cns_nospec_gb300 import _lib as L
    from cns_nospec_gb300 import build as B
    from cns_nospec_gb300 import initdata as I
    B.build()
    lib = C.load()
    L.check(lib.cns_set_device(dist.local))
    n = args.n
    dx = I.box_dx(n)
    U0 = I.initial_state(n, perturb=1e-3, seed=1)

    fp64_peak = C._lib.C.c_double(0.0)
    L.check(lib.cns_measure_fp64_peak(C._lib.C.byref(fp64_peak)))
    fp64_peak = fp64_peak.value

    # ---- device-resident FP64 plain form: the headline value --------------------------------
    box = C.Box(n, dx, I.CFL, I.ETA, I.ALAM, precision=C.CNS_FP64)
    box.upload(U0)
    tile64, _, _ = box.autotune(trial_steps=2)  # state restored afterwards
    box.advance_timed(args.warmup)
    lib.cns_device_synchronize()
    dist.barrier()
    with ClockSampler(dist.local) as clk:
        lib.cns_device_synchronize()
        kms, klaunch, total_ms = box.advance_timed(args.steps)
        lib.cns_device_synchronize()
    dist.barrier()
    box.sync()
    t_max = dist.max(total_ms)
    cells = n ** 3
    value = dist.world * cells * args.steps / (t_max * 1e-3)
    U64 = box.download()
    box.close()

    # ---- mixed form on the same box ----------------------------------------------------------
    mbox = C.Box(n, dx, I.CFL, I.ETA, I.ALAM, precision=C.CNS_MIXED)
    mbox.upload(U0)
    tile32, kern32, _ = mbox.autotune(trial_steps=2)
    mbox.advance_timed(args.warmup)
    mms, _, mtotal = mbox.advance_timed(args.steps)
    mbox.sync()
    mbox.close()
    mixed_value = cells * args.steps / (mtotal * 1e-3)
    # error of the mixed form against FP64 after exactly 100 RK3 steps from the same state
    ends = {}
    for prec in (C.CNS_FP64, C.CNS_MIXED):
        eb = C.Box(n, dx, I.CFL, I.ETA, I.ALAM, precision=prec)
        eb.upload(U0)
        eb.advance(100)
        eb.sync()
        ends[prec] = eb.download()
        eb.close()
    mixed_err = I.normwise_error(ends[C.CNS_MIXED], ends[C.CNS_FP64])[0]
    del U64

    # ---- end to end through the reference-facing C ABI: host buffers, copies timed ----------
    h = C.read_configurations(n, dx, I.CFL, I.ETA, I.ALAM)
    Uh, pinned, _keep = pinned_like(U0.shape)
    Uh[...] = U0
    k_e2e = max(1, min(args.steps, 20))
    C.new_advance(Uh, None, None, None, None, h)  # warm (allocates the cached device state)
    Uh[...] = U0
    lib.cns_device_synchronize()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(k_e2e):
        C.new_advance(Uh, None, None, None, None, h)
    lib.cns_device_synchronize()
    e2e_s = dist.max(time.perf_counter() - t0)
    dist.barrier()
    e2e_value = dist.world * cells * k_e2e / e2e_s
    # bytes that cross the CPU-GPU link per call: in place (page-locked U) the interior goes in and
    # the interior plus the ghost images come out; staged, the whole array both ways
    flag = ctypes.c_int(0)
    L.check(lib.cns_host_in_place(ctypes.c_void_p(Uh.ctypes.data), ctypes.c_longlong(Uh.nbytes), ctypes.byref(flag)))
    in_place = bool(flag.value)
    h2d_bytes = n ** 3 * 5 * 8 if in_place else int(Uh.nbytes)
    d2h_bytes = int(Uh.nbytes)

    # ---- roofline of the dominant kernel ----------------------------------------------------
    names = L.KERNEL_NAMES
    dom = int(np.argmax(kms))
    dom_launch_ms = kms[dom] / max(klaunch[dom], 1)
    if names[dom] == "k_assemble":
        flops_launch = FLOPS_ASSEMBLE_PER_STEP / 3.0 * cells
    else:
        flops_launch = FLOPS_DERIV * cells
    achieved_tf = flops_launch / (dom_launch_ms * 1e-3) / 1e12
    traffic, tsrc = measured_traffic(names[dom], n)
    step_ms = t_max / args.steps
    hbm_gbs = BYTES_PER_CELL_UPDATE * cells / (step_ms * 1e-3) / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    launches_per_step = sum(klaunch) / args.steps

    result = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": box_workload(n),
                   "n": n, "form": "fp64 plain", "parallelism": f"replicas x{dist.world}" if dist.world > 1 else "1 box",
                   "arithmetic": "FP64; 19 of the 39 8-tap stencil sums per cell and stage formed exactly in "
                                 "64-bit integers on the significands and rounded once to FP64",
                   "l2": f"working set {Box_bytes(C, n) / 1e9:.2f} GB > 129 MB L2 (no flush needed)",
                   "tile_log2_ijk": {"fp64": list(tile64), "mixed": list(tile32)},
                   "mixed_assembly_kernel": {C.CNS_ASSEMBLE_TMA: "tma", C.CNS_ASSEMBLE_TMA_WS: "tma_ws"}.get(kern32, "direct")},
        "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d_bytes,
                "d2h_bytes_per_step": d2h_bytes, "in_place": in_place,
                "api": "cns_new_advance (host U in, 1 RK3 step, U out)",
                "pinned_host": pinned, "steps": k_e2e},
        "roofline": {"bound": "fp64", "kernel": names[dom], "achieved": achieved_tf, "peak": fp64_peak,
                     "unit": "TFLOP/s", "frac": achieved_tf / fp64_peak,
                     "peak_source": "measured live: FP64 FMA probe kernel (cns_measure_fp64_peak)",
                     "flops_per_launch": flops_launch, "launch_ms": dom_launch_ms,
                     "flops_basis": "the reference's FP64 operation count (2,450 per cell-update, less k_deriv's "
                                    "3 x 132, over 3 launches); the fused kernel retires fewer FP64 instructions "
                                    "than that count, so frac can exceed 1",
                     "fp64_pipe_busy_ncu": 0.744, "int_pipe_busy_ncu": 0.361,
                     "pipe_source": "ncu sm__pipe_fp64_cycles_active and sm__inst_executed_pipe_alu of stage 1 "
                                    "(part of the stencil sums run exactly on the integer pipes), "
                                    "profiles/k_assemble_fp64_128cube.md",
                     "traffic": traffic, "traffic_source": tsrc},
        "hbm": {"achieved_gbs": hbm_gbs, "peak_gbs": hbm_peak, "frac": hbm_gbs / hbm_peak,
                "bytes_per_cell_update": BYTES_PER_CELL_UPDATE, "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "fp64_step": {"achieved_tflops": FLOPS_PER_CELL_UPDATE * cells / (step_ms * 1e-3) / 1e12,
                      "frac_of_fp64_peak": FLOPS_PER_CELL_UPDATE * cells / (step_ms * 1e-3) / 1e12 / fp64_peak},
        "kernels_ms_per_step": {names[i]: kms[i] / args.steps for i in range(L.KERN_COUNT)},
        "mixed": {"value": mixed_value, "unit": "cell-updates/s", "speedup_vs_fp64": mixed_value / (value / dist.world),
                  "max_normwise_err_vs_fp64_after_100_steps": float(mixed_err.max()),
                  "err_per_var": [float(x) for x in mixed_err], "steps": args.steps,
                  "kernels_ms_per_step": {names[i]: mms[i] / args.steps for i in range(L.KERN_COUNT)}},
        "gpu_launches": int(sum(klaunch)),
        "launches_per_step": launches_per_step,
        "clocks": clk.summary(),
    }
    return result


def Box_bytes(C, n):
    return C.Box.bytes_for(n, C.CNS_FP64)


def run_case(args):
    """Just the kernels of one form on the n^3 box: what an ncu capture should see."""
    import cns_nospec_gb300 as C
    from cns_nospec_gb300 import _lib as L
    from cns_nospec_gb300 import initdata as I
    lib = C.load()
    L.check(lib.cns_set_device(0))
    if args.case == "e2e":
        Uh, pinned, _keep = pinned_like((args.n + 8,) * 3 + (5,))
        Uh[...] = I.initial_state(args.n, perturb=1e-3, seed=1)
        h = C.read_configurations(args.n, I.box_dx(args.n), I.CFL, I.ETA, I.ALAM)
        for _ in range(args.warmup):
            C.new_advance(Uh, None, None, None, None, h)
        lib.cns_device_synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            C.new_advance(Uh, None, None, None, None, h)
        lib.cns_device_synchronize()
        print(json.dumps({"case": "e2e", "n": args.n, "calls": args.steps, "pinned_host": pinned,
                          "ms_per_call": 1e3 * (time.perf_counter() - t0) / max(args.steps, 1)}))
        return
    prec = C.CNS_FP64 if args.case == "fp64" else C.CNS_MIXED
    box = C.Box(args.n, I.box_dx(args.n), I.CFL, I.ETA, I.ALAM, precision=prec)
    if args.kernel:
        box.set_kernel({"ws": C.CNS_ASSEMBLE_TMA_WS, "tma": C.CNS_ASSEMBLE_TMA, "direct": C.CNS_ASSEMBLE_DIRECT}[args.kernel])
    box.init_field(perturb=1e-3, seed=1)
    box.advance_timed(args.warmup)
    ms, launches, total = box.advance_timed(args.steps)
    box.sync()
    print(json.dumps({"case": args.case, "n": args.n, "steps": args.steps, "total_ms": total,
                      "kernel_ms": dict(zip(L.KERNEL_NAMES, ms)), "launches": dict(zip(L.KERNEL_NAMES, launches))}))


def batch_specs(count=256, seed=2, nmin=16, nmax=96):
    """Uneven periodic boxes: per-axis sizes log-uniform over [nmin, nmax], velocity
    amplitudes, eta and alam x U(0.8, 1.2), seeded (numpy PCG64)."""
    import math
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for b in range(count):
        n = tuple(int(round(math.exp(x))) for x in rng.uniform(math.log(nmin), math.log(nmax), 3))
        amp = tuple(float(x) for x in rng.uniform(0.8, 1.2, 3))
        f_eta, f_alam = (float(x) for x in rng.uniform(0.8, 1.2, 2))
        out.append((n, amp, f_eta, f_alam, 100 + b))
    return out


def run_batch(args):
    """256 uneven boxes (16..96 cells per axis), 50 RK3 steps, one persistent launch per kernel
    and stage for all boxes, the step captured in a CUDA graph, tile shapes autotuned."""
    import cns_nospec_gb300 as C
    from cns_nospec_gb300 import _lib as L
    from cns_nospec_gb300 import initdata as I
    lib = C.load()
    L.check(lib.cns_set_device(0))
    prec = C.CNS_MIXED if args.precision == "mixed" else C.CNS_FP64
    specs = batch_specs(args.boxes)
    boxes, cells = [], 0
    batch = C.Batch()
    for n, amp, fe, fa, seed in specs:
        b = C.Box(n, I.box_dx(n), I.CFL, I.ETA * fe, I.ALAM * fa, precision=prec)
        b.init_field(amp, 1e-3, seed)
        batch.add(b)
        boxes.append(b)
        cells += n[0] * n[1] * n[2]
    t0 = time.perf_counter()
    policy, tuned_ms = batch.autotune(trial_steps=2)
    tune_s = time.perf_counter() - t0
    batch.advance(args.warmup)
    batch.sync()
    t0 = time.perf_counter()
    batch.advance(args.steps)
    batch.sync()
    el = time.perf_counter() - t0
    for b in boxes:
        b.sync()
    value = cells * args.steps / el
    # the first 32 boxes one at a time (each its own graph), for the batching efficiency
    solo_cells, solo_t = 0, 0.0
    for b, (n, *_r) in zip(boxes[:32], specs[:32]):
        batch.remove(b)
        b.advance(1)
        b.sync()
        ts = time.perf_counter()
        b.advance(5)
        b.sync()
        solo_t += time.perf_counter() - ts
        solo_cells += n[0] * n[1] * n[2] * 5
    res = {"workload": f"batch of {len(boxes)} uneven periodic boxes (16..96 per axis, seed 2), {args.precision}",
           "cells_per_step": cells, "steps": args.steps, "value": value, "unit": "cell-updates/s",
           "ms_per_step": 1e3 * el / args.steps, "autotune_policy": policy,
           "autotune_ms_per_step_trial": tuned_ms, "autotune_s": tune_s, "launches_per_step": 7,
           "first32_one_at_a_time_cell_updates_per_s": solo_cells / solo_t,
           "device_bytes": sum(C.Box.bytes_for(s[0], prec) for s in specs)}
    batch.close()
    for b in boxes:
        b.close()
    return res


def run_mixed256(args):
    """256^3 box, the perturbed sinusoidal field: FP64 and mixed forms, 100 RK3 steps each; normwise error
    of the mixed form against FP64 per conserved variable, and cell-updates/s of both."""
    import cns_nospec_gb300 as C
    from cns_nospec_gb300 import _lib as L
    from cns_nospec_gb300 import initdata as I
    lib = C.load()
    L.check(lib.cns_set_device(0))
    n = args.n
    out, rate = {}, {}
    for prec in (C.CNS_FP64, C.CNS_MIXED):
        b = C.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=prec)
        b.init_field((1.0, 1.0, 1.0), 1e-3, 1)
        ms, launches, total = b.advance_timed(args.steps)
        b.sync()
        rate[prec] = n ** 3 * args.steps / (total * 1e-3)
        out[prec] = b.download()
        b.close()
    mx, rms = I.normwise_error(out[C.CNS_MIXED], out[C.CNS_FP64])
    return {"workload": f"periodic box {n}^3, sinusoidal field with a 1e-3 perturbation (seed 1), {args.steps} RK3 steps", "fp64_cell_updates_per_s":
            rate[C.CNS_FP64], "mixed_cell_updates_per_s": rate[C.CNS_MIXED],
            "speedup": rate[C.CNS_MIXED] / rate[C.CNS_FP64], "max_normwise_err": [float(x) for x in mx],
            "rms_normwise_err": [float(x) for x in rms], "vars": ["rho", "rho u", "rho v", "rho w", "rho E"]}


def run_serve(args):
    """Poisson stream of independent solves (n 24..192, 10..200 steps, coefficients x U(0.8,1.2),
    50/50 FP64/mixed), HBM budget, continuous batching; p50/p99 latency and throughput, beside
    a single 512^3 FP64 box advanced alone."""
    import cns_nospec_gb300 as C
    from cns_nospec_gb300 import _lib as L
    from cns_nospec_gb300 import initdata as I
    from cns_nospec_gb300 import serve as S
    lib = C.load()
    L.check(lib.cns_set_device(0))
    reqs = S.request_stream(rate=args.rate, count=args.requests, seed=4)
    srv = S.Server(budget_bytes=args.budget_gb * 1e9)
    rep = srv.run(reqs, realtime=True)
    sat = S.Server(budget_bytes=args.budget_gb * 1e9).run(
        S.request_stream(rate=args.rate, count=args.requests, seed=5, start_all_at_zero=True), realtime=False)
    # single-box throughput of each form, for the batching efficiency of the saturated run:
    # the time the same solves would take back to back, each at its form's 128^3 rate
    single = {}
    for prec in (C.CNS_FP64, C.CNS_MIXED):
        b = C.Box(128, I.box_dx(128), I.CFL, I.ETA, I.ALAM, precision=prec)
        b.init_field((1.0, 1.0, 1.0), 1e-3, 1)
        b.autotune(trial_steps=2)
        _, _, total = b.advance_timed(20)
        b.sync()
        single[prec] = 128 ** 3 * 20 / (total * 1e-3)
        b.close()
    # everything the device advanced (failed solves included) against the same cell-updates
    # at single-box rates: the loop's overhead and the batching gain for small boxes
    alone_s = sum(d.req.n[0] * d.req.n[1] * d.req.n[2] * d.steps_done / single[d.req.precision] for d in sat["done"])
    sat["single_box_rates"] = {"fp64": single[C.CNS_FP64], "mixed": single[C.CNS_MIXED]}
    sat["efficiency_vs_single_box"] = alone_s / sat["busy_s"] if sat["busy_s"] > 0 else None
    big = {}
    if args.big > 0:
        n = args.big
        b = C.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
        b.init_field((1.0, 1.0, 1.0), 1e-3, 1)
        ms, _, total = b.advance_timed(args.big_steps)
        b.sync()
        big = {"n": n, "steps": args.big_steps, "cell_updates_per_s": n ** 3 * args.big_steps / (total * 1e-3),
               "device_bytes": C.Box.bytes_for(n)}
        b.close()
    strip = lambda r: {k: v for k, v in r.items() if k != "done"}
    return {"workload": f"{args.requests} requests, Poisson rate {args.rate}/s, n 24..192, steps 10..200, "
                        f"50/50 FP64/mixed, budget {args.budget_gb} GB",
            "realtime": strip(rep), "saturated": strip(sat), "single_box_alone": big,
            "max_active": max((e["active"] for e in srv.log), default=0)}


def main():
    args = parse()
    if args.case:
        run_case(args)
        return
    if args.workload != "box":
        fn = {"batch": run_batch, "mixed256": run_mixed256, "serve": run_serve, "cpu": run_cpu_table}[args.workload]
        print(json.dumps(fn(args)))
        return
    dist = Dist()
    try:
        if args.impl == "reference":
            res = run_reference(args, dist)
        else:
            res = run_ours(args, dist)
            if dist.rank == 0 and res is not None and not args.no_cpu_baseline:
                res["cpu_baseline"] = cpu_baseline(args.n, args.cpu_seconds)
        if dist.rank == 0 and res is not None:
            print(json.dumps(res))
    finally:
        dist.close()


if __name__ == "__main__":
    main()
