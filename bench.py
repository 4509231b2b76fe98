"""Benchmark: cell-updates/s of the RK3 advance on one periodic box.

Workload (default): 256^3 cells + 4 ghost cells a side, the CNS_NoSpec initial field with a
seeded +-1e-3 perturbation of rho, u, v, w; a step is one full RK3 step (new_advance,
cpu/advance.cpp:13-154) of that box.  `value` is the plain FP64 form, device-resident and
graph-replayed; the same line carries the mixed FP32/FP64 form on the same box (its rate and its
error against the FP64 form after 100 steps), the end-to-end rate through the reference-facing
call with page-locked and with pageable host arrays, the 128^3 box, a batch of 256 uneven boxes
and a short serving stream.

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

# The reference's FP64 operation count of one cell-update (one cell, one full RK3 step; each
# +, -, *, / one flop): 3 x (ctoprim 16 + hypterm 358 + diffterm 415) + RK combines 15 + 30 + 30
# + Courant 8 = 2450.  Reported as a reference-op throughput; the roofline uses the FP64
# operations the kernels execute (counted by ncu).
FLOPS_PER_CELL_UPDATE = 2450
# Compulsory HBM traffic of one cell-update with the FP64 state: stage 1 reads U^n and writes
# U^1 (80 B); stages 2 and 3 read U^(k), U^n and write U^(k+1) (120 B each).
BYTES_PER_CELL_UPDATE = 320
MIXED_ERROR_STEPS = 100


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--size", dest="n", type=int, default=256, help="cells per axis of the periodic box")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="only the headline box (no 128^3 box, batch, serving stream or pageable e2e)")
    p.add_argument("--cpu-seconds", type=float, default=16.0, help="CPU baseline sample length (timed part)")
    p.add_argument("--case", choices=["fp64", "mixed", "e2e", "e2e_pageable"], default=None,
                   help="profiling case: only upload + warmup + steps of one form (for ncu), then exit; "
                        "e2e: warmup + steps calls of cns_new_advance on a page-locked host array "
                        "(e2e_pageable: on a pageable one)")
    p.add_argument("--kernel", choices=["ws", "tma", "direct", "fx", "fxd"], default=None,
                   help="--case: the assembly kernel (default: the library's choice; ws is mixed-only, fx (TMA) and "
                        "fxd (direct) on fixed-point taps FP64-only)")
    p.add_argument("--workload", choices=["box", "batch", "mixed256", "serve", "cpu"], default="box",
                   help="box: the headline line (default); batch: 256 uneven boxes; "
                        "mixed256: FP64 vs mixed at --size; serve: the request stream; "
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


def workload_config(n):
    """`config` of the JSON line: identical on both arms (the arms' own details go elsewhere)."""
    # the FP64 box's device state: U, the stage state, two 16-field primitive/flux sets and the
    # 4-field derivative set, 46 doubles per ghost-inclusive cell
    big = 46 * 8 * (n + 8) ** 3 > 129e6
    return {"workload": box_workload(n), "n": n, "steps_per_call": 1,
            "l2": "inputs larger than L2 (no flush)" if big else "inputs smaller than L2 (resident between steps)"}


def pinned_like(shape):
    """A pinned host float64 array when torch is importable (plumbing only), else pageable."""
    try:
        import torch
        t = torch.empty(shape, dtype=torch.float64, pin_memory=True)
        return t.numpy(), True, t
    except Exception:
        return np.empty(shape, dtype=np.float64), False, None


def profile_json(name: str):
    """A committed ncu summary in machine-readable form (profiles/<name>.json), or {}."""
    try:
        with open(os.path.join(ROOT, "profiles", name + ".json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


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
    host cores: one single-threaded process per core, each advancing its own n^3 box (one
    untimed step, then about `seconds` of timed steps; oracle_processes); beside it one core
    alone at 32^3."""
    from cns_nospec_gb300 import initdata as I
    from oracle import oracle as O
    O.build(ref=os.path.isdir(O.REF_SRC))
    threads = host_split("port")
    nproc = host_processes(n, threads)
    value, steps, wall = oracle_processes(n, 1000, 1, seconds, nproc, threads=threads)
    O.set_threads(1)
    V = I.initial_state(32, perturb=1e-3, seed=1)
    k, t1 = 0, time.perf_counter()
    while True:
        V, _ = O.advance(V, 1, I.box_dx(32), I.CFL, I.ETA, I.ALAM, which="port")
        k += 1
        e1 = time.perf_counter() - t1
        if e1 >= 1.0 or k >= 50:
            break
    return {"value": value, "unit": "cell-updates/s", "cores": nproc * threads, "cpu_model": cpu_model(),
            "kind": "port", "sample": f"{nproc} processes x {threads} threads, {steps} RK3 steps in all of their own "
                                      f"{n}^3 boxes, {wall:.1f} s", "one_core_32": 32 ** 3 * k / e1}


def _oracle_process(n, steps, warmup, seconds, which, threads, barrier, out):
    """One run of the reference algorithm (a child process of oracle_processes) on `threads`
    threads: `warmup` untimed steps, a barrier with the other processes, then up to `steps` timed
    steps or `seconds` of them.  Puts the steps done and the wall-clock start and end of the timed
    part."""
    from cns_nospec_gb300 import initdata as I
    from oracle import oracle as O
    O.set_threads(threads)
    U = I.initial_state(n, perturb=1e-3, seed=1)
    dx = I.box_dx(n)
    for _ in range(warmup):
        U, _ = O.advance(U, 1, dx, I.CFL, I.ETA, I.ALAM, which=which)
    barrier.wait(timeout=900)
    k, t0 = 0, time.time()
    while k < steps:
        U, _ = O.advance(U, 1, dx, I.CFL, I.ETA, I.ALAM, which=which)
        k += 1
        if time.time() - t0 >= seconds:
            break
    out.put((k, t0, time.time()))


def host_processes(n: int, threads: int = 1) -> int:
    """Processes for oracle_processes: one per `threads` host cores, but no more than half of the
    host's memory holds (an n^3 oracle step holds about 34 doubles per ghost-inclusive cell: U,
    Unew, Q, D, F and diffterm's nine temporaries)."""
    cores = max(1, (os.cpu_count() or 1) // threads)
    try:
        mem = os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")
    except (ValueError, OSError, AttributeError):
        return cores
    per = 34 * 8 * (n + 8) ** 3
    return max(1, min(cores, int(mem // 2 // per)))


def host_split(which: str) -> int:
    """Threads per process for the reference algorithm on the host cores.  The reference's
    own cpu/ objects are single-threaded: one process per core.  The port threads its loops
    (OpenMP): two threads per process, which on the 16 Neoverse-V2 cores of a GB300 host gives the
    throughput of 16 single-threaded processes (1.69e7 cell-updates/s at 256^3 either way) in half
    the time per step (7.9 s against 15.9 s), where 4 x 4 gave 1.64e7 and 1 x 16 1.37e7."""
    threads = 2 if which == "port" and (os.cpu_count() or 1) >= 2 else 1
    return threads


def oracle_processes(n, steps, warmup, seconds, nproc, which="port", threads=1):
    """The reference algorithm on the host cores: `nproc` independent processes (spawned) of
    `threads` threads each, each advancing its own copy of the n^3 box, their timed parts started
    together.  Throughput = all processes' cell-updates / (last end - first start).  Returns
    (throughput, steps done in all, wall seconds)."""
    import multiprocessing as mp
    import queue
    ctx = mp.get_context("spawn")
    barrier, out = ctx.Barrier(nproc), ctx.Queue()
    procs = [ctx.Process(target=_oracle_process, args=(n, steps, warmup, seconds, which, threads, barrier, out))
             for _ in range(nproc)]
    for p in procs:
        p.start()
    res, t0 = [], time.time()
    try:
        while len(res) < nproc:
            try:
                res.append(out.get(timeout=5))
            except queue.Empty:
                if any(p.exitcode not in (None, 0) for p in procs) or time.time() - t0 > 1800:
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
    """--impl reference: the reference algorithm on the host cores, on the same workload, with
    the same warm-up and timed step counts as the GPU arm.  Where the reference tree exists its
    own cpu/ objects run (oracle/_ref); elsewhere (where it is absent and x86 objects do not
    travel) the oracle port, which gives the same bits.  Its cpu/ path is single-threaded, so it
    uses the cores as independent processes, each advancing its own copy of the box (host_split,
    oracle_processes): `warmup` untimed steps each, then `steps` timed steps each (a step of this
    arm: every process advances its box one RK3 step), bounded to 20 minutes."""
    if dist.rank != 0:
        return None
    from oracle import oracle as O
    O.build(ref=os.path.isdir(O.REF_SRC))
    use_ref = O.have_ref() and os.path.isdir(O.REF_SRC)
    which = "ref" if use_ref else "port"
    n = args.n
    threads = host_split(which)
    procs = host_processes(n, threads)
    v, done, wall = oracle_processes(n, args.steps, args.warmup, 1200.0, procs, which=which, threads=threads)
    steps = max(1, done // procs)
    kind = "reference" if use_ref else "port"
    sample = (f"{procs} processes x {threads} threads, each ({args.warmup} untimed + {steps} timed) RK3 steps of "
              f"its own {n}^3 box, {wall:.1f} s timed")
    return {"metric": "cell-updates/s", "value": v, "unit": "cell-updates/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(n),
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": procs * threads, "cpu_model": cpu_model(),
                             "kind": kind, "sample": sample},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def time_box(C, n, prec, warmup, steps, sampler=None):
    """One n^3 box of the perturbed field in form `prec`: autotuned (state restored), `warmup`
    steps, then `steps` graph-replayed steps timed with CUDA events on the box's stream (under
    `sampler`, the clock sampler, when given), then the same number of steps again through the
    event-per-kernel path for the kernel split.  Returns a dict."""
    from cns_nospec_gb300 import initdata as I
    box = C.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=prec)
    box.init_field((1.0, 1.0, 1.0), 1e-3, 1)
    tile, kern, _ = box.autotune(trial_steps=4)
    box.advance(warmup)
    box.sync()
    if sampler is not None:
        with sampler:
            ms = box.advance_ms(steps)
    else:
        ms = box.advance_ms(steps)
    kms, klaunch, _ = box.advance_timed(steps)
    box.sync()
    launches = box.launches_per_step() * steps
    box.close()
    return {"ms": ms, "value": n ** 3 * steps / (ms * 1e-3), "tile": tile, "kernel": kern, "kernel_ms": kms,
            "kernel_launches": klaunch, "launches": launches}


def mixed_error(C, n, steps):
    """Normwise max and RMS error per conserved variable of the mixed form against the FP64 form
    after `steps` RK3 steps from the same device-generated state."""
    from cns_nospec_gb300 import initdata as I
    ends = {}
    for prec in (C.CNS_FP64, C.CNS_MIXED):
        b = C.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=prec)
        b.init_field((1.0, 1.0, 1.0), 1e-3, 1)
        b.advance(steps)
        b.sync()
        ends[prec] = b.download()
        b.close()
    mx, rms = I.normwise_error(ends[C.CNS_MIXED], ends[C.CNS_FP64])
    return {"steps": steps, "vars": ["rho", "rho u", "rho v", "rho w", "rho E"],
            "max": [float(x) for x in mx], "rms": [float(x) for x in rms], "worst": float(mx.max())}


def time_e2e(C, lib, n, U0, Uh, calls, dist):
    """cns_new_advance (the reference's new_advance) on the host array Uh, one RK3 step per call,
    `calls` calls timed on the host clock with a device synchronize on both sides: the upload of
    U, the step and the download of U each call.  Returns (cell-updates/s, ms per call)."""
    from cns_nospec_gb300 import initdata as I
    h = C.read_configurations(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    Uh[...] = U0
    C.new_advance(Uh, None, None, None, None, h)  # warm (creates the cached device state)
    Uh[...] = U0
    lib.cns_device_synchronize()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(calls):
        C.new_advance(Uh, None, None, None, None, h)
    lib.cns_device_synchronize()
    el = dist.max(time.perf_counter() - t0)
    dist.barrier()
    return dist.world * n ** 3 * calls / el, 1e3 * el / calls


def fp64_roofline(kernel_ms, klaunch, names, cells, fp64_peak):
    """The roofline of the FP64 form's dominant kernel: the FP64 operations it executes per cell
    (ncu's DFMA, DADD and DMUL thread-instruction counts, a DFMA counting 2) over its live launch
    time, against the FP64 FMA rate this process measured.  The per-cell counts and DRAM bytes come
    from the committed capture (profiles/fp64_counters.json; per cell, so they scale to any box)."""
    dom = int(np.argmax(kernel_ms))
    name = names[dom]
    launch_ms = kernel_ms[dom] / max(klaunch[dom], 1)
    cnt = profile_json("fp64_counters").get(name, {})
    out = {"bound": "fp64", "kernel": name, "launch_ms": launch_ms, "peak": fp64_peak, "unit": "TFLOP/s",
           "peak_source": "measured live: FP64 FMA probe kernel (cns_measure_fp64_peak)"}
    if "fp64_flops_per_cell" in cnt:
        flops = cnt["fp64_flops_per_cell"] * cells
        inst = cnt["fp64_inst_per_cell"] * cells
        achieved = flops / (launch_ms * 1e-3) / 1e12
        # the probe's DFMA rate in warp-lane instructions per second is fp64_peak / 2
        out.update({"achieved": achieved, "frac": achieved / fp64_peak, "flops_per_launch": flops,
                    "fp64_inst_rate_frac": inst / (launch_ms * 1e-3) / (fp64_peak * 1e12 / 2),
                    "basis": "FP64 operations executed, counted by ncu per cell (DFMA = 2, DADD and DMUL = 1)",
                    "fp64_pipe_active_ncu": cnt.get("fp64_pipe_active"),
                    "alu_pipe_active_ncu": cnt.get("alu_pipe_active"),
                    "issue_active_ncu": cnt.get("issue_active"),
                    "counters": "fp64_counters.json: " + name})
    else:
        out.update({"achieved": None, "frac": None, "counters": None})
    # DRAM bytes per cell measured on a box of this size where there is one (the stencils' plane
    # re-reads stay in L2 at 128^3, not at 256^3), else the 128^3 figure
    tr = cnt.get("dram_bytes_per_cell_by_n", {}).get(str(round(cells ** (1 / 3))), cnt.get("dram_bytes_per_cell"))
    out["traffic"] = tr * cells if tr is not None else None
    return out


def run_ours(args, dist):
    import cns_nospec_gb300 as C
    from cns_nospec_gb300 import _lib as L
    from cns_nospec_gb300 import build as B
    from cns_nospec_gb300 import initdata as I
    B.build()
    lib = C.load()
    L.check(lib.cns_set_device(dist.local))
    n, cells = args.n, args.n ** 3
    names = L.KERNEL_NAMES
    fp64_peak = ctypes.c_double(0.0)
    L.check(lib.cns_measure_fp64_peak(ctypes.byref(fp64_peak)))
    fp64_peak = fp64_peak.value

    # ---- the headline: device-resident FP64 plain form, graph-replayed --------------------
    dist.barrier()
    clk = ClockSampler(dist.local)
    f64 = time_box(C, n, C.CNS_FP64, args.warmup, args.steps, sampler=clk)
    t_max = dist.max(f64["ms"])
    dist.barrier()
    value = dist.world * cells * args.steps / (t_max * 1e-3)
    step_ms = t_max / args.steps

    # ---- mixed form on the same box, and its error after 100 steps ----------------------
    mix = time_box(C, n, C.CNS_MIXED, args.warmup, args.steps)
    err = mixed_error(C, n, MIXED_ERROR_STEPS)

    # ---- end to end through the reference-facing call, host arrays ----------------------
    b0 = C.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    b0.init_field((1.0, 1.0, 1.0), 1e-3, 1)
    U0 = b0.download()
    b0.close()
    calls = max(1, min(args.steps, 20))
    Uh, pinned, _keep = pinned_like(U0.shape)
    e2e_value, e2e_ms = time_e2e(C, lib, n, U0, Uh, calls, dist)
    flag = ctypes.c_int(0)
    L.check(lib.cns_host_in_place(ctypes.c_void_p(Uh.ctypes.data), ctypes.c_longlong(Uh.nbytes), ctypes.byref(flag)))
    in_place = bool(flag.value)
    e2e = {"value": e2e_value, "unit": "cell-updates/s",
           "h2d_bytes_per_step": cells * 5 * 8 if in_place else int(Uh.nbytes), "d2h_bytes_per_step": int(Uh.nbytes),
           "ms_per_call": e2e_ms, "calls": calls, "pinned_host": pinned, "in_place": in_place,
           "api": "cns_new_advance (host U in, 1 RK3 step, U out)"}
    del Uh, _keep
    extras = {}
    if not args.no_extras and dist.world == 1:
        Up = np.array(U0)  # pageable, as the reference's malloc'd arrays are
        pv, pms = time_e2e(C, lib, n, U0, Up, calls, dist)
        L.check(lib.cns_host_in_place(ctypes.c_void_p(Up.ctypes.data), ctypes.c_longlong(Up.nbytes),
                                      ctypes.byref(flag)))
        extras["e2e_pageable"] = {"value": pv, "unit": "cell-updates/s", "ms_per_call": pms, "calls": calls,
                                  "in_place": bool(flag.value), "vs_pinned_e2e": pv / e2e_value,
                                  "h2d_bytes_per_step": cells * 5 * 8 if flag.value else int(Up.nbytes),
                                  "d2h_bytes_per_step": int(Up.nbytes),
                                  "api": "cns_new_advance on a pageable (malloc'd) host array"}
        del Up
    del U0

    roof = fp64_roofline(f64["kernel_ms"], f64["kernel_launches"], names, cells, fp64_peak)
    hbm_gbs = BYTES_PER_CELL_UPDATE * cells / (step_ms * 1e-3) / 1e9
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm_peak = json.load(f).get("hbm_gbs")
    except (OSError, ValueError):
        hbm_peak = None
    if hbm_peak is None:
        hbm_peak, hbm_src = 6800.0, "fallback 6.8 TB/s"
    else:
        hbm_src = "MEASURED_PEAKS.json hbm_gbs"
    ksplit = lambda r: {names[i]: r["kernel_ms"][i] / args.steps for i in range(L.KERN_COUNT)}
    result = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n),
        "form": {"plain": "FP64 (CNS_ASSEMBLE_FX); of the 39 8-tap stencil sums per cell and stage, the 21 of the "
                          "derivative pass and the Laplacians are exact integer sums of 62-bit fixed-point copies of "
                          "u, v, w, e (on cubic cells the second differences of a field that share a factor in one "
                          "sum) and the 5 k-axis flux divergences and the k-axis mixed viscous term exact integer "
                          "sums of the FP64 significands, each sum rounded once to FP64; the other 12 FP64 chains",
                 "plain_kernel": {C.CNS_ASSEMBLE_FX: "fx", C.CNS_ASSEMBLE_DIRECT: "direct"}.get(f64["kernel"], "other"),
                 "parallelism": f"replicas x{dist.world}" if dist.world > 1 else "1 box",
                 "tile_log2_ijk": {"fp64": list(f64["tile"]), "mixed": list(mix["tile"])},
                 "mixed_assembly_kernel": {C.CNS_ASSEMBLE_TMA: "tma", C.CNS_ASSEMBLE_TMA_WS: "tma_ws"}.get(
                     mix["kernel"], "direct"),
                 "timing": "graph-replayed steps between CUDA events on the box's stream"},
        "e2e": e2e,
        "mixed": {"value": mix["value"], "unit": "cell-updates/s", "speedup_vs_fp64": mix["value"] / (value / dist.world),
                  "error_vs_fp64": err, "steps": args.steps, "kernels_ms_per_step": ksplit(mix)},
        "roofline": roof,
        "hbm": {"achieved_gbs": hbm_gbs, "peak_gbs": hbm_peak, "frac": hbm_gbs / hbm_peak,
                "bytes_per_cell_update": BYTES_PER_CELL_UPDATE, "peak_source": hbm_src},
        "reference_op_throughput": {"tflops": FLOPS_PER_CELL_UPDATE * cells / (step_ms * 1e-3) / 1e12,
                                    "basis": "the reference's FP64 operation count, 2,450 per cell-update"},
        "kernels_ms_per_step": ksplit(f64),
        "gpu_launches": f64["launches"],
        "launches_per_step": f64["launches"] / args.steps,
        "clocks": clk.summary(),
    }
    result.update(extras)
    if not args.no_extras and dist.world == 1:
        result["box_128"] = run_box128(C, args)
        result["batch"] = run_batch_short(C, args)
        result["serve"] = run_serve_short(C, args)
    return result


def run_box128(C, args):
    """The 128^3 box (100-step configuration): both forms' rates and the mixed error."""
    f = time_box(C, 128, C.CNS_FP64, args.warmup, max(args.steps, 50))
    m = time_box(C, 128, C.CNS_MIXED, args.warmup, max(args.steps, 50))
    return {"workload": box_workload(128), "fp64": f["value"], "mixed": m["value"],
            "speedup": m["value"] / f["value"], "mixed_error_vs_fp64": mixed_error(C, 128, MIXED_ERROR_STEPS)}


def run_case(args):
    """Just the kernels of one form on the n^3 box: what an ncu capture should see."""
    import cns_nospec_gb300 as C
    from cns_nospec_gb300 import _lib as L
    from cns_nospec_gb300 import initdata as I
    lib = C.load()
    L.check(lib.cns_set_device(0))
    if args.case in ("e2e", "e2e_pageable"):
        if args.case == "e2e":
            Uh, pinned, _keep = pinned_like((args.n + 8,) * 3 + (5,))
        else:
            Uh, pinned = np.empty((args.n + 8,) * 3 + (5,)), False
        Uh[...] = I.initial_state(args.n, perturb=1e-3, seed=1)
        h = C.read_configurations(args.n, I.box_dx(args.n), I.CFL, I.ETA, I.ALAM)
        for _ in range(args.warmup):
            C.new_advance(Uh, None, None, None, None, h)
        lib.cns_device_synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            C.new_advance(Uh, None, None, None, None, h)
        lib.cns_device_synchronize()
        print(json.dumps({"case": args.case, "n": args.n, "calls": args.steps, "pinned_host": pinned,
                          "ms_per_call": 1e3 * (time.perf_counter() - t0) / max(args.steps, 1)}))
        return
    prec = C.CNS_FP64 if args.case == "fp64" else C.CNS_MIXED
    box = C.Box(args.n, I.box_dx(args.n), I.CFL, I.ETA, I.ALAM, precision=prec)
    if args.kernel:
        box.set_kernel({"ws": C.CNS_ASSEMBLE_TMA_WS, "tma": C.CNS_ASSEMBLE_TMA, "direct": C.CNS_ASSEMBLE_DIRECT,
                        "fx": C.CNS_ASSEMBLE_TMA_FX, "fxd": C.CNS_ASSEMBLE_FX}[args.kernel])
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


def batch_run(C, prec, count, steps, warmup, solo=32):
    """`count` uneven boxes (16..96 cells per axis, seed 2) advanced together: one persistent
    launch per kernel and stage for all boxes, the step captured in a CUDA graph, the policy
    (tile shapes, assembly kernel) autotuned; `steps` graph-replayed steps timed with CUDA events.
    Beside it the first `solo` boxes advanced one at a time (each its own graph)."""
    from cns_nospec_gb300 import initdata as I
    specs = batch_specs(count)
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
    batch.advance(warmup)
    batch.sync()
    ms = batch.advance_ms(steps)
    for b in boxes:
        b.sync()
    value = cells * steps / (ms * 1e-3)
    solo_cells, solo_ms = 0, 0.0
    for b, (n, *_r) in zip(boxes[:solo], specs[:solo]):
        batch.remove(b)
        b.advance(1)
        b.sync()
        solo_ms += b.advance_ms(5)
        solo_cells += n[0] * n[1] * n[2] * 5
    batch.close()
    for b in boxes:
        b.close()
    solo_rate = solo_cells / (solo_ms * 1e-3)
    return {"boxes": len(specs), "cells_per_step": cells, "steps": steps, "value": value, "unit": "cell-updates/s",
            "ms_per_step": ms / steps, "autotune_policy": policy, "autotune_s": tune_s, "launches_per_step": 7,
            "first_boxes_one_at_a_time": {"boxes": solo, "value": solo_rate}, "batched_vs_one_at_a_time": value / solo_rate,
            "device_bytes": sum(C.Box.bytes_for(sp[0], prec) for sp in specs)}


def run_batch(args):
    """--workload batch: 256 uneven boxes, --steps RK3 steps (the configuration's 50)."""
    import cns_nospec_gb300 as C
    from cns_nospec_gb300 import _lib as L
    lib = C.load()
    L.check(lib.cns_set_device(0))
    prec = C.CNS_MIXED if args.precision == "mixed" else C.CNS_FP64
    res = batch_run(C, prec, args.boxes, args.steps, args.warmup)
    res["workload"] = f"batch of {args.boxes} uneven periodic boxes (16..96 per axis, seed 2), {args.precision}"
    return res


def run_batch_short(C, args):
    """The batch of 256 uneven boxes in both forms, a bounded number of steps (the default line)."""
    steps = min(args.steps, 10)
    return {"workload": "256 uneven periodic boxes (16..96 cells per axis, seed 2), one launch per kernel and stage, "
                        f"graph-replayed, autotuned; {steps} timed steps",
            "fp64": batch_run(C, C.CNS_FP64, 256, steps, 3), "mixed": batch_run(C, C.CNS_MIXED, 256, steps, 3)}


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


def serve_run(C, rate, requests, budget_gb, big, big_steps):
    """Poisson stream of independent solves (n 24..192, 10..200 steps, coefficients x U(0.8,1.2),
    50/50 FP64/mixed), HBM budget, continuous batching: p50/p99 latency and throughput in real
    time (arrivals honoured) and saturated (all waiting at t=0), the saturated run's efficiency
    against the same solves at single-box rates, and a single big FP64 box advanced alone."""
    from cns_nospec_gb300 import initdata as I
    from cns_nospec_gb300 import serve as S
    srv = S.Server(budget_bytes=budget_gb * 1e9)
    rep = srv.run(S.request_stream(rate=rate, count=requests, seed=4), realtime=True)
    sat = S.Server(budget_bytes=budget_gb * 1e9).run(
        S.request_stream(rate=rate, count=requests, seed=5, start_all_at_zero=True), realtime=False)
    # single-box throughput of each form, for the batching efficiency of the saturated run:
    # the time the same solves would take back to back, each at its form's 128^3 rate
    single = {}
    for prec in (C.CNS_FP64, C.CNS_MIXED):
        b = C.Box(128, I.box_dx(128), I.CFL, I.ETA, I.ALAM, precision=prec)
        b.init_field((1.0, 1.0, 1.0), 1e-3, 1)
        b.autotune(trial_steps=2)
        b.advance(3)
        ms = b.advance_ms(20)
        single[prec] = 128 ** 3 * 20 / (ms * 1e-3)
        b.close()
    # everything the device advanced (failed solves included) against the same cell-updates
    # at single-box rates: the loop's overhead and the batching gain for small boxes
    alone_s = sum(d.req.n[0] * d.req.n[1] * d.req.n[2] * d.steps_done / single[d.req.precision] for d in sat["done"])
    sat["single_box_rates"] = {"fp64": single[C.CNS_FP64], "mixed": single[C.CNS_MIXED]}
    sat["efficiency_vs_single_box"] = alone_s / sat["busy_s"] if sat["busy_s"] > 0 else None
    sat["efficiency_vs_single_box_wall"] = alone_s / sat["wall_s"] if sat["wall_s"] > 0 else None
    alone = {}
    if big > 0:
        b = C.Box(big, I.box_dx(big), I.CFL, I.ETA, I.ALAM)
        b.init_field((1.0, 1.0, 1.0), 1e-3, 1)
        b.advance(1)
        ms = b.advance_ms(big_steps)
        alone = {"n": big, "steps": big_steps, "cell_updates_per_s": big ** 3 * big_steps / (ms * 1e-3),
                 "device_bytes": C.Box.bytes_for(big)}
        b.close()
    strip = lambda r: {k: v for k, v in r.items() if k != "done"}
    return {"workload": f"{requests} requests, Poisson rate {rate}/s, n 24..192, steps 10..200, "
                        f"50/50 FP64/mixed, budget {budget_gb} GB",
            "realtime": strip(rep), "saturated": strip(sat), "single_box_alone": alone,
            "max_active": max((e["active"] for e in srv.log), default=0)}


def run_serve(args):
    """--workload serve: the request stream at --rate with --requests requests."""
    import cns_nospec_gb300 as C
    from cns_nospec_gb300 import _lib as L
    lib = C.load()
    L.check(lib.cns_set_device(0))
    return serve_run(C, args.rate, args.requests, args.budget_gb, args.big, args.big_steps)


def run_serve_short(C, args):
    """A bounded serving stream for the default line: 32 requests at 3/s."""
    return serve_run(C, 3.0, 32, 120.0, 512, 3)


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
            if dist.rank == 0 and dist.world == 1 and res is not None and not args.no_cpu_baseline:
                res["cpu_baseline"] = cpu_baseline(args.n, args.cpu_seconds)
        if dist.rank == 0 and res is not None:
            print(json.dumps(res))
    finally:
        dist.close()


if __name__ == "__main__":
    main()
