"""Continuous-batching server for independent periodic-box solves.

Requests (box size, step count, coefficients, precision tag) arrive over time.  The loop keeps
every admitted box's state resident in HBM, admits waiting requests in arrival order whenever
the device-memory budget (and an optional slot limit) allows, and advances ALL admitted boxes
together through one cns_batch (one launch per kernel and stage for every box of a precision;
each box keeps its own dt), as many RK3 steps per host round trip as the next event allows
(a box reaching its step count, a health check, an expected arrival).  Boxes leave the batch as soon as they
reach their step count, which frees their memory for the next arrivals.  Each box's result is
bit-identical to the same solve run alone: every cell's arithmetic is independent of what
else shares the launch.

    stream = request_stream(rate=4.0, count=100, seed=4)
    report = Server(budget_bytes=120e9).run(stream)
    report["latency_p50_s"], report["latency_p99_s"], report["cell_updates_per_s"]
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import _lib as L
from .initdata import ALAM, CFL, ETA, box_dx
from .solver import Batch, Box


@dataclass
class Request:
    rid: int
    arrival: float            # seconds after the stream starts
    n: tuple                  # interior cells per axis
    steps: int
    precision: int            # CNS_FP64 or CNS_MIXED
    amp: tuple = (1.0, 1.0, 1.0)
    eta: float = ETA
    alam: float = ALAM
    perturb: float = 1e-3
    seed: int = 1

    @property
    def work(self) -> float:
        """cell-updates this request asks for"""
        return float(self.n[0] * self.n[1] * self.n[2] * self.steps)


@dataclass
class Done:
    req: Request
    admitted: float
    finished: float
    result: Optional[np.ndarray] = None
    health: int = 0           # non-zero: the solve's state went non-physical (HEALTH_* bits)
    steps_done: int = 0       # RK3 steps the device ran for it (fewer than asked if evicted)

    @property
    def latency(self) -> float:
        return self.finished - self.req.arrival


def request_stream(rate: float, count: int, seed: int = 4, nmin: int = 24, nmax: int = 192, smin: int = 10,
                   smax: int = 200, mixed_fraction: float = 0.5, start_all_at_zero: bool = False) -> List[Request]:
    """Poisson arrivals at `rate` per second; n log-uniform over [nmin, nmax] (cubic boxes);
    steps uniform over [smin, smax]; velocity amplitudes, eta and alam x U(0.8, 1.2); each
    request tagged mixed with probability `mixed_fraction`.  Seeded (numpy PCG64)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for rid in range(count):
        if not start_all_at_zero:
            t += rng.exponential(1.0 / rate)
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        steps = int(rng.integers(smin, smax + 1))
        amp = tuple(float(x) for x in rng.uniform(0.8, 1.2, 3))
        eta = ETA * float(rng.uniform(0.8, 1.2))
        alam = ALAM * float(rng.uniform(0.8, 1.2))
        prec = L.CNS_MIXED if rng.uniform() < mixed_fraction else L.CNS_FP64
        out.append(Request(rid, t, (n, n, n), steps, prec, amp, eta, alam, 1e-3, 1000 + rid))
    return out


def run_alone(req: Request) -> np.ndarray:
    """The request solved by itself (the reference point of the alone-vs-mix check)."""
    box = Box(req.n, box_dx(req.n), CFL, req.eta, req.alam, precision=req.precision)
    box.init_field(req.amp, req.perturb, req.seed)
    box.advance(req.steps)
    box.sync()
    out = box.download()
    box.close()
    return out


@dataclass
class Server:
    budget_bytes: float = 120e9
    max_active: int = 1 << 30
    keep_results: bool = False
    health_every: int = 16     # check the active boxes' health every this many steps (0 = only at the end)
    box_cls: type = Box        # the device backend (tests substitute a host fake)
    batch_cls: type = Batch
    log: List[dict] = field(default_factory=list)

    def run(self, requests: List[Request], realtime: bool = True) -> Dict:
        """Serve `requests`.  realtime=True honours arrival times (sleeping while idle);
        False treats every request as already waiting (a saturation run)."""
        Box_, Batch_ = self.box_cls, self.batch_cls
        pending = deque(sorted(requests, key=lambda r: (r.arrival, r.rid)))
        active: Dict[int, tuple] = {}   # rid -> (box, req, steps_done, bytes, admitted_at)
        done: List[Done] = []
        batch = Batch_()
        used = 0
        peak_used = 0
        iters = 0                       # host round trips (batch advances)
        steps = 0                       # RK3 steps the batch ran
        step_s = 0.0                    # measured device time of one batch step
        executed = 0
        busy = 0.0
        t0 = time.perf_counter()
        try:
            while pending or active:
                now = time.perf_counter() - t0
                # admission: arrival order, memory budget and slot limit
                while pending and (not realtime or pending[0].arrival <= now) and len(active) < self.max_active:
                    req = pending[0]
                    need = Box_.bytes_for(req.n, req.precision)
                    if need > self.budget_bytes:
                        raise ValueError(f"request {req.rid} needs {need} B, above the whole budget")
                    if used + need > self.budget_bytes:
                        break
                    pending.popleft()
                    box = Box_(req.n, box_dx(req.n), CFL, req.eta, req.alam, precision=req.precision)
                    box.init_field(req.amp, req.perturb, req.seed)
                    batch.add(box)
                    self.log.append({"t": time.perf_counter() - t0, "admit": req.rid, "active": len(active) + 1,
                                     "used": used + need})
                    used += need
                    peak_used = max(peak_used, used)
                    active[req.rid] = (box, req, 0, need, time.perf_counter() - t0)
                if not active:
                    if pending and realtime:
                        time.sleep(max(0.0, min(pending[0].arrival - (time.perf_counter() - t0), 0.05)))
                    continue
                # advance up to the next event without returning to the host in between: the
                # first box to reach its step count, the next health check and, in real time,
                # the next arrival (at the measured per-step time)
                k = min(req.steps - steps_done for _, req, steps_done, *_r in active.values())
                if self.health_every > 0:
                    k = min(k, self.health_every - steps % self.health_every)
                if realtime and pending and step_s > 0:
                    wait = pending[0].arrival - (time.perf_counter() - t0)
                    k = min(k, max(1, int(wait / step_s)))
                k = max(1, k)
                ts = time.perf_counter()
                batch.advance(k)
                batch.sync()
                dt_busy = time.perf_counter() - ts
                busy += dt_busy
                step_s = dt_busy / k
                iters += 1
                steps += k
                executed += k * sum(r.n[0] * r.n[1] * r.n[2] for _, r, *_ in active.values())
                fin = time.perf_counter() - t0
                check = self.health_every > 0 and steps % self.health_every == 0
                for rid in list(active):
                    box, req, n_done, need, adm = active[rid]
                    n_done += k
                    # evict a diverged solve early instead of running it to its last step
                    if n_done >= req.steps or (check and box.health()):
                        batch.remove(box)
                        # a solve whose state went non-physical fails alone; the others go on
                        health = box.health()
                        res = box.download() if (self.keep_results and not health) else None
                        box.close()
                        used -= need
                        del active[rid]
                        done.append(Done(req, adm, fin, res, health, n_done))
                    else:
                        active[rid] = (box, req, n_done, need, adm)
        finally:
            for box, *_ in active.values():
                box.close()
            batch.close()
        wall = time.perf_counter() - t0
        ok = [d for d in done if not d.health]
        lat = np.array([d.latency for d in ok]) if ok else np.zeros(1)
        work = sum(d.req.work for d in ok)
        first = min((r.arrival for r in requests), default=0.0)
        return {
            "requests": len(done),
            "failed": len(done) - len(ok),
            "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p99_s": float(np.percentile(lat, 99)),
            "latency_max_s": float(lat.max()),
            "cell_updates": work,                 # of the solves that finished healthy
            "cell_updates_executed": executed,    # everything the device advanced, failed solves included
            "cell_updates_per_s": work / max(wall - (first if realtime else 0.0), 1e-9),
            "cell_updates_per_busy_s": work / max(busy, 1e-9),
            "executed_per_busy_s": executed / max(busy, 1e-9),
            "busy_s": busy,
            "wall_s": wall,
            "host_round_trips": iters,
            "batch_steps": steps,
            "peak_bytes": peak_used,
            "done": done,
        }
