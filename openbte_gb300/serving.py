"""Continuous-batching kappa_eff server on one GPU.

Requests (mesh, material, boundary conditions, contact) arrive over time; each
becomes a plan (sweep schedule and tables, built on host threads while the GPU
works on earlier requests) and then a solve. Up to ``slots`` solves run at
once, each on its own CUDA stream, so their sweeps and Krylov work overlap on
the device; a request is admitted when a slot is free and its HBM footprint
(plan tables + solver scratch) fits the budget. Plans are cached by content:
a repeated geometry keeps its mesh, sweep orders, tables and converged state
resident and can warm-start from it.

Admission is first-fit in arrival order: the oldest queued request that fits
the free memory starts first; a request whose footprint alone exceeds the
budget is rejected (``status='rejected'``) instead of waiting forever.

The scheduling logic talks to a backend with three calls (``build``,
``solve``, ``release``); :class:`GPUBackend` is the real one, tests can plug a
fake one to exercise admission and ordering without a GPU.
"""
from __future__ import annotations

import collections
import concurrent.futures as cf
import dataclasses
import threading
import time
from typing import Any, Optional

import numpy as np


@dataclasses.dataclass
class Request:
    geo: Any
    mat: Any
    bcs: Any
    ek: Any
    precision: str = "fp32_refine"
    rtol: float = 1e-6
    rid: int = 0
    arrival: float = 0.0          # seconds after the start of a replayed stream
    warm_start: bool = False
    tag: dict = dataclasses.field(default_factory=dict)


@dataclasses.dataclass
class Result:
    rid: int
    status: str                   # 'ok' | 'not_converged' | 'rejected' | 'error'
    kappa: float = float("nan")
    error: str = ""
    t_submit: float = 0.0
    t_built: float = 0.0
    t_start: float = 0.0
    t_done: float = 0.0
    footprint: int = 0
    n_sweeps: int = 0
    n_sweeps_fp64: int = 0
    slot: int = -1
    cached_plan: bool = False

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit

    @property
    def queue_time(self) -> float:
        return self.t_start - self.t_built


class GPUBackend:
    """Plans and solves on one CUDA device through the C ABI."""

    def __init__(self, device=0, restart=30, max_sweeps=2000, cache_plans=8):
        import torch
        self.torch = torch
        self.device = device
        self.restart = restart
        self.max_sweeps = max_sweeps
        self.cache_plans = cache_plans
        self._tl = threading.local()
        self._cache: "collections.OrderedDict[str, Any]" = collections.OrderedDict()
        self._busy = collections.Counter()
        self._lock = threading.Lock()

    def _stream(self):
        s = getattr(self._tl, "stream", None)
        if s is None:
            s = self.torch.cuda.Stream(device=self.device)
            self._tl.stream = s
        return s

    def budget(self, fraction: float) -> int:
        free, _ = self.torch.cuda.mem_get_info(self.device)
        return int(free * fraction)

    def build(self, req: Request):
        """-> (plan, footprint bytes, reused?)"""
        from .runtime import HostProblem, Plan
        hp = HostProblem(req.geo, req.mat, req.bcs, req.ek)
        key = hp.key()
        with self._lock:
            pl = self._cache.get(key)
            if pl is not None:
                self._cache.move_to_end(key)
                self._busy[key] += 1
                return pl, self._footprint(pl, req), True
        st = self._stream()
        with self.torch.cuda.stream(st):
            pl = Plan(hp, self.device, stream=st.cuda_stream)
        pl.key = key
        with self._lock:
            self._cache[key] = pl
            self._busy[key] += 1
        return pl, self._footprint(pl, req), False

    def _footprint(self, pl, req):
        a, b = pl.footprint(req.precision, self.restart)
        return int(a + b)

    def solve(self, pl, req: Request, slot: int) -> dict:
        from .bte import solve_plan
        torch = self.torch
        st = self._stream()
        pl.set_stream(st.cuda_stream)
        with torch.cuda.stream(st):
            dT0 = torch.zeros(pl.n, dtype=torch.float64, device=f"cuda:{self.device}")
            # the periodic-inflow preconditioner stays off: its blocks and set-up buffers are not part of the
            # footprint a request is admitted by (and a request's plan is usually solved once)
            info, *_ = solve_plan(pl, dT0, precision=req.precision, rtol=req.rtol, max_sweeps=self.max_sweeps,
                                  restart=self.restart, warm_start=req.warm_start, precond=-1)
        st.synchronize()
        return {"kappa": info.kappa_eff, "converged": bool(info.converged), "n_sweeps": info.n_sweeps,
                "n_sweeps_fp64": info.n_sweeps_fp64}

    def release(self, pl):
        """Solve finished: the plan stays cached (resident) unless the cache is over its size."""
        with self._lock:
            self._busy[pl.key] -= 1
            while len(self._cache) > self.cache_plans:
                victim = next((k for k in self._cache if self._busy[k] <= 0), None)
                if victim is None:
                    break
                self._cache.pop(victim)

    def evict_idle(self) -> int:
        """Drop every idle cached plan; returns how many were dropped."""
        with self._lock:
            idle = [k for k in self._cache if self._busy[k] <= 0]
            for k in idle:
                self._cache.pop(k)
        return len(idle)


class Server:
    """Continuous batching: a host pool builds plans, `slots` GPU workers solve concurrently."""

    def __init__(self, backend=None, slots: int = 4, builders: int = 4, hbm_budget: Optional[int] = None,
                 hbm_fraction: float = 0.7):
        self.backend = backend if backend is not None else GPUBackend()
        self.slots = slots
        self.budget = int(hbm_budget) if hbm_budget is not None else self.backend.budget(hbm_fraction)
        self._builders = cf.ThreadPoolExecutor(max_workers=builders, thread_name_prefix="obte-build")
        self._cv = threading.Condition()
        self._queue: "collections.deque" = collections.deque()   # built, waiting for admission
        self._used = 0
        self._running = 0
        self._closed = False
        self.results = []
        self.max_concurrent = 0
        self._workers = [threading.Thread(target=self._slot_loop, args=(i,), daemon=True, name=f"obte-slot{i}")
                         for i in range(slots)]
        for w in self._workers:
            w.start()

    # -- public -----------------------------------------------------------------------
    def submit(self, req: Request) -> cf.Future:
        fut: cf.Future = cf.Future()
        res = Result(rid=req.rid, status="error", t_submit=time.perf_counter())
        self._builders.submit(self._build, req, res, fut)
        return fut

    def close(self):
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        self._builders.shutdown(wait=True)
        for w in self._workers:
            w.join()

    # -- stages -------------------------------------------------------------------------
    def _build(self, req, res, fut):
        try:
            plan, foot, cached = self.backend.build(req)
        except Exception as e:  # noqa: BLE001 - reported per request
            res.status, res.error, res.t_done = "error", f"{type(e).__name__}: {e}", time.perf_counter()
            self._finish(res, fut)
            return
        res.t_built = time.perf_counter()
        res.footprint = foot
        res.cached_plan = cached
        if foot > self.budget:
            self.backend.release(plan)
            res.status = "rejected"
            res.error = f"footprint {foot} B exceeds the HBM budget {self.budget} B"
            res.t_done = time.perf_counter()
            self._finish(res, fut)
            return
        with self._cv:
            self._queue.append((req, res, fut, plan))
            self._cv.notify_all()

    def _take(self):
        """First queued request (arrival order) that fits the free memory; None when closing."""
        with self._cv:
            while True:
                for i, item in enumerate(self._queue):
                    if self._used + item[1].footprint <= self.budget:
                        del self._queue[i]
                        self._used += item[1].footprint
                        self._running += 1
                        self.max_concurrent = max(self.max_concurrent, self._running)
                        return item
                if self._closed and not self._queue:
                    return None
                if self._queue and self._running == 0 and hasattr(self.backend, "evict_idle"):
                    # nothing runs but the head does not fit: cached idle plans hold the memory
                    if self.backend.evict_idle():
                        continue
                self._cv.wait(timeout=0.05)

    def _slot_loop(self, slot):
        while True:
            item = self._take()
            if item is None:
                return
            req, res, fut, plan = item
            res.slot = slot
            res.t_start = time.perf_counter()
            try:
                out = self.backend.solve(plan, req, slot)
                res.kappa = out["kappa"]
                res.n_sweeps = out.get("n_sweeps", 0)
                res.n_sweeps_fp64 = out.get("n_sweeps_fp64", 0)
                res.status = "ok" if out.get("converged", True) else "not_converged"
            except Exception as e:  # noqa: BLE001
                res.status, res.error = "error", f"{type(e).__name__}: {e}"
            res.t_done = time.perf_counter()
            self.backend.release(plan)
            with self._cv:
                self._used -= res.footprint
                self._running -= 1
                self._cv.notify_all()
            self._finish(res, fut)

    def _finish(self, res, fut):
        with self._cv:
            self.results.append(res)
        fut.set_result(res)


def replay(server: Server, requests, rate: Optional[float] = None, seed: int = 0):
    """Submit `requests` with Poisson arrivals at `rate` per second (None: all at once); wait for all."""
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    t = 0.0
    futs = []
    for r in requests:
        if rate:
            t += rng.exponential(1.0 / rate)
            r.arrival = t
            delay = t0 + t - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
        futs.append(server.submit(r))
    return [f.result() for f in futs]


def summarize(results, wall_s: Optional[float] = None) -> dict:
    ok = [r for r in results if r.status in ("ok", "not_converged")]
    lat = np.array([r.latency for r in ok]) if ok else np.zeros(1)
    if wall_s is None and ok:
        wall_s = max(r.t_done for r in ok) - min(r.t_submit for r in results)
    errs = sorted({r.error for r in results if r.status == "error" and r.error})
    return {"completed": len(ok), "rejected": sum(r.status == "rejected" for r in results),
            "errors": sum(r.status == "error" for r in results), "error_messages": errs[:3],
            "solves_per_s": len(ok) / wall_s if wall_s else 0.0,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_queue_ms": float(np.mean([r.queue_time for r in ok]) * 1e3) if ok else 0.0,
            "wall_s": wall_s}
