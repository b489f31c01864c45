"""Continuous-batching kappa_eff server on one GPU.

Requests (mesh, material, boundary conditions, contact) arrive over time and go through four stages:

1. build (host threads): the plan's sweep schedule in C++ and its device footprint (tables + solver
   scratch); a repeated geometry finds its plan in the cache instead;
2. admission: first-fit in arrival order against the HBM budget.  The budget covers every byte the
   server holds on the device: plans that are prepared (running, waiting for a slot, or idle in the
   cache) and reservations of admitted plans not yet prepared.  Idle cached plans are evicted, least
   recently used first, when a request does not fit otherwise.  A request whose footprint alone exceeds
   the budget is rejected (``status='rejected'``) instead of waiting forever;
3. prepare (host threads): device tables packed and uploaded, solver scratch allocated
   (``obte_bte_plan_prepare``), so that GPU time goes to solves only;
4. solve: up to ``slots`` solves run at once, each on its own CUDA stream, so their sweeps and Krylov work
   overlap on the device.  At most ``slots`` prepared requests wait for a slot (``ahead``).

Plans are cached by content: a repeated geometry keeps its mesh, sweep orders, tables and converged
state resident and can warm-start from it; it also builds the periodic-inflow preconditioner on its
second solve, with the preconditioner's memory added to the plan's footprint.

The scheduling logic talks to a backend with the calls ``build``, ``solve`` and ``release`` (and
optionally ``extra_bytes``, ``prepare``, ``resident_bytes``, ``evict_idle``, ``drop_optional``);
:class:`GPUBackend` is the real one, tests plug a fake one to exercise admission and ordering without a
GPU.
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
    t_admitted: float = 0.0
    t_prepared: float = 0.0
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


# sweep-table sets a solve of each precision reads (FP32+refine: FP32 sweeps and one FP64 pass)
_TABLES = {"fp64": {"fp64"}, "fp32": {"fp32"}, "fp32_refine": {"fp32", "fp64"}}
# FP32+refine at this tolerance or looser runs no FP64 sweep (its output pass is FP32, obte_bte_solve), so
# its plan needs only the FP32 tables
_PASS32_RTOL = 5e-6


def _table_precision(req) -> str:
    """The precision whose device tables a request's solve reads."""
    if req.precision == "fp32_refine" and req.rtol >= _PASS32_RTOL:
        return "fp32"
    return req.precision


class _Lease:
    """One request's hold on a cached plan: `use` counts the requests that took the plan before it."""

    __slots__ = ("plan", "use", "bound", "builds_precond")

    def __init__(self, plan, use):
        self.plan = plan
        self.use = use
        self.bound = None             # device bytes this request's preconditioner build may take
        self.builds_precond = False


class GPUBackend:
    """Plans and solves on one CUDA device through the C ABI.

    Every plan the backend holds is in ``_cache`` (least recently used first): busy ones (a request is
    between build and release) and idle ones kept for repeated geometries.  ``resident_bytes`` is the
    device memory of the prepared ones, which the server's admission counts.

    A repeated geometry builds the plan's periodic-inflow preconditioner: the plan's second request
    (``precond_repeats``) reserves the build's upper bound (``Plan.precond_bytes``) at admission, builds it
    during its solve, and the plan's resident bytes then include what the preconditioner keeps.  Requests
    on one plan solve one at a time (a plan has one set of solver vectors)."""

    def __init__(self, device=0, restart=30, max_sweeps=2000, cache_plans=8, precond_repeats=True):
        import torch
        self.torch = torch
        self.device = device
        self.restart = restart
        self.max_sweeps = max_sweeps
        self.cache_plans = cache_plans
        self.precond_repeats = precond_repeats
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
        """Host part of a plan (the C++ schedule) or the cached plan -> (lease, footprint bytes, reused?)"""
        from .runtime import HostProblem
        hp = HostProblem(req.geo, req.mat, req.bcs, req.ek)
        key = hp.key()
        with self._lock:
            pl = self._cache.get(key)
            if pl is not None:
                self._cache.move_to_end(key)
                self._busy[key] += 1
                lease = _Lease(pl, pl.uses)
                pl.uses += 1
                return lease, self._footprint(pl, req), True
        pl = self._new_plan(hp)
        pl.key = key
        pl.tables = set()        # table sets uploaded
        pl.resident = 0          # device bytes once prepared (tables, solver vectors, preconditioner)
        pl.pending = 0           # reserved for a preconditioner build in progress
        pl.uses = 1
        pl.solve_lock = threading.Lock()
        with self._lock:
            other = self._cache.get(key)
            if other is not None:
                # the same geometry was built by another thread meanwhile: share that plan, drop this one
                self._cache.move_to_end(key)
                self._busy[key] += 1
                lease = _Lease(other, other.uses)
                other.uses += 1
                dup, pl = pl, other
            else:
                self._cache[key] = pl
                self._busy[key] += 1
                lease, dup = _Lease(pl, 0), None
        del dup                  # a duplicate plan is destroyed here, outside the lock
        return lease, self._footprint(pl, req), lease.use > 0

    def _new_plan(self, hp):
        from .runtime import Plan
        st = self._stream()
        with self.torch.cuda.stream(st):
            return Plan(hp, self.device, stream=st.cuda_stream)

    def _footprint(self, pl, req):
        a, b = pl.footprint(_table_precision(req), self.restart)
        return int(a + b)

    def _precond_bound(self, lease) -> int:
        """Device bytes the lease's solve may add by building the preconditioner (the plan's second use
        builds it), fixed when first asked (at admission)."""
        if lease.bound is None:
            lease.bound = lease.plan.precond_bytes()[1] if self.precond_repeats and lease.use == 1 else 0
        return lease.bound

    def extra_bytes(self, lease, req) -> int:
        """Device bytes that preparing and solving `req` on the lease's plan adds (0 for a plan already
        prepared for it, unless this solve builds the preconditioner)."""
        pl = lease.plan
        tables = 0 if _TABLES[_table_precision(req)] <= pl.tables else max(0, self._footprint(pl, req) - pl.resident)
        return tables + self._precond_bound(lease)

    def drop_optional(self, lease) -> bool:
        """The lease's solve will not build the preconditioner (its bound does not fit); True if it was to."""
        if self._precond_bound(lease):
            lease.bound = 0
            return True
        return False

    def prepare(self, lease, req: Request):
        """Upload the plan's device tables and allocate its solver scratch (host threads, before a slot);
        from here on the bytes the server reserved for the request count in ``resident_bytes``."""
        pl = lease.plan
        bound = self._precond_bound(lease)
        if not _TABLES[_table_precision(req)] <= pl.tables:
            with pl.solve_lock:          # not while another request solves on the plan
                if not _TABLES[_table_precision(req)] <= pl.tables:
                    self._prepare_plan(pl, req)
                    with self._lock:
                        pl.tables |= _TABLES[_table_precision(req)]
        with self._lock:
            pl.tables |= _TABLES[_table_precision(req)]
            pl.resident = max(pl.resident, self._footprint(pl, req))
            if bound:
                lease.builds_precond = True
                pl.pending += bound

    def _prepare_plan(self, pl, req):
        st = self._stream()
        pl.set_stream(st.cuda_stream)
        pl.prepare(_table_precision(req), self.restart)

    def resident_bytes(self) -> int:
        with self._lock:
            return sum(pl.resident + pl.pending for pl in self._cache.values())

    def _solve_plan(self, pl, req, precond):
        """One solve of `pl` on this thread's stream, waited for -> SolveInfo."""
        from .bte import solve_plan
        torch = self.torch
        st = self._stream()
        pl.set_stream(st.cuda_stream)
        with torch.cuda.stream(st):
            dT0 = torch.zeros(pl.n, dtype=torch.float64, device=f"cuda:{self.device}")
            info, *_ = solve_plan(pl, dT0, precision=req.precision, rtol=req.rtol, max_sweeps=self.max_sweeps,
                                  restart=self.restart, warm_start=req.warm_start, precond=precond)
        st.synchronize()
        return info

    def solve(self, lease, req: Request, slot: int) -> dict:
        pl = lease.plan
        # only the request that reserved the build's memory builds the preconditioner; the others use it
        # once it exists (0: the default policy, whose build on a second solve has then been tried) and
        # otherwise leave it off
        with pl.solve_lock:
            if lease.builds_precond:
                precond = 1
            else:
                precond = 0 if pl.precond_bytes()[1] == 0 else -1
            try:
                info = self._solve_plan(pl, req, precond)
            finally:
                if lease.builds_precond:
                    with self._lock:
                        pl.pending -= lease.bound
                        pl.resident = max(pl.resident, self._footprint(pl, req))
                    lease.builds_precond = False
        return {"kappa": info.kappa_eff, "converged": bool(info.converged), "n_sweeps": info.n_sweeps,
                "n_sweeps_fp64": info.n_sweeps_fp64}

    def release(self, lease):
        """A request is done with the plan: it stays cached (resident) unless the cache is over its size."""
        pl = lease.plan
        victims = []
        with self._lock:
            self._busy[pl.key] -= 1
            while len(self._cache) - len(victims) > self.cache_plans:
                victim = next((k for k in self._cache if self._busy[k] <= 0 and k not in victims), None)
                if victim is None:
                    break
                victims.append(victim)
            dropped = [self._cache.pop(k) for k in victims]
        del dropped       # plans are destroyed here, outside the lock

    def evict_idle(self, need: Optional[int] = None) -> int:
        """Drop idle cached plans, least recently used first, until `need` bytes are freed (None: all of them);
        returns the bytes freed."""
        freed = 0
        with self._lock:
            dropped = []
            for k in list(self._cache):
                if need is not None and freed >= need:
                    break
                if self._busy[k] <= 0:
                    pl = self._cache.pop(k)
                    freed += pl.resident
                    dropped.append(pl)
        del dropped
        return freed


class Server:
    """Continuous batching: host threads build and prepare plans, `slots` GPU workers solve concurrently."""

    def __init__(self, backend=None, slots: int = 4, builders: int = 4, hbm_budget: Optional[int] = None,
                 hbm_fraction: float = 0.7, ahead: Optional[int] = None, preparers: int = 2):
        self.backend = backend if backend is not None else GPUBackend()
        self.slots = slots
        self.ahead = slots if ahead is None else ahead
        self.budget = int(hbm_budget) if hbm_budget is not None else self.backend.budget(hbm_fraction)
        self._builders = cf.ThreadPoolExecutor(max_workers=builders, thread_name_prefix="obte-build")
        self._preparers = cf.ThreadPoolExecutor(max_workers=max(1, preparers), thread_name_prefix="obte-prep")
        self._cv = threading.Condition()
        self._waiting: "collections.deque" = collections.deque()   # built, waiting for admission
        self._ready: "collections.deque" = collections.deque()     # prepared, waiting for a slot
        # device memory: with a backend that reports resident bytes, held = resident + reserved (admitted,
        # not yet prepared); otherwise held = the footprints of the admitted requests
        self._resident = getattr(self.backend, "resident_bytes", None)
        self._reserved = 0
        self._used = 0
        self._admitted = 0          # admitted and not finished
        self._preparing = 0
        self._running = 0
        self._closed = False
        self.results = []
        self.max_concurrent = 0
        self.max_held = 0
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
        # every submitted request is built (and queued) before the slots may see the server closed
        self._builders.shutdown(wait=True)
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        for w in self._workers:
            w.join()
        self._preparers.shutdown(wait=True)

    # -- memory accounting (call with self._cv held) --------------------------------------
    def _held(self) -> int:
        return (self._resident() + self._reserved) if self._resident else self._used

    def _need(self, item) -> int:
        req, res, _, plan = item
        extra = getattr(self.backend, "extra_bytes", None)
        return extra(plan, req) if extra is not None else res.footprint

    def _admit_locked(self):
        """Admit waiting requests (first fit in arrival order) while slots plus look-ahead and memory allow."""
        while self._waiting and self._admitted < self.slots + self.ahead:
            held = self._held()
            pick = None
            for i, item in enumerate(self._waiting):
                need = self._need(item)
                if held + need <= self.budget:
                    pick = (i, item, need)
                    break
            if pick is None:
                evict = getattr(self.backend, "evict_idle", None)
                if evict is not None and evict(held + self._need(self._waiting[0]) - self.budget) > 0:
                    continue
                # nothing admitted will free memory: the head request gives up its optional reservations
                # (a preconditioner build) rather than wait forever
                drop = getattr(self.backend, "drop_optional", None)
                if self._admitted == 0 and drop is not None and drop(self._waiting[0][3]):
                    continue
                return
            i, item, need = pick
            del self._waiting[i]
            item[1].t_admitted = time.perf_counter()
            self._admitted += 1
            if self._resident:
                self._reserved += need
            else:
                self._used += need
            self.max_held = max(self.max_held, self._held())
            self._preparing += 1
            self._preparers.submit(self._prepare, item, need)

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
            self._waiting.append((req, res, fut, plan))
            self._admit_locked()
            self._cv.notify_all()

    def _prepare(self, item, need):
        req, res, fut, plan = item
        err = None
        try:
            prep = getattr(self.backend, "prepare", None)
            if prep is not None:
                prep(plan, req)
        except Exception as e:  # noqa: BLE001
            err = f"{type(e).__name__}: {e}"
        res.t_prepared = time.perf_counter()
        with self._cv:
            self._preparing -= 1
            if self._resident:
                self._reserved -= need       # now counted in the backend's resident bytes
            if err is None:
                self._ready.append(item)
                self._cv.notify_all()
                return
        res.status, res.error, res.t_done = "error", err, time.perf_counter()
        self._done(plan, res, fut, need)

    def _take(self):
        """Next prepared request (arrival order of admission); None when closed and nothing is left."""
        with self._cv:
            while True:
                if self._ready:
                    item = self._ready.popleft()
                    self._running += 1
                    self.max_concurrent = max(self.max_concurrent, self._running)
                    return item
                if self._closed and not self._waiting and not self._preparing and self._admitted == self._running:
                    self._cv.notify_all()
                    return None
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
            with self._cv:
                self._running -= 1
            self._done(plan, res, fut, res.footprint)

    def _done(self, plan, res, fut, need):
        """The request leaves the server: release its plan, free its admission, admit the next ones."""
        self.backend.release(plan)
        with self._cv:
            self._admitted -= 1
            if not self._resident:
                self._used -= need
            self._admit_locked()
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
