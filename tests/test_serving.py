"""Serving loop scheduling on CPU with a fake backend: admission by footprint, slot limits, rejection."""
import threading
import time

from openbte_gb300.serving import Request, Server, replay, summarize


class FakeBackend:
    def __init__(self):
        self.lock = threading.Lock()
        self.running = 0
        self.max_running = 0
        self.used = 0
        self.max_used = 0
        self.order = []

    def budget(self, fraction):
        return 100

    def build(self, req):
        time.sleep(0.001)
        return object(), req.tag["foot"], False

    def solve(self, plan, req, slot):
        with self.lock:
            self.running += 1
            self.used += req.tag["foot"]
            self.max_running = max(self.max_running, self.running)
            self.max_used = max(self.max_used, self.used)
            self.order.append(req.rid)
        time.sleep(req.tag["t"])
        with self.lock:
            self.running -= 1
            self.used -= req.tag["foot"]
        return {"kappa": req.tag["kappa"], "converged": True}

    def release(self, plan):
        pass


def _req(rid, foot, t=0.02, kappa=1.0):
    return Request(geo=None, mat=None, bcs=None, ek=None, rid=rid, tag={"foot": foot, "t": t, "kappa": kappa})


def test_slots_and_budget_are_respected():
    be = FakeBackend()
    srv = Server(backend=be, slots=3, builders=2, hbm_budget=100)
    reqs = [_req(i, 30, kappa=float(i)) for i in range(10)]
    res = replay(srv, reqs)
    srv.close()
    assert all(r.status == "ok" for r in res)
    assert [r.kappa for r in res] == [float(i) for i in range(10)]
    assert be.max_running <= 3 and be.max_running >= 2
    assert be.max_used <= 100


def test_oversized_request_is_rejected_not_queued_forever():
    be = FakeBackend()
    srv = Server(backend=be, slots=2, builders=1, hbm_budget=100)
    res = replay(srv, [_req(0, 50), _req(1, 500), _req(2, 50)])
    srv.close()
    st = {r.rid: r.status for r in res}
    assert st == {0: "ok", 1: "rejected", 2: "ok"}
    assert "exceeds the HBM budget" in [r for r in res if r.rid == 1][0].error


def test_first_fit_lets_small_requests_pass_a_large_one():
    be = FakeBackend()
    srv = Server(backend=be, slots=4, builders=1, hbm_budget=100)
    # 0 occupies 60; 1 needs 60 (waits); 2 needs 30 and fits next to 0
    res = replay(srv, [_req(0, 60, t=0.2), _req(1, 60, t=0.01), _req(2, 30, t=0.01)])
    srv.close()
    assert all(r.status == "ok" for r in res)
    assert be.order.index(2) < be.order.index(1)
    s = summarize(res)
    assert s["completed"] == 3 and s["p99_ms"] >= s["p50_ms"]


def test_backend_errors_are_reported_per_request():
    class Failing(FakeBackend):
        def solve(self, plan, req, slot):
            if req.rid == 1:
                raise RuntimeError("boom")
            return super().solve(plan, req, slot)
    srv = Server(backend=Failing(), slots=2, builders=1, hbm_budget=100)
    res = replay(srv, [_req(0, 10), _req(1, 10), _req(2, 10)])
    srv.close()
    st = {r.rid: r.status for r in res}
    assert st == {0: "ok", 1: "error", 2: "ok"}


def test_plan_cache_key_separates_contents():
    """The plan-cache key (SHA-256 over dtype, shape and bytes) is equal for equal arrays and differs when any
    value, dtype or shape differs; non-contiguous views hash like their contiguous copies."""
    import numpy as np
    from openbte_gb300.runtime import fingerprint
    a = np.arange(12.0).reshape(3, 4)
    assert fingerprint(a, 1, None) == fingerprint(a.copy(), 1, None)
    assert fingerprint(a) != fingerprint(a.reshape(4, 3))
    assert fingerprint(a) != fingerprint(a.astype(np.float32))
    b = a.copy()
    b[2, 3] = np.nextafter(b[2, 3], 99)
    assert fingerprint(a) != fingerprint(b)
    assert fingerprint(a.T) == fingerprint(np.ascontiguousarray(a.T))
    assert fingerprint(np.zeros((3, 0))) != fingerprint(np.zeros((0, 3)))
    assert fingerprint(None) != fingerprint(0)


class CachingBackend(FakeBackend):
    """Fake device memory with a plan cache: a plan's bytes are held from prepare until eviction, and idle
    cached plans keep them (the overcommit case: cached plans plus a new request exceed the budget)."""

    def __init__(self):
        super().__init__()
        self.cache = {}            # key -> [bytes held, busy count]
        self.held = 0
        self.max_held = 0
        self.evicted = []

    def build(self, req):
        key = req.tag["key"]
        with self.lock:
            ent = self.cache.setdefault(key, [0, 0])
            ent[1] += 1
        return key, req.tag["foot"], False

    def extra_bytes(self, key, req):
        return 0 if self.cache[key][0] else req.tag["foot"]

    def prepare(self, key, req):
        with self.lock:
            ent = self.cache[key]
            if not ent[0]:
                ent[0] = req.tag["foot"]
                self.held += ent[0]
                self.max_held = max(self.max_held, self.held)

    def resident_bytes(self):
        with self.lock:
            return sum(v[0] for v in self.cache.values())

    def solve(self, plan, req, slot):
        time.sleep(req.tag["t"])
        with self.lock:
            self.order.append(req.rid)
        return {"kappa": req.tag["kappa"], "converged": True}

    def release(self, key):
        with self.lock:
            self.cache[key][1] -= 1

    def evict_idle(self, need=None):
        freed = 0
        with self.lock:
            for k in list(self.cache):
                if need is not None and freed >= need:
                    break
                if self.cache[k][1] <= 0:
                    freed += self.cache[k][0]
                    self.held -= self.cache[k][0]
                    self.evicted.append(k)
                    del self.cache[k]
        return freed


def test_cached_idle_plans_count_against_the_budget():
    be = CachingBackend()
    srv = Server(backend=be, slots=2, builders=1, hbm_budget=100)
    # three plans of 40 stay cached after their solves (120 > 100 once the third is prepared unless the
    # first is evicted); a repeat of plan "a" reuses its resident tables
    reqs = [Request(None, None, None, None, rid=i, tag={"key": k, "foot": 40, "t": 0.01, "kappa": 1.0})
            for i, k in enumerate(["a", "b", "c", "a", "d"])]
    res = []
    for r in reqs:            # one at a time, so that earlier plans are idle in the cache
        res += replay(srv, [r])
    srv.close()
    assert all(r.status == "ok" for r in res)
    assert be.max_held <= 100, be.max_held
    assert srv.max_held <= 100
    assert be.evicted, "idle cached plans must be evicted to admit new ones"


class _PlanStub:
    """Stands in for runtime.Plan on the CPU: tables + solver bytes, and a preconditioner whose build
    takes `bound` bytes and leaves `kept` resident."""

    def __init__(self, bound=500, kept=300):
        self.n = 4
        self.bound, self.kept, self.built = bound, kept, False
        self.prepared = 0
        self.active = 0
        self.overlap = False
        self.peak = 0

    def footprint(self, precision, restart):
        return 100 + (self.kept if self.built else 0), 50

    def precond_bytes(self):
        return (self.kept if self.built else 0), (0 if self.built else self.bound)

    def set_stream(self, s):
        pass

    def prepare(self, precision, restart):
        self.prepared += 1


def _stub_backend(monkeypatch, plan):
    import openbte_gb300.runtime as runtime
    from openbte_gb300.serving import GPUBackend

    class _HP:
        def __init__(self, *a):
            pass

        def key(self):
            return "k"

    monkeypatch.setattr(runtime, "HostProblem", _HP)

    class StubBackend(GPUBackend):
        def __init__(self):
            super().__init__()
            self.seen = []

        def _new_plan(self, hp):
            return plan

        def _stream(self):
            return type("Stream", (), {"cuda_stream": 0})()

        def _solve_plan(self, pl, req, precond):
            pl.active += 1
            pl.overlap |= pl.active > 1
            self.seen.append((req.rid, precond, self.resident_bytes()))
            time.sleep(0.02)
            if precond == 1:
                pl.built = True
            pl.active -= 1
            return type("Info", (), {"kappa_eff": 1.0, "converged": 1, "n_sweeps": 3, "n_sweeps_fp64": 1})()

    return StubBackend()


def test_repeated_plan_reserves_and_builds_the_preconditioner(monkeypatch):
    """GPUBackend's accounting with a stub plan: the second request of a geometry reserves the build's
    bound, builds (precond=1) with it counted as resident, and the plan keeps only the built bytes; the
    requests of one plan never solve at the same time."""
    plan = _PlanStub()
    be = _stub_backend(monkeypatch, plan)
    srv = Server(backend=be, slots=3, builders=2, hbm_budget=10_000)
    res = replay(srv, [Request(None, None, None, None, rid=i) for i in range(4)])
    srv.close()
    assert all(r.status == "ok" for r in res), [r.error for r in res]
    assert not plan.overlap
    assert plan.prepared == 1
    by_rid = {rid: (pc, held) for rid, pc, held in be.seen}
    builder = [rid for rid, (pc, _) in by_rid.items() if pc == 1]
    assert len(builder) == 1
    # while the build ran, its bound was held on top of the plan's 150 bytes
    assert by_rid[builder[0]][1] >= 150 + 500
    assert plan.pending == 0
    assert be.resident_bytes() == 150 + 300
    assert srv.max_held <= 10_000


def test_preconditioner_build_that_cannot_fit_is_dropped(monkeypatch):
    """A budget that holds the plan but never the build's bound: the repeated request gives up the build
    (solves with the preconditioner off) instead of waiting forever."""
    plan = _PlanStub(bound=500)
    be = _stub_backend(monkeypatch, plan)
    srv = Server(backend=be, slots=2, builders=1, hbm_budget=600)
    res = []
    for i in range(3):
        res += replay(srv, [Request(None, None, None, None, rid=i)])
    srv.close()
    assert all(r.status == "ok" for r in res)
    assert srv.max_held <= 600
    assert [pc for _, pc, _ in be.seen] == [-1, -1, -1] and not plan.built


def test_concurrent_builds_of_one_geometry_share_a_plan(monkeypatch):
    """Two builder threads that miss the cache for the same geometry at once end up on one cached plan."""
    import threading as th
    import openbte_gb300.runtime as runtime
    from openbte_gb300.serving import GPUBackend

    class _HP:
        def __init__(self, *a):
            pass

        def key(self):
            return "same"

    monkeypatch.setattr(runtime, "HostProblem", _HP)
    gate = th.Barrier(2)
    made = []

    class Racy(GPUBackend):
        def _new_plan(self, hp):
            gate.wait(timeout=5)          # both threads are past the cache lookup
            p = _PlanStub()
            made.append(p)
            return p

    be = Racy()
    out = []
    ts = [th.Thread(target=lambda: out.append(be.build(Request(None, None, None, None)))) for _ in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert len(made) == 2 and len(be._cache) == 1
    plans = {id(lease.plan) for lease, _, _ in out}
    assert len(plans) == 1
    assert sorted(lease.use for lease, _, _ in out) == [0, 1]
    assert sorted(cached for _, _, cached in out) == [False, True]


def test_loose_refine_requests_prepare_fp32_tables_only(monkeypatch):
    """A FP32+refine request at a tolerance of 5e-6 or looser never sweeps in FP64, so its plan is prepared
    (and its footprint counted) with the FP32 tables only; a tighter one gets both."""
    class RecPlan(_PlanStub):
        def __init__(self):
            super().__init__()
            self.seen = []

        def footprint(self, precision, restart):
            self.seen.append(("footprint", precision))
            return super().footprint(precision, restart)

        def prepare(self, precision, restart):
            self.seen.append(("prepare", precision))
            super().prepare(precision, restart)

    for rtol, want in ((1e-5, "fp32"), (5e-6, "fp32"), (1e-8, "fp32_refine")):
        plan = RecPlan()
        be = _stub_backend(monkeypatch, plan)
        srv = Server(backend=be, slots=1, builders=1, hbm_budget=10_000)
        res = replay(srv, [Request(None, None, None, None, precision="fp32_refine", rtol=rtol)])
        srv.close()
        assert res[0].status == "ok"
        assert {p for _, p in plan.seen} == {want}, (rtol, plan.seen)
        assert ("prepare", want) in plan.seen
