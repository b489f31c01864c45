"""Benchmark: served FP32+refine kappa_eff solves/s and p50/p99 latency vs plain FP64, on one GB300.

Default workload (``c3_serve_512x50``): the seeded serving stream of 512 2D requests arriving as a
Poisson process at 50 requests/s.  Each request draws porosity U(0.05, 0.40), a circular or square
pore (50/50), a seeded periodic Delaunay mesh of log-uniform 2k-60k triangles, 48 or 96 directions and
30-100 MFPs of the synthetic lognormal material (bulk 150 W/mK).  Meshes are built before the timed
region (the reference's ``BTE_RTA`` takes a built ``Mesh`` too); everything after that is timed:
each request goes through ``serving.Server`` (host schedule build, HBM admission, table upload, solve
on one of the GPU slots, kappa_eff back to the host).  The stream is timed as one run; a "step" is
1/K of it (``config.requests_per_step``).  Also measured: FP64 solves of every request (the kappa
error of each served result), plain FP64 one at a time on a seeded subset, the same requests the
reference arm solves, and the resident 60k-triangle solve of the 2D scale-up config (``resident_c1``,
which also carries the sweep kernel's roofline).

Other workloads (``--workload``): ``c1_60k_100x96`` (one kappa_eff solve per step on a resident plan),
``c2_100k_30x16x32`` (3D), ``c4_inverse_128x50x64`` (inverse-design gradient).

``--impl reference`` times the unmodified reference (``baseline/_ref``, imported through
``oracle/ref_loader.py``) on the host cores: for the serving stream, one request per step (Fourier
first guess, then ``BTE_RTA`` with its own process pool on all cores, bte_rtol 1e-6, which keeps its
kappa within 1e-4 of its converged value) on a seeded sample of the same stream restricted to meshes
of at most 4,000 triangles (full reference solves of the larger requests take minutes each).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload ...]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (n_elements, n_mfp, n_dir, porosity, pore, seed); 3D: n_dir = (n_theta, n_phi)
    "c1_60k_100x96": (60000, 100, 96, 0.25, "square", 1),
    "c0_2k_30x48": (2000, 30, 48, 0.25, "square", 1),
    "c2_100k_30x16x32": (100000, 30, (16, 32), 0.10, "sphere", 1),
    # the 3D benchmark mesh with 4 x 8 directions: device tables of ~0.5 GB, for profiler captures
    "c2_100k_30x4x8": (100000, 30, (4, 8), 0.10, "sphere", 1),
    # the 2D cell at a third of the benchmark size: FP64 tables with their reciprocal table ~2 GB, for
    # profiler captures of the FP64 sweep
    "c1_20k_100x96": (20000, 100, 96, 0.25, "square", 1),
    # inverse design: pixels per side, n_mfp, n_dir, density-field seed
    "c4_inverse_128x50x64": (128, 50, 64, None, "pixels", 0),
}
# serving streams: name -> (requests, arrival rate per second)
SERVE = {"c3_serve_512x50": (512, 50.0)}
# largest mesh of the requests the reference arm solves in full (one step each)
REF_MAX_TRI = 4000
# the reference's tolerance for the served workload: with the Fourier first guess, bte_rtol 1e-6 keeps its
# kappa within 3e-6 of its converged value on the 2k-triangle cell (1e-5: 1.5e-4; its default 1e-4: 1e-3)
REF_BTE_RTOL = 1e-6
L2_BYTES = 129 * 1024 * 1024
# DRAM bytes of one sweep launch (dram__bytes.sum.per_second x gpu__time_duration of one ncu capture of
# `bench.py --workload <w> --profile-sweeps 2` with the current kernel; profiles/bte_sweep_*.md); the
# iterate stays in shared memory, so this is about an eighth of the algorithmic bytes
SWEEP_DRAM_BYTES = {("c1_60k_100x96", "fp32"): 2.873e8, ("c1_60k_100x96", "fp64"): 5.1e9,
                    ("c1_20k_100x96", "fp64"): 1.70e9, ("c2_100k_30x4x8", "fp32"): 2.501e8}
SWEEP_DRAM_SOURCE = {("c1_60k_100x96", "fp32"): "profiles/bte_sweep_fp32_c1_60k_100x96.md",
                     ("c1_60k_100x96", "fp64"): "profiles/bte_sweep_fp64_c1_20k_100x96.md (scaled by elements)",
                     ("c1_20k_100x96", "fp64"): "profiles/bte_sweep_fp64_c1_20k_100x96.md",
                     ("c2_100k_30x4x8", "fp32"): "profiles/bte_sweep_fp32_c2_110k_30x4x8.md"}


def problem(workload):
    from openbte_gb300 import objects as O
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.mesh import mesh_from_cell
    from openbte_gb300.material import synthetic_isotropic_2d
    n_tri, n_mfp, n_dir, phi, pore, seed = WORKLOADS[workload]
    if pore == "sphere":
        from openbte_gb300.geometry import porous_cube_3d
        from openbte_gb300.material import synthetic_isotropic_3d
        cell = porous_cube_3d(n_tri, phi, seed=seed)
        geo = mesh_from_cell(cell)
        mat = synthetic_isotropic_3d(n_mfp, n_dir[0], n_dir[1])
        bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0, "Periodic_z": 0}, diffuse="Boundary")
        ek = O.EffectiveThermalConductivity(normalization=-1.0 / cell.size, contact="Periodic_x")
        return geo, mat, bcs, ek
    geo = mesh_from_cell(porous_cell_2d(n_tri, phi, pore, seed=seed))
    mat = synthetic_isotropic_2d(n_mfp, n_dir)
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    return geo, mat, bcs, ek


def _stream_mesh(args):
    """Mesh of one serving request (built in a worker process)."""
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.mesh import mesh_from_cell
    n_tri, phi, pore, seed = args
    return mesh_from_cell(porous_cell_2d(n_tri, phi, pore, seed=seed))


def stream_spec(n_req, seed=0):
    """Seeded request mix: (triangles, porosity, pore, mesh seed, directions, MFPs) per request, in arrival order:
    porosity U(0.05, 0.40), circle/square pore 50/50, log-uniform 2k-60k triangles, 48 or 96 directions,
    30-100 MFPs."""
    rng = np.random.default_rng(seed)
    spec = []
    for i in range(n_req):
        phi = float(rng.uniform(0.05, 0.40))
        pore = "circle" if rng.random() < 0.5 else "square"
        n_tri = int(round(math.exp(rng.uniform(math.log(2000), math.log(60000)))))
        n_dir = int(rng.choice([48, 96]))
        n_mfp = int(rng.integers(30, 101))
        spec.append((n_tri, phi, pore, 1000 + i, n_dir, n_mfp))
    return spec


def reference_sample(k, seed=0, max_tri=REF_MAX_TRI):
    """The first k requests of the seeded stream with at most max_tri triangles: [(request index, spec)]."""
    out = []
    for i, sp in enumerate(stream_spec(max(4096, 64 * k), seed)):
        if sp[0] <= max_tri:
            out.append((i, sp))
            if len(out) == k:
                break
    return out


def serving_stream(n_req, seed=0, only=None):
    """Requests of the seeded stream (meshes built in a spawn pool, before any timing); `only`: request
    indices to build (default: the first n_req)."""
    import multiprocessing as mp
    from openbte_gb300 import objects as O
    from openbte_gb300.material import synthetic_isotropic_2d
    from openbte_gb300.serving import Request
    spec = stream_spec(max(n_req, 1 + max(only)) if only else n_req, seed)
    idx = list(only) if only else list(range(n_req))
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        meshes = pool.map(_stream_mesh, [spec[i][:4] for i in idx])
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    reqs = []
    for i, geo in zip(idx, meshes):
        n_tri, phi, pore, _, n_dir, n_mfp = spec[i]
        reqs.append(Request(geo, synthetic_isotropic_2d(n_mfp, n_dir), bcs, ek, rid=i,
                            tag={"n_elems": geo.n_elems, "phi": phi, "pore": pore, "n_dir": n_dir, "n_mfp": n_mfp}))
    return reqs


def serve_requests(reqs, precision, rtol, device, slots, builders, preparers, rate=None, seed=1, restart=30):
    """Replay `reqs` through a fresh server (Poisson arrivals at `rate`, None: all at once).
    Returns (results, wall seconds, server, backend)."""
    import torch
    from openbte_gb300.serving import GPUBackend, Server, replay
    for r in reqs:
        r.precision = precision
        r.rtol = rtol
    be = GPUBackend(device=device, restart=restart)
    srv = Server(backend=be, slots=slots, builders=builders, preparers=preparers)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = replay(srv, reqs, rate=rate, seed=seed)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    srv.close()
    return res, wall, srv, be


def run_serve(args, dev, world, rank, local):
    """The serving stream (configs[3]): served FP32+refine against plain FP64 on the same GPU."""
    import torch
    from openbte_gb300 import _lib
    from openbte_gb300.serving import summarize
    lib = _lib.load()
    n_req, rate = SERVE[args.workload]
    os.environ["OBTE_HOST_THREADS"] = str(args.host_threads)
    # GPU-slot threads sleep while their solve runs instead of spinning on a core: the cores go to the
    # threads that build and upload the next requests' plans
    os.environ["OBTE_BLOCKING_SYNC"] = "1"
    pool = dict(device=local, slots=args.slots, builders=args.builders, preparers=args.preparers,
                restart=args.serve_restart)
    t0 = time.time()
    reqs = serving_stream(n_req)
    mesh_s = time.time() - t0
    # warm-up: a few requests of the stream through a throwaway server in each precision
    warm = reqs[:max(3, args.warmup)]
    for prec in ("fp32_refine", "fp64"):
        serve_requests(warm, prec, args.serve_rtol, **pool)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    barrier()
    l0 = lib.obte_launch_count()
    b0 = lib.obte_h2d_bytes()
    with Clocks(local) as clk:
        res, wall, srv, be = serve_requests(reqs, "fp32_refine", args.serve_rtol, rate=rate, seed=1, **pool)
    launches = lib.obte_launch_count() - l0
    h2d = lib.obte_h2d_bytes() - b0
    barrier()
    summ = summarize(res, wall)
    t_job = max_over_ranks(wall, world, dev)
    ok = [r for r in res if r.status == "ok"]
    value = world * len(ok) / t_job
    # FP64 solve of every request: the kappa error of each served FP32+refine result
    res64, wall64, srv64, _ = serve_requests(reqs, "fp64", 1e-9, rate=None, **pool)
    k64 = {r.rid: r.kappa for r in res64 if r.status == "ok"}
    errs = [abs(r.kappa - k64[r.rid]) / abs(k64[r.rid]) for r in ok if r.rid in k64]
    # plain FP64 one request at a time (one slot, back to back) on a seeded subset, same tolerance as the
    # served FP32+refine form
    sub = reqs[::args.fp64_subset_every]
    res1, wall1, _, _ = serve_requests(sub, "fp64", args.serve_rtol, rate=None, **dict(pool, slots=1))
    lat1 = np.array([r.t_done - r.t_start for r in res1 if r.status == "ok"])
    fp64_rate = len(lat1) / wall1
    # the requests the reference arm solves (its timed steps), served here the same two ways
    ref_ids = [i for i, _ in reference_sample(args.warmup + args.steps)][args.warmup:]
    same = serving_stream(0, only=ref_ids)
    r_one, w_one, _, _ = serve_requests(same, "fp32_refine", args.serve_rtol, rate=None, **dict(pool, slots=1))
    r_srv, w_srv, _, _ = serve_requests(same, "fp32_refine", args.serve_rtol, rate=None, **pool)
    # bytes: plan tables the library copied host -> device in the timed run (plus each request's initial state
    # set on the device); per-ordinate kappa K read back per request
    d2h = sum(r.tag["n_dir"] * r.tag["n_mfp"] * 8 for r in reqs)
    K = args.steps
    line = {
        "metric": "kappa_eff solves/s (served FP32+refine, <=1e-4 kappa error)",
        "value": value, "unit": "solves/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": t_job * 1e3 / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded request stream: meshes, materials, Poisson arrivals)",
        "config": {"workload": args.workload, "requests": n_req, "rate_per_s": rate,
                   "requests_per_step": n_req / K, "step": "1/K of the stream, timed as one run",
                   "precision": "fp32_refine", "rtol": args.serve_rtol,
                   "unknowns_per_sweep_mean": float(np.mean([r.tag["n_elems"] * r.tag["n_dir"] * r.tag["n_mfp"]
                                                             for r in reqs])),
                   "server": {"slots": args.slots, "builders": args.builders, "preparers": args.preparers,
                              "host_threads_per_build": args.host_threads},
                   "value_scope": "end to end: host meshes in, kappa_eff out (schedule build, table upload, "
                                  "solve, read-back all inside the timed region)",
                   "l2": "every request is a new mesh (plans, tables and Krylov vectors of 2k-60k-element "
                         "problems; the stream's working set is far above L2)",
                   "parallelism": f"replicas{world}" if world > 1 else "single"},
        "latency_ms": {"p50": summ["p50_ms"], "p99": summ["p99_ms"]},
        "served": {k: summ[k] for k in ("completed", "rejected", "errors", "error_messages", "mean_queue_ms", "wall_s")}
                  | {"max_concurrent": srv.max_concurrent, "max_hbm_held_gb": srv.max_held / 1e9,
                     "sweeps_per_request_mean": float(np.mean([r.n_sweeps for r in ok])) if ok else None,
                     "mesh_build_s_untimed": mesh_s},
        "kappa_rel_err_vs_fp64": {"max": float(max(errs)) if errs else None,
                                  "median": float(np.median(errs)) if errs else None, "requests": len(errs),
                                  "fp64_rtol": 1e-9},
        "fp64_one_at_a_time": {"solves_per_s": fp64_rate, "requests": len(lat1),
                               "subset": f"every {args.fp64_subset_every}th request of the stream",
                               "rtol": args.serve_rtol,
                               "latency_ms": {"p50": float(np.percentile(lat1, 50) * 1e3),
                                              "p99": float(np.percentile(lat1, 99) * 1e3)} if len(lat1) else None},
        "fp64_served_rtol1e-9": {"solves_per_s": len(k64) / wall64, "wall_s": wall64},
        "speedup_vs_fp64_one_at_a_time": value / fp64_rate if fp64_rate else None,
        "reference_sample": {"requests": ref_ids, "max_triangles": REF_MAX_TRI,
                             "one_at_a_time_solves_per_s": len(r_one) / w_one,
                             "served_solves_per_s": len(r_srv) / w_srv},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": int(h2d / K),
                "d2h_bytes_per_step": int(d2h / K)},
        "gpu_launches": int(round(launches / K)),
        "clocks": clk.summary(),
    }
    return line


def algorithmic_sweep_bytes(geo, mat, b_T):
    """Per-sweep algorithmic bytes: N_cells*N_ord*b_T + N_dir*(4*N_cells + 8*F_d)."""
    n = geo.n_elems
    n_mfp, n_dir = np.asarray(mat.t_coeff).shape
    F_d = 2 * len(geo.internal)
    return n * n_mfp * n_dir * b_T + n_dir * (4 * n + 8 * F_d)


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx = float(p[1])
            except ValueError:
                continue
            for name, v in zip(names, p[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(geo, mat, bcs, ek, budget_s=20.0, seed=0):
    """Time the oracle (the reference algorithm: per-ordinate SuperLU factor + solves) on a seeded
    ordinate sample of the same workload and extrapolate to solves/s on all host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bte_oracle
    from openbte_gb300 import objects as O
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.mesh import mesh_from_cell
    from openbte_gb300.material import synthetic_isotropic_2d
    cores = os.cpu_count() or 1
    n_mfp, n_dir = np.asarray(mat.t_coeff).shape
    if geo.dim == 3:
        return {"value": None, "unit": "solves/s", "cores": cores, "kind": "port",
                "sample": "not measured: SuperLU of one ordinate of the periodic operator on the 3D mesh takes "
                          "minutes (~290 s at 110k tetrahedra), beyond the bench's budget"}
    # source iterations the reference needs for <=1e-4 kappa error, measured on a small proxy cell
    pg = mesh_from_cell(porous_cell_2d(600, 0.25, "square", seed=5))
    pm = synthetic_isotropic_2d(8, 16)
    pb = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    pe = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    hist = []
    kref = bte_oracle.bte_rta(pg, pm, pb, effective_thermal_conductivity=pe, bte_rtol=1e-12, bte_max_iter=3000)[0]
    bte_oracle.bte_rta(pg, pm, pb, effective_thermal_conductivity=pe, bte_rtol=0, bte_max_iter=200, history=hist)
    n_iter = next((i + 1 for i, (k, _) in enumerate(hist) if abs(k - kref) / abs(kref) <= 1e-4), len(hist))
    ops = bte_oracle.setup_operators(geo, mat, bcs)
    solver = bte_oracle.OrdinateSolver(geo, np.asarray(mat.mfps, dtype=np.float64), ops)
    rng = np.random.default_rng(seed)
    t_fac, t_sol, k = [], [], 0
    t_start = time.time()
    B = np.ones(geo.n_elems)
    while time.time() - t_start < budget_s and k < 64:
        q, m = int(rng.integers(n_dir)), int(rng.integers(n_mfp))
        t0 = time.perf_counter()
        solver.solve(q, m, B)
        t1 = time.perf_counter()
        solver.solve(q, m, B)
        t2 = time.perf_counter()
        t_fac.append(t1 - t0 - (t2 - t1))
        t_sol.append(t2 - t1)
        solver.cache.clear()
        k += 1
    per_ord = float(np.mean(t_fac) + n_iter * np.mean(t_sol))
    t_solve = n_mfp * n_dir * per_ord / cores
    return {"value": 1.0 / t_solve, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": f"{k} seeded ordinates (of {n_mfp * n_dir}) of the same mesh: SuperLU factor "
                      f"{np.mean(t_fac) * 1e3:.1f} ms + {n_iter} solves x {np.mean(t_sol) * 1e3:.2f} ms "
                      f"(iterations for <=1e-4 kappa error measured on a 600-triangle proxy), "
                      f"extrapolated to {n_mfp * n_dir} ordinates over {cores} cores",
            "seconds_per_solve": t_solve}


def density_field(n, seed):
    """Seeded smoothed Gaussian random field on an n x n periodic grid, mapped to [0, 1] (pixel order i*n + j)."""
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((n, n))
    k = np.fft.fftfreq(n)
    kk = k[:, None] ** 2 + k[None, :] ** 2
    z = np.real(np.fft.ifft2(np.fft.fft2(z) * np.exp(-kk * (n / 8.0) ** 2)))
    return ((z - z.min()) / (z.max() - z.min())).reshape(-1)


def cpu_baseline_inverse(n_full, n_mfp_full, n_dir_full, budget_s=20.0):
    """The oracle's TIM solve + adjoint gradient (sparse direct solve, one core) on small seeded pixel
    grids of the same model, extrapolated linearly in unknowns to the full problem."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import tim_oracle
    from openbte_gb300.material import lognormal_kappa
    n, nm, nq = 8, 4, 8
    mfps = np.logspace(0, 4, nm)
    mat = tim_oracle.material(mfps, lognormal_kappa(mfps), nq)
    grid = tim_oracle.pixel_grid(n, 100.0)
    rho = density_field(n, 1)
    t0, k = time.time(), 0
    while k < 1 or (time.time() - t0 < budget_s / 2 and k < 5):
        tim_oracle.kappa_and_gradient(rho, grid, mat, method="adjoint")
        k += 1
    per = (time.time() - t0) / k
    scale = (n_full ** 2 * n_mfp_full * n_dir_full) / (n * n * nm * nq)
    return {"value": 1.0 / (per * scale), "unit": "gradient evals/s", "cores": 1, "kind": "port",
            "sample": f"{n}x{n} pixels, {nm} MFPs x {nq} directions (oracle sparse direct solve + explicit "
                      f"adjoint, {per:.2f} s each), extrapolated linearly in unknowns by {scale:.0f}x"}


def run_inverse(args, dev):
    """Config 4: kappa_eff and dkappa/drho of a 128^2 pixel cell (50 MFPs x 64 directions) per step."""
    import torch
    from openbte_gb300 import _lib
    from openbte_gb300.inverse import IsotropicMaterial, PixelSolver
    n, n_mfp, n_dir, _, _, seed = WORKLOADS[args.workload]
    lib = _lib.load()
    rho = density_field(n, seed)
    # a design loop: every step is a new density field (the base field plus a seeded perturbation), so
    # every step replaces the transmissions of the solver's cached plan
    fields = [np.clip(rho + 0.1 * (density_field(n, seed + 1 + i) - 0.5), 0.0, 1.0)
              for i in range(args.warmup + args.steps)]
    mat = IsotropicMaterial.lognormal(n_mfp, n_dir)
    # --warm-start: each field's solve starts from the previous field's solution, as the reference's design
    # loop reuses its previous solution (openbte/inverse/bte.py:234-236)
    solver = PixelSolver(n, mat, size=100.0, precision=args.precision, rtol=1e-8, restart=100,
                         warm_start=args.warm_start)
    if args.profile_gradients:
        out = []
        for i in range(args.profile_gradients):
            t0 = time.perf_counter()
            k, g = solver.kappa_and_gradient(rho if i == 0 else fields[i % len(fields)])
            g.cpu()
            out.append({"ms": (time.perf_counter() - t0) * 1e3, "sweeps": solver.last_info.n_sweeps, "kappa": k})
        print(json.dumps({"profile_gradients": out, "workload": args.workload, "precision": args.precision}))
        return
    for i in range(args.warmup):
        solver.kappa_and_gradient(fields[i])
    torch.cuda.synchronize()
    l0 = lib.obte_launch_count()
    lat, kaps, sweeps = [], [], []
    with Clocks(dev.index or 0) as clk:
        for i in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            k, g = solver.kappa_and_gradient(fields[args.warmup + i])   # host rho in; kappa and gradient to the host
            gh = g.cpu().numpy()
            lat.append(time.perf_counter() - t0)
            kaps.append(k)
            sweeps.append(solver.last_info.n_sweeps)
    launches = (lib.obte_launch_count() - l0) / args.steps
    info = solver.last_info
    upload_bytes = solver.last_upload_bytes
    ref = PixelSolver(n, mat, size=100.0, precision="fp64", rtol=1e-10, restart=100, reuse_plan=False)
    kap64, _ = ref.kappa_and_gradient(fields[-1])
    t = float(np.median(lat))
    line = {
        "metric": "inverse-design gradient evals/s (kappa_eff + dkappa/drho over all pixels, FP32+refine)",
        "value": 1.0 / t, "unit": "gradient evals/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded smoothed Gaussian random field)",
        "config": {"workload": args.workload, "pixels": n * n, "n_mfp": n_mfp, "n_dir": n_dir,
                   "unknowns_per_sweep": n * n * n_mfp * n_dir, "precision": args.precision, "rtol": 1e-8,
                   "l2": "inputs and per-ordinate field (210 MB) larger than L2", "parallelism": "single",
                   "fields": "a new density field every step (base field + 0.1 x seeded field); one PixelSolver, "
                             "its plan built once and its transmissions replaced per field",
                   "warm_start": bool(args.warm_start),
                   "acceleration": "diffusion-synthetic (OBTE_DSA=0 turns it off)"
                                   if os.environ.get("OBTE_DSA", "1") != "0" else "off (OBTE_DSA=0)"},
        "kappa_eff": kaps[-1], "kappa_fp64": kap64, "kappa_rel_err_vs_fp64": abs(kaps[-1] - kap64) / abs(kap64),
        "sweeps_per_eval": float(np.median(sweeps)), "fp64_sweeps_per_eval": info.n_sweeps_fp64,
        "gradient_abs_max": float(np.abs(gh).max()),
        "e2e": {"value": 1.0 / t, "unit": "gradient evals/s",
                "h2d_bytes_per_step": int(n * n * 8 + upload_bytes),
                "d2h_bytes_per_step": int(n * n * 8 + 2 * n * n * 8)},
        "gpu_launches": int(round(launches)),
        "clocks": clk.summary(),
    }
    if args.fd_pixels > 0:
        # adjoint gradient against central differences on seeded random pixels.  The solves are refined to
        # 1e-12 (a step of h = 1e-3 moves kappa by ~1e-4 relative, so kappa must be far more accurate than the
        # 1e-4 bar); pixels are drawn where rho - h > 0 and rho + h <= 1 keep the transmission in (0, 1].
        fd_solver = PixelSolver(n, mat, size=100.0, precision="fp32_refine", rtol=1e-13, restart=100,
                                max_sweeps=6000)
        k0, g0 = fd_solver.kappa_and_gradient(rho)
        g0 = g0.cpu().numpy()
        # step h_p = min(1e-3, rho_p / 300): t(rho) is steep at small densities, where the largest
        # gradients are, so the step must stay well below rho_p (truncation ~ (h/rho)^2 ~ 1e-5); kappa is refined
        # to 1e-13 so that its error over 2 h stays near 1e-5 of the gradient; rho_p >= 1e-6, rho_p + h <= 1
        ok = (rho >= 1e-6) & (rho <= 1 - 1e-3)
        rng = np.random.default_rng(123)
        gscale = float(np.percentile(np.abs(g0), 99))   # robust scale (the largest entries are isolated)

        def fd_at(pi):
            hp = min(1e-3, rho[pi] / 300.0)
            r1, r2 = rho.copy(), rho.copy()
            r1[pi] += hp
            r2[pi] -= hp
            return (fd_solver.kappa_and_gradient(r1)[0] - fd_solver.kappa_and_gradient(r2)[0]) / (2 * hp)

        # (a) uniformly random pixels: most sit where the gradient is tiny, so compare on the gradient's scale
        pa = rng.choice(np.nonzero(ok)[0], args.fd_pixels, replace=False)
        fa = np.array([fd_at(pi) for pi in pa])
        # (b) random pixels among the top quartile of |dkappa/drho|: relative error per pixel
        sig = np.nonzero(ok & (np.abs(g0) >= np.percentile(np.abs(g0[ok]), 75)))[0]
        pb = rng.choice(sig, min(args.fd_pixels, len(sig)), replace=False)
        fb = np.array([fd_at(pi) for pi in pb])
        rel = np.abs(g0[pb] - fb) / np.abs(fb)
        line["finite_difference_check"] = {
            "h": "min(1e-3, rho/300)", "rtol": 1e-13,
            "random_pixels": int(len(pa)),
            "random_max_abs_err_over_p99_grad": float(np.abs(g0[pa] - fa).max() / gscale),
            "significant_pixels": int(len(pb)),
            "significant_max_rel_err": float(rel.max()), "significant_median_rel_err": float(np.median(rel)),
            "significant_vector_rel_err": float(np.linalg.norm(g0[pb] - fb) / np.linalg.norm(fb))}
        # A pixel's density moves kappa by ~2 h g / kappa ~ 1e-7 relative at these steps (16,384 pixels share
        # it), so a central difference at h amplifies the solves' error by 1e7; Richardson extrapolation of two
        # larger steps, (4 fd(h1 / 2) - fd(h1)) / 3 with h1 = min(1e-2, rho / 30), cancels the h^2 truncation
        # term while dividing the noise amplification by ~10.
        def fd_h(pi, hp):
            r1, r2 = rho.copy(), rho.copy()
            r1[pi] += hp
            r2[pi] -= hp
            return (fd_solver.kappa_and_gradient(r1)[0] - fd_solver.kappa_and_gradient(r2)[0]) / (2 * hp)

        okr = ok & (rho <= 1 - 1e-2)
        pr = [pi for pi in pb if okr[pi]]
        h1 = np.array([min(1e-2, rho[pi] / 30.0) for pi in pr])
        f1 = np.array([fd_h(pi, h) for pi, h in zip(pr, h1)])
        f2 = np.array([fd_h(pi, h / 2) for pi, h in zip(pr, h1)])
        fr = (4 * f2 - f1) / 3
        relr = np.abs(g0[pr] - fr) / np.abs(fr)
        line["finite_difference_check"]["richardson"] = {
            "h1": "min(1e-2, rho/30) and h1/2", "pixels": len(pr),
            "max_rel_err": float(relr.max()), "median_rel_err": float(np.median(relr)),
            "vector_rel_err": float(np.linalg.norm(g0[pr] - fr) / np.linalg.norm(fr)),
            "max_rel_err_fd_h1_half_alone": float((np.abs(g0[pr] - f2) / np.abs(f2)).max())}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_inverse(n, n_mfp, n_dir)
    print(json.dumps(line))


def max_over_ranks(x, world, device):
    """The largest x over the ranks of the process group (one replica per rank; the slowest sets the time)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reference_serve(args, steps, warmup, n_process=None):
    """Unmodified reference solves, one request per step, on the seeded sample of the serving stream.

    Each step is the reference's own pipeline for one request: ``Fourier`` (openbte/fourier.py:15-185)
    for the first guess, then ``BTE_RTA`` (openbte/bte.py:19-271) at bte_rtol 1e-6 with its forking
    process pool (openbte/utils.py:186-219) on every host core.  The request's mesh (this package's
    seeded cell written as msh2 and read by the reference's own ``get_mesh``) and material are built
    before the step, as the GPU arm's meshes are.  Returns (per-step seconds, kappas, request ids, cores)."""
    import contextlib
    import io
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_loader
    from openbte_gb300.geometry import porous_cell_2d, write_msh2
    from openbte_gb300.material import synthetic_isotropic_2d
    if not ref_loader.available():
        return None
    R = ref_loader.load(in_process=False)
    cores = n_process or (os.cpu_count() or 1)
    sample = reference_sample(warmup + steps)
    bcs = R.objects.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = R.objects.EffectiveThermalConductivity(normalization=-1.0, contact="Periodic_x")
    times, kappas, ids = [], [], []
    argv = sys.argv
    with tempfile.TemporaryDirectory() as tmp:
        for k, (rid, (n_tri, phi, pore, seed, n_dir, n_mfp)) in enumerate(sample):
            path = write_msh2(porous_cell_2d(n_tri, phi, pore, seed=seed), os.path.join(tmp, f"r{rid}"))
            with contextlib.redirect_stdout(io.StringIO()):
                geo = R.mesh.get_mesh(path[:-4])
            mat = R.objects.Material(*synthetic_isotropic_2d(n_mfp, n_dir))
            sys.argv = [argv[0], "-np", str(cores)]      # the reference's runner reads its worker count here
            try:
                t0 = time.perf_counter()
                with contextlib.redirect_stdout(io.StringIO()):
                    f = R.fourier.Fourier(geo, mat.thermal_conductivity, bcs, effective_thermal_conductivity=ek)
                    b = R.bte.BTE_RTA(geo, mat, bcs, fourier=f, effective_thermal_conductivity=ek,
                                      bte_rtol=REF_BTE_RTOL)
                dt = time.perf_counter() - t0
            finally:
                sys.argv = argv
            if k >= warmup:
                times.append(dt)
                kappas.append(float(b.kappa_eff))
                ids.append(rid)
    return times, kappas, ids, cores


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload in SERVE:
        t0 = time.time()
        out = reference_serve(args, args.steps, args.warmup)
        if out is None:
            print(json.dumps({"impl": "reference", "unavailable": "the reference is not installed under baseline/_ref"}))
            return
        times, kappas, ids, cores = out
        v = len(times) / sum(times)
        sample = (f"{len(times)} requests of the seeded serving stream with at most {REF_MAX_TRI} triangles "
                  f"(request ids {ids}), each a full unmodified reference solve (Fourier + BTE_RTA at bte_rtol "
                  f"{REF_BTE_RTOL}, {cores} worker processes), after {args.warmup} warm-up requests; larger "
                  f"requests of the stream are not run (minutes each), so this is the reference on the "
                  f"stream's smallest requests")
        print(json.dumps({"impl": "reference", "metric": "kappa_eff solves/s (served FP32+refine, <=1e-4 kappa error)",
                          "value": v, "unit": "solves/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded request stream)",
                          "config": {"workload": args.workload, "sample_max_triangles": REF_MAX_TRI,
                                     "bte_rtol": REF_BTE_RTOL},
                          "latency_ms": {"p50": float(np.percentile(times, 50) * 1e3),
                                         "p99": float(np.percentile(times, 99) * 1e3)},
                          "kappa_eff": kappas,
                          "cpu_baseline": {"value": v, "unit": "solves/s", "cores": cores, "kind": "reference",
                                           "sample": sample},
                          "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                          "wall_s": time.time() - t0}))
        return
    if args.workload.startswith("c4_"):
        n, n_mfp, n_dir = WORKLOADS[args.workload][:3]
        t0 = time.time()
        cbs = [cpu_baseline_inverse(n, n_mfp, n_dir, budget_s=max(2.0, 20.0 / max(1, args.steps + args.warmup)))
               for _ in range(args.warmup + args.steps)]
        v = float(np.median([c["value"] for c in cbs[args.warmup:]]))
        print(json.dumps({"impl": "reference", "metric": "inverse-design gradient evals/s (kappa_eff + dkappa/drho "
                          "over all pixels, FP32+refine)", "value": v, "unit": "gradient evals/s", "n_gpus": 0,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic", "config": {"workload": args.workload},
                          "cpu_baseline": {"value": v, "unit": "gradient evals/s", "cores": 1, "kind": "port",
                                           "sample": cbs[-1]["sample"]},
                          "e2e": {"value": v, "unit": "gradient evals/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}, "wall_s": time.time() - t0}))
        return
    geo, mat, bcs, ek = problem(args.workload)
    if geo.dim == 3:
        print(json.dumps({"impl": "reference", "unavailable": "the reference's per-ordinate SuperLU on the "
                          "3D benchmark mesh takes minutes per ordinate (~290 s at 110k tetrahedra)"}))
        return
    t0 = time.time()
    steps = []
    for _ in range(args.warmup + args.steps):
        cb = cpu_baseline(geo, mat, bcs, ek, budget_s=max(2.0, 20.0 / max(1, args.steps + args.warmup)))
        steps.append(cb)
    vals = [c["value"] for c in steps[args.warmup:]]
    v = float(np.median(vals))
    last = steps[-1]
    line = {"impl": "reference", "metric": "kappa_eff solves/s (served FP32+refine, <=1e-4 kappa error)",
            "value": v, "unit": "solves/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 / v, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": {"workload": args.workload},
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": last["cores"], "kind": last["kind"],
                             "sample": last["sample"]},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.time() - t0}
    print(json.dumps(line))


def run_resident(args, dev, world, rank, local):
    """One kappa_eff solve per step on a resident plan (c1 / c2 workloads); the profile options print
    their own line and return None."""
    import torch
    import torch.distributed as dist
    from openbte_gb300 import _lib
    from openbte_gb300.bte import BTE_RTA, solve_plan
    from openbte_gb300.fourier import Fourier, get_fourier_plan
    from openbte_gb300.runtime import HostProblem, get_plan
    lib = _lib.load()

    geo, mat, bcs, ek = problem(args.workload)
    if args.profile_fourier:
        t0 = time.time()
        fplan = get_fourier_plan(geo, mat.thermal_conductivity, bcs, ek, [], local)
        fplan_s = time.time() - t0
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        half = args.profile_fourier // 2
        for i in range(args.profile_fourier):
            if i == half:
                ev[0].record()
            finfo, _, _ = fplan.solve(device=local)
        ev[1].record()
        ev[1].synchronize()
        print(json.dumps({"profile_fourier": args.profile_fourier, "workload": args.workload,
                          "plan_s": fplan_s, "ms_per_solve": ev[0].elapsed_time(ev[1]) / max(1, args.profile_fourier - half),
                          "outer_iterations": finfo.n_iter, "cg_iterations": finfo.n_cg, "kappa": finfo.kappa,
                          "preconditioner": "jacobi" if os.environ.get("OBTE_FOURIER_JACOBI", "0") != "0" else "amg"}))
        return
    hp = HostProblem(geo, mat, bcs, ek)
    t0 = time.time()
    plan = get_plan(hp, local)
    plan_s = time.time() - t0
    n_mfp, n_dir = np.asarray(mat.t_coeff).shape
    if args.profile_solves:
        dT0 = torch.zeros(geo.n_elems, dtype=torch.float64, device=dev)
        out = []
        for i in range(args.profile_solves):
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record()
            info, *_ = solve_plan(plan, dT0, precision=args.precision, rtol=args.rtol, max_sweeps=2000, restart=40)
            ev[1].record()
            ev[1].synchronize()
            out.append({"ms": ev[0].elapsed_time(ev[1]), "sweeps": info.n_sweeps, "kappa": info.kappa_eff})
        pb, ps, pms = C.c_int32(), C.c_int32(), C.c_double()
        _lib.check(lib.obte_bte_precond_info(plan.handle, C.byref(pb), C.byref(ps), C.byref(pms)), "precond_info")
        print(json.dumps({"profile_solves": out, "workload": args.workload, "precision": args.precision,
                          "preconditioner": {"blocks": pb.value, "setup_sweeps": ps.value, "setup_ms": pms.value}}))
        return
    if args.profile_sweeps:
        u = torch.zeros(plan.nu, dtype=torch.float64, device=dev)
        uo = torch.zeros_like(u)
        ms = {}
        for prec in ("fp32", "fp64", "df"):
            if os.environ.get("OBTE_DETERMINISTIC") and prec == "df":
                continue
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            for i in range(args.profile_sweeps):
                if i == args.profile_sweeps // 2:
                    ev[0].record()
                _lib.check(lib.obte_bte_sweep(plan.handle, _lib.PRECISION[prec], C.c_void_p(u.data_ptr()),
                                              C.c_void_p(uo.data_ptr()), 1), "sweep")
            ev[1].record()
            ev[1].synchronize()
            ms[prec] = ev[0].elapsed_time(ev[1]) / max(1, args.profile_sweeps - args.profile_sweeps // 2)
        print(json.dumps({"profile_sweeps": args.profile_sweeps, "workload": args.workload,
                          "ms_per_sweep": ms, "group_env": os.environ.get("OBTE_SWEEP_G")}))
        return
    dT0 = torch.zeros(geo.n_elems, dtype=torch.float64, device=dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    fplan = get_fourier_plan(geo, mat.thermal_conductivity, bcs, ek, [], local)

    def one(prec):
        # one kappa_eff solve: the BTE source iteration to its fixed point from DeltaT = 0
        # (kappa_eff does not depend on the first guess; the Fourier pipeline is timed separately)
        return solve_plan(plan, dT0, precision=prec, rtol=args.rtol, max_sweeps=2000, restart=40)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # reference kappa at FP64 for the error check (also warms the FP64 tables)
    info64, *_ = one("fp64")
    kappa64 = info64.kappa_eff
    for _ in range(args.warmup):
        one(args.precision)
    barrier()
    lat = []
    l0 = lib.obte_launch_count()
    with Clocks(local) as clk:
        barrier()
        t_start = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            info, dT, J, K, S = one(args.precision)
            e1.record(stream)
            e1.synchronize()
            lat.append(e0.elapsed_time(e1) / 1e3)
        barrier()
        t_total = time.perf_counter() - t_start
    launches = (lib.obte_launch_count() - l0) / args.steps
    kappa = info.kappa_eff
    t_step = max_over_ranks(max(sum(lat), 1e-12) / args.steps, world, dev)
    value = world / t_step

    # plain FP64 on the same GPU
    lat64 = []
    for _ in range(max(1, args.fp64_steps)):
        flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        i64, *_ = one("fp64")
        e1.record(stream)
        e1.synchronize()
        lat64.append(e0.elapsed_time(e1) / 1e3)

    # e2e through the public API with host arrays
    e2e_lat = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        r = BTE_RTA(geo, mat, bcs, effective_thermal_conductivity=ek, bte_rtol=args.rtol,
                    precision=args.precision, restart=40, max_sweeps=2000)
        e2e_lat.append(time.perf_counter() - t1)
    # host->device: the initial temperature handed to BTE_RTA; device->host: BTE temperature,
    # flux, per-ordinate kappa and suppression
    h2d = geo.n_elems * 8
    d2h = geo.n_elems * 8 * (1 + np.asarray(mat.sigma).shape[2]) + 2 * n_mfp * n_dir * 8
    # the reference pipeline on the device: Fourier first guess, then BTE from it
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e2 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    finfo, T0, _ = fplan.solve(device=local)
    e1.record(stream)
    pinfo, *_ = solve_plan(plan, T0, precision=args.precision, rtol=args.rtol, max_sweeps=2000, restart=40)
    e2.record(stream)
    e2.synchronize()
    fourier_ms = e0.elapsed_time(e1)
    pipeline_ms = e0.elapsed_time(e2)

    # roofline of the dominant kernel: one sweep of every ordinate
    fp32 = args.precision != "fp64"
    u = torch.zeros(plan.nu, dtype=torch.float64, device=dev)
    uo = torch.zeros_like(u)
    prec_code = _lib.PRECISION["fp32" if fp32 else "fp64"]
    for _ in range(3):
        lib.obte_bte_sweep(plan.handle, prec_code, C.c_void_p(u.data_ptr()), C.c_void_p(uo.data_ptr()), 1)
    nsw = 20
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record(stream)
    for _ in range(nsw):
        _lib.check(lib.obte_bte_sweep(plan.handle, prec_code, C.c_void_p(u.data_ptr()), C.c_void_p(uo.data_ptr()), 1))
    ev[1].record(stream)
    ev[1].synchronize()
    t_sweep = ev[0].elapsed_time(ev[1]) / 1e3 / nsw
    bytes_sweep = algorithmic_sweep_bytes(geo, mat, 4 if fp32 else 8)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = bytes_sweep / t_sweep / 1e9

    pb, ps, pms = C.c_int32(), C.c_int32(), C.c_double()
    _lib.check(lib.obte_bte_precond_info(plan.handle, C.byref(pb), C.byref(ps), C.byref(pms)), "precond_info")
    line = {
        "metric": "kappa_eff solves/s (served FP32+refine, <=1e-4 kappa error)",
        "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if fp32 else "f64", "data": "synthetic",
        "config": {"workload": args.workload, "n_elems": geo.n_elems, "n_mfp": int(n_mfp), "n_dir": int(n_dir),
                   "unknowns_per_sweep": int(geo.n_elems * n_mfp * n_dir), "precision": args.precision,
                   "rtol": args.rtol, "l2": "flushed between steps (2x L2 write)",
                   "parallelism": f"replicas{world}" if world > 1 else "single"},
        "latency_ms": {"p50": float(np.percentile(lat, 50) * 1e3), "p99": float(np.percentile(lat, 99) * 1e3)},
        "pipeline": {"ms": pipeline_ms, "fourier_ms": fourier_ms, "fourier_outer_iterations": finfo.n_iter,
                     "fourier_cg_iterations": finfo.n_cg, "kappa_fourier": finfo.kappa,
                     "bte_sweeps_from_fourier_guess": pinfo.n_sweeps,
                     "kappa_rel_diff_vs_zero_guess": abs(pinfo.kappa_eff - info.kappa_eff) / abs(info.kappa_eff)},
        "fp64": {"solves_per_s": 1.0 / float(np.median(lat64)), "ms": float(np.median(lat64) * 1e3),
                 "sweeps": i64.n_sweeps},
        "speedup_vs_fp64": float(np.median(lat64) / t_step),
        "kappa_eff": kappa, "kappa_fp64": kappa64, "kappa_rel_err_vs_fp64": abs(kappa - kappa64) / abs(kappa64),
        "sweeps_per_solve": info.n_sweeps, "fp64_sweeps_per_solve": info.n_sweeps_fp64,
        "e2e": {"value": 1.0 / float(np.median(e2e_lat)), "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(round(launches)),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": SWEEP_DRAM_BYTES.get((args.workload, "fp32" if fp32 else "fp64")),
                     "traffic_source": SWEEP_DRAM_SOURCE.get((args.workload, "fp32" if fp32 else "fp64")),
                     "kernel": "bte_sweep_kernel", "ms_per_launch": t_sweep * 1e3,
                     "algorithmic_bytes": int(bytes_sweep), "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
        "clocks": clk.summary(),
        "plan_build_s": plan_s,
        # periodic-inflow preconditioner, built once per plan on its first (warm-up) solve
        "preconditioner": {"blocks": pb.value, "setup_sweeps": ps.value, "setup_ms": pms.value},
        "wall_timed_s": t_total,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(geo, mat, bcs, ek)
        line["cpu_baseline"].pop("seconds_per_solve", None)
    return line

def _resident_args(args):
    """The resident 60k-triangle solve of the 2D scale-up config, run beside the serving stream."""
    a = argparse.Namespace(**vars(args))
    a.workload = "c1_60k_100x96"
    a.steps = max(3, min(args.steps, 10))
    a.warmup = 3
    a.precision = "fp32_refine"
    a.rtol = 1e-7
    a.fp64_steps = 1
    a.no_cpu_baseline = True
    return a


def reference_cpu_sample(args, steps=3):
    """cpu_baseline of the serving line: the reference arm on a bounded sample, in a child process (the
    reference forks its workers, which must not happen in a process that holds a CUDA context)."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", args.workload,
           "--steps", str(steps), "--warmup", "1", "--sample-only"]
    try:
        out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=dict(os.environ, RANK="0"))
        for l in reversed(out.stdout.splitlines()):
            if l.startswith("{"):
                d = json.loads(l)
                return d.get("cpu_baseline")
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"{type(e).__name__}: {e}"}
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c3_serve_512x50", choices=sorted(WORKLOADS) + sorted(SERVE))
    ap.add_argument("--precision", default="fp32_refine", choices=["fp32_refine", "fp32", "fp64"])
    ap.add_argument("--rtol", type=float, default=1e-7)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-restart", type=int, default=30, help="GMRES restart length of served solves")
    ap.add_argument("--serve-rtol", type=float, default=1e-5,
                    help="serving stream: residual tolerance of each request (FP32+refine and one-at-a-time FP64)")
    ap.add_argument("--slots", type=int, default=12, help="serving stream: concurrent GPU solves")
    ap.add_argument("--builders", type=int, default=8, help="serving stream: host threads building plans")
    ap.add_argument("--preparers", type=int, default=8, help="serving stream: host threads uploading tables")
    ap.add_argument("--host-threads", type=int, default=2, help="serving stream: host threads per plan build")
    ap.add_argument("--fp64-subset-every", type=int, default=8,
                    help="serving stream: plain FP64 one at a time on every n-th request")
    ap.add_argument("--cold-start", dest="warm_start", action="store_false",
                    help="config 4: start each density field's solve from zero instead of the previous field's "
                         "solution (the default warm start is the reference design loop's own x0 reuse)")
    ap.add_argument("--fd-pixels", type=int, default=0,
                    help="config 4: also check dkappa/drho against central differences on this many pixels")
    ap.add_argument("--profile-sweeps", type=int, default=0,
                    help="only build the plan and run this many FP32 and FP64 sweeps (for ncu captures)")
    ap.add_argument("--profile-fourier", type=int, default=0,
                    help="only build the Fourier plan and run this many Fourier first-guess solves")
    ap.add_argument("--profile-solves", type=int, default=0,
                    help="only build the plan and run this many kappa_eff solves (for launch lists)")
    ap.add_argument("--profile-gradients", type=int, default=0,
                    help="config 4: only run this many gradient evaluations on new density fields (for launch lists)")
    ap.add_argument("--sample-only", action="store_true",
                    help="reference arm: a bounded cpu_baseline sample (the warm-up may be shorter than 3 steps)")
    args = ap.parse_args()
    if args.warmup < 3 and not args.sample_only:
        args.warmup = 3
    if args.impl == "reference":
        return reference_arm(args)

    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.workload.startswith("c4_"):
        if rank == 0:
            run_inverse(args, dev)
        if world > 1:
            dist.destroy_process_group()
        return

    if args.workload in SERVE:
        line = run_serve(args, dev, world, rank, local)
        if rank == 0:
            os.environ.pop("OBTE_BLOCKING_SYNC", None)
            res = run_resident(_resident_args(args), dev, 1, 0, local)
            if res is not None:
                line["roofline"] = dict(res["roofline"], workload="c1_60k_100x96 (resident plan)")
                line["resident_c1"] = {k: res[k] for k in ("value", "ms_per_step", "latency_ms", "fp64",
                                                          "speedup_vs_fp64", "kappa_rel_err_vs_fp64", "sweeps_per_solve",
                                                          "fp64_sweeps_per_solve", "e2e", "pipeline", "preconditioner")}
                line["resident_c1"]["config"] = res["config"]
            if not args.no_cpu_baseline:
                line["cpu_baseline"] = reference_cpu_sample(args)
    else:
        line = run_resident(args, dev, world, rank, local)
    if rank == 0 and line is not None:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
