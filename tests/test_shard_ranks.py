"""Direction sharding of the sweep over ranks (the multi-GPU design): two gloo ranks on the CPU.

Each rank sweeps the ordinates of a contiguous block of directions (all MFPs of a direction together, so a
direction's schedule lives on one rank); the one exchange per sweep is the sum over ranks of the partial
reductions: lattice temperature DeltaT', wall temperatures T_B' and flux J (all-reduce), with the
per-ordinate K and S of disjoint directions gathered by the same sum.  The reference does this reduction over
its worker processes through shared memory (openbte/objects.py:86-101), splitting the ordinates as here
(openbte/utils.py:209).  The per-rank sweep is the oracle's exact per-ordinate solve restricted to the
rank's directions; the all-reduced result must equal the one-rank pass.  The diffuse-wall re-emission
weights are normalised over all ordinates (openbte/bte.py:73-78), so every rank uses the global ones.
"""
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _state(case_name, seed):
    from conftest import load_case
    import bte_oracle
    geo, mat, bcs, ek, _ = load_case(case_name)
    ops = bte_oracle.setup_operators(geo, mat, bcs)
    solver = bte_oracle.OrdinateSolver(geo, np.asarray(mat.mfps, dtype=np.float64), ops)
    ct = bte_oracle.contact_terms(geo, mat, bcs, ek)
    rng = np.random.default_rng(seed)
    dT = 0.3 * rng.standard_normal(geo.n_elems)
    TB = 0.3 * rng.standard_normal(len(ops["i_diffuse"]))
    return ops, solver, mat, ct, dT, TB


def _rank(rank, world, port, case_name, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    sys.path.insert(0, os.path.dirname(here))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch
    import torch.distributed as dist
    import bte_oracle
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ops, solver, mat, ct, dT, TB = _state(case_name, seed=9)
        shard = np.array_split(np.arange(ops["n_angles"]), world)[rank]
        parts = bte_oracle._one_pass(ops, solver, mat, ct, dT, TB, True, dirs=shard)
        out = []
        for a in parts:                      # DeltaT', T_B', J, K, S: one sum over ranks each
            t = torch.tensor(np.asarray(a), dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.SUM)
            out.append(t.numpy())
        q.put((rank, len(shard), [o.tolist() for o in out]))
    finally:
        dist.destroy_process_group()


def test_direction_shards_all_reduce_to_the_one_rank_sweep():
    import bte_oracle
    name = "a600"
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, name, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted((q.get(timeout=300) for _ in procs), key=lambda x: x[0])
    finally:
        for p in procs:
            p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    assert sum(g[1] for g in got) == 16 and min(g[1] for g in got) > 0
    ops, solver, mat, ct, dT, TB = _state(name, seed=9)
    full = bte_oracle._one_pass(ops, solver, mat, ct, dT, TB, True)
    for rank, _, parts in got:
        for a, b in zip(parts, full):
            b = np.asarray(b)
            np.testing.assert_allclose(np.asarray(a), b, rtol=0, atol=1e-13 * max(np.abs(b).max(), 1.0))
