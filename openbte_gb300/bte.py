"""``BTE_RTA`` drop-in: the steady-state RTA source iteration on the GPU.

Same signature, inputs and ``SolverResults`` dictionary as the reference
(openbte/bte.py:19-271). The per-ordinate sparse LU solves and the forked
process pool are replaced by device sweeps (see ``csrc/sweep.cu``) driven by
a Krylov solve of the source-iteration fixed point (``csrc/krylov.cu``).

Extra keyword arguments (all optional):
  precision   'fp64' (default) | 'fp32_refine' | 'fp32'
  device      CUDA device index (default 0)
  restart     GMRES restart length
  max_sweeps  cap on transport sweeps (default max(4*bte_max_iter, 400))
"""
from __future__ import annotations

import ctypes as C
import warnings

import numpy as np

from . import _lib
from .objects import SolverResults
from .runtime import HostProblem, get_plan


def _tensor_ptr(t):
    return C.c_void_p(t.data_ptr())


def solve_plan(plan, dT0, precision="fp64", rtol=1e-10, max_sweeps=1000, restart=30, refine_steps=3,
               inner_rtol=1e-5, warm_start=False, precond=0, dsa=0):
    """Solve on a prepared plan. dT0: torch CUDA float64 tensor [n]. Returns (info, dT, J, K, S) tensors.

    precond: periodic-inflow preconditioner, 0 = built on the plan's second solve, 1 = on the first,
    -1 = off.  dsa: diffusion-synthetic acceleration, 1 = on, -1 = off, 0 = on for problems with partially
    transmitting sides.  Neither changes the converged solution, only the number of sweeps.

    Allocations and the solve run on the plan's stream; the plan lock keeps one solve per plan at a time.
    """
    import contextlib
    import torch
    dev = dT0.device
    n = plan.n
    hp = plan.hp
    on_stream = (torch.cuda.stream(torch.cuda.ExternalStream(plan.stream, device=dev)) if plan.stream
                 else contextlib.nullcontext())
    with plan.lock, on_stream:
        dT = torch.empty(n, dtype=torch.float64, device=dev)
        J = torch.empty((n, hp.sigma.shape[2]), dtype=torch.float64, device=dev)
        K = torch.empty((hp.n_mfp, hp.n_dir), dtype=torch.float64, device=dev)
        S = torch.empty((hp.n_mfp, hp.n_dir), dtype=torch.float64, device=dev)
        o = _lib.SolveOpts()
        o.precision = _lib.PRECISION[precision]
        o.rtol = float(rtol)
        o.max_sweeps = int(max_sweeps)
        o.restart = int(restart)
        o.refine_steps = int(refine_steps)
        o.inner_rtol = float(inner_rtol)
        o.warm_start = 1 if warm_start else 0
        o.precond = int(precond)
        o.dsa = int(dsa)
        info = _lib.SolveInfo()
        st = plan.lib.obte_bte_solve(plan.handle, C.byref(o), _tensor_ptr(dT0), _tensor_ptr(dT), _tensor_ptr(J),
                                     _tensor_ptr(K), _tensor_ptr(S), C.byref(info))
    if st not in (_lib.OBTE_OK, _lib.OBTE_ERR_NOT_CONVERGED):
        _lib.check(st, "obte_bte_solve")
    return info, dT, J, K, S


def BTE_RTA(geo, mat, bcs, fourier=None, effective_thermal_conductivity=None, heat_source=None, direct=True,
            bte_max_iter=100, bte_rtol=1e-4, **kwargs) -> SolverResults:
    """Steady-state RTA BTE (openbte/bte.py:19-271) on the GPU.

    ``direct`` is accepted for signature compatibility (the reference's
    ``direct=False`` path is broken, openbte/bte.py:188); ``bte_rtol`` bounds
    the fixed-point residual ‖F(u)-u‖/‖u‖, which is tighter than the
    reference's change-of-norm test at the same value.
    """
    import torch
    precision = kwargs.get("precision", "fp64")
    device = int(kwargs.get("device", 0))
    restart = int(kwargs.get("restart", 30))
    max_sweeps = int(kwargs.get("max_sweeps", max(4 * int(bte_max_iter), 400)))
    hp = HostProblem(geo, mat, bcs, effective_thermal_conductivity, heat_source)
    plan = get_plan(hp, device)
    if fourier is None:
        dT0 = np.zeros(geo.n_elems)
    else:
        dT0 = np.asarray(fourier.variables["Temperature_Fourier"]["data"], dtype=np.float64)
    dT0_d = torch.from_numpy(np.ascontiguousarray(dT0)).to(f"cuda:{device}")
    info, dT, J, K, S = solve_plan(plan, dT0_d, precision=precision, rtol=bte_rtol, max_sweeps=max_sweeps,
                                   restart=restart, refine_steps=kwargs.get("refine_steps", 3),
                                   inner_rtol=kwargs.get("inner_rtol", 1e-5), precond=kwargs.get("precond", 0),
                                   dsa=kwargs.get("dsa", 0))
    if not info.converged:
        warnings.warn(f"BTE_RTA did not reach bte_rtol={bte_rtol} in {info.n_sweeps} sweeps "
                      f"(residual {info.residual:.3e})", RuntimeWarning)
    K_h = K.cpu().numpy()
    kappa_eff = float(np.sum(K_h))
    variables = {"Temperature_BTE": {"data": dT.cpu().numpy(), "units": "K"},
                 "Flux_BTE": {"data": J.cpu().numpy() * 1e9, "units": "W/m/m"}}
    aux = {"suppression": S.cpu().numpy(), "kappa_eff": kappa_eff, "kappa_mode": K_h,
           "n_sweeps": info.n_sweeps, "n_sweeps_fp64": info.n_sweeps_fp64, "n_sweeps_df": info.n_sweeps_df,
           "residual": info.residual,
           "converged": bool(info.converged), "precision": precision}
    return SolverResults(kappa_eff=kappa_eff, variables=variables, aux=aux)
