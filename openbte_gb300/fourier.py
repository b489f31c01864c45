"""``Fourier`` drop-in: the diffusive first guess solved on the GPU.

Same signature and ``SolverResults`` dictionary as the reference
(openbte/fourier.py:15-185). The SuperLU factorisation becomes a device
conjugate-gradient solve; the deferred non-orthogonal correction, the
least-squares gradient and the diffusive kappa run as kernels
(``csrc/fourier.cu``).

Like the reference, the returned ``kappa_eff`` is 0: its ``while ... else``
(openbte/fourier.py:179-180) resets the value after every normal exit of the
loop. The diffusive kappa that the reference prints is in
``aux['kappa_eff']``.
"""
from __future__ import annotations

import ctypes as C
from collections import OrderedDict

import numpy as np

from . import _lib
from .objects import SolverResults
from .runtime import context, fingerprint, ptr

PIN = 10   # element pinned when no mixed boundary exists (openbte/fourier.py:43)

_PLANS: "OrderedDict[str, FourierPlan]" = OrderedDict()


class FourierPlan:
    def __init__(self, geometry, kappa, bcs, ek, heat_source, device=0):
        self.lib = _lib.load()
        self.ctx = context(device)
        g = geometry
        dim = int(g.dim)
        n = int(g.n_elems)
        nv = int(len(g.elems[0]))
        a = {}
        a["sem"] = np.ascontiguousarray(g.side_elem_map, dtype=np.int64)
        a["na"] = np.ascontiguousarray(g.normal_areas, dtype=np.float64)
        a["dists"] = np.ascontiguousarray(g.dists, dtype=np.float64)
        a["vol"] = np.ascontiguousarray(g.elem_volumes, dtype=np.float64)
        a["areas"] = np.ascontiguousarray(g.side_areas, dtype=np.float64)
        a["w"] = np.ascontiguousarray(g.interp_weights, dtype=np.float64)
        a["gw"] = np.ascontiguousarray(g.gradient_weights, dtype=np.float64)
        esm = g.elem_side_map
        a["esm"] = np.ascontiguousarray(np.array([esm[e] for e in range(n)], dtype=np.int64))
        a["internal"] = np.ascontiguousarray(g.internal, dtype=np.int64)
        # periodic: every region of the mesh, with its jump (openbte/objects.py:346-355)
        ps, pj = [], []
        for region, sides in g.periodic_sides.items():
            jump = bcs.periodic[region]
            ps.append(np.asarray(sides, dtype=np.int64))
            pj.append(np.full(len(sides), float(jump)))
        a["per"] = np.ascontiguousarray(np.concatenate(ps) if ps else np.zeros(0, np.int64))
        a["perj"] = np.ascontiguousarray(np.concatenate(pj) if pj else np.zeros(0))
        ms, mv, mh = [], [], []
        for key, c in bcs.mixed.items():
            sides = np.asarray(g.side_physical_regions[key], dtype=np.int64)
            ms.append(sides)
            mv.append(np.full(len(sides), float(c["value"])))
            mh.append(np.full(len(sides), float(c["boundary_conductance"])))
        a["mix"] = np.ascontiguousarray(np.concatenate(ms) if ms else np.zeros(0, np.int64))
        a["mixv"] = np.ascontiguousarray(np.concatenate(mv) if mv else np.zeros(0))
        a["mixh"] = np.ascontiguousarray(np.concatenate(mh) if mh else np.zeros(0))
        a["kappa"] = np.ascontiguousarray(np.asarray(kappa, dtype=np.float64)[:dim, :dim])
        p = _lib.FourierProblem()
        p.dim, p.n_elems, p.n_sides, p.elem_nv = dim, n, a["sem"].shape[0], nv
        p.side_elem_map = ptr(a["sem"], C.c_int64)
        p.normal_areas = ptr(a["na"])
        p.dists = ptr(a["dists"])
        p.elem_volumes = ptr(a["vol"])
        p.side_areas = ptr(a["areas"])
        p.interp_weights = ptr(a["w"])
        p.gradient_weights = ptr(a["gw"])
        p.elem_side_map = ptr(a["esm"], C.c_int64)
        p.n_internal, p.internal = len(a["internal"]), ptr(a["internal"], C.c_int64)
        p.n_periodic, p.periodic_sides, p.periodic_jump = len(a["per"]), ptr(a["per"], C.c_int64), ptr(a["perj"])
        p.n_mixed, p.mixed_sides = len(a["mix"]), ptr(a["mix"], C.c_int64)
        p.mixed_value, p.mixed_conductance = ptr(a["mixv"]), ptr(a["mixh"])
        p.contact_kind = _lib.CONTACT_NONE
        if ek is not None:
            bc = bcs.get_bc_by_name(ek.contact)
            p.normalization = float(ek.normalization)
            if bc == "Mixed":
                a["contact"] = np.ascontiguousarray(g.side_physical_regions[ek.contact], dtype=np.int64)
                p.contact_kind = _lib.CONTACT_MIXED
                p.contact_alpha = float(bcs.mixed[ek.contact]["value"])
                p.contact_conductance = float(bcs.mixed[ek.contact]["boundary_conductance"])
            else:
                a["contact"] = np.ascontiguousarray(g.periodic_sides[ek.contact], dtype=np.int64)
                p.contact_kind = _lib.CONTACT_PERIODIC
                p.contact_alpha = float(bcs.periodic[ek.contact])
            p.n_contact, p.contact_sides = len(a["contact"]), ptr(a["contact"], C.c_int64)
        p.kappa = ptr(a["kappa"])
        if heat_source is not None and len(heat_source) > 0:
            a["hs"] = np.ascontiguousarray(heat_source, dtype=np.float64)
            p.heat_source = ptr(a["hs"])
        p.pin_elem = PIN
        self._keep = a
        h = C.c_void_p()
        _lib.check(self.lib.obte_fourier_plan_create(self.ctx, C.byref(p), C.byref(h)), "obte_fourier_plan_create")
        self.handle = h
        self.n, self.dim = n, dim

    def solve(self, max_iter=40, rtol=1e-8, cg_rtol=1e-13, device=0):
        import torch
        dev = f"cuda:{device}"
        T = torch.empty(self.n, dtype=torch.float64, device=dev)
        J = torch.empty((self.n, self.dim), dtype=torch.float64, device=dev)
        o = _lib.FourierOpts()
        o.max_iter, o.rtol, o.cg_rtol, o.cg_max_iter = int(max_iter), float(rtol), float(cg_rtol), 50000
        info = _lib.FourierInfo()
        _lib.check(self.lib.obte_fourier_solve(self.handle, C.byref(o), C.c_void_p(T.data_ptr()),
                                               C.c_void_p(J.data_ptr()), C.byref(info)), "obte_fourier_solve")
        return info, T, J

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.lib.obte_fourier_plan_destroy(self.handle)
        except Exception:
            pass


def get_fourier_plan(geometry, kappa, bcs, ek, heat_source, device=0):
    key = fingerprint(geometry.side_elem_map, geometry.normal_areas, geometry.elem_volumes, geometry.internal,
                      np.asarray(kappa), repr(sorted(bcs.periodic.items())), repr(sorted(bcs.mixed.items(), key=str)),
                      repr(ek), None if heat_source is None or len(heat_source) == 0 else np.asarray(heat_source),
                      device)
    pl = _PLANS.get(key)
    if pl is None:
        pl = FourierPlan(geometry, kappa, bcs, ek, heat_source, device)
        _PLANS[key] = pl
        while len(_PLANS) > 8:
            _PLANS.popitem(last=False)
    else:
        _PLANS.move_to_end(key)
    return pl


def Fourier(geometry, thermal_conductivity, boundary_conditions, effective_thermal_conductivity=None,
            heat_source=[], global_temperature=0, modified_fourier=False, fourier_max_iter=40, fourier_rtol=1e-8,
            verbose=True, **kwargs) -> SolverResults:
    """Steady heat conduction (openbte/fourier.py:15-185) on the GPU."""
    if modified_fourier:
        raise NotImplementedError("modified_fourier (experimental in the reference) is not implemented on the GPU")
    device = int(kwargs.get("device", 0))
    pl = get_fourier_plan(geometry, thermal_conductivity, boundary_conditions, effective_thermal_conductivity,
                          heat_source, device)
    info, T, J = pl.solve(fourier_max_iter, fourier_rtol, kwargs.get("cg_rtol", 1e-13), device)
    if verbose:
        print("Kappa (Fourier): {:E}, Iterations {:n}".format(info.kappa, info.n_iter))
    variables = {"Temperature_Fourier": {"data": T.cpu().numpy(), "units": "K"},
                 "Flux_Fourier": {"data": J.cpu().numpy() * 1e9, "units": "W/m/m"}}
    return SolverResults(kappa_eff=0, variables=variables,
                         aux={"kappa_eff": info.kappa, "n_iter": info.n_iter, "n_cg": info.n_cg})
