"""Device runtime: one library context per CUDA device, plan construction and caching.

Device memory for inputs and outputs comes from PyTorch tensors (the library
only sees raw pointers); work runs on torch's current stream of the device.
"""
from __future__ import annotations

import ctypes as C
import hashlib
from collections import OrderedDict

import numpy as np

from . import _lib

_CTX = {}


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("openbte_gb300 needs a CUDA device; there is no CPU fallback")
    return torch


def context(device: int = 0, stream=None):
    """Library context for `device` bound to a CUDA stream handle (default: torch's current stream).

    Contexts are cached per (device, stream) so threads that use their own streams get their own
    contexts.
    """
    torch = _torch()
    lib = _lib.load()
    if stream is None:
        stream = torch.cuda.current_stream(device).cuda_stream
    key = (device, int(stream or 0))
    ctx = _CTX.get(key)
    if ctx is None:
        h = C.c_void_p()
        _lib.check(lib.obte_context_create(device, C.c_void_p(stream), C.byref(h)), "obte_context_create")
        ctx = h
        _CTX[key] = ctx
    return ctx


def _i64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64))


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def ptr(a, ctype=C.c_double):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def fingerprint(*arrays) -> str:
    # SHA-256: hardware-accelerated on x86-64 and Arm hosts (about 2.5x blake2b here); arrays are hashed
    # through the buffer protocol, without a copy
    h = hashlib.sha256()
    for a in arrays:
        if a is None:
            h.update(b"none")
            continue
        if isinstance(a, (int, float, str, bool)):
            h.update(repr(a).encode())
            continue
        a = np.ascontiguousarray(np.asarray(a))
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.reshape(-1).view(np.uint8))
    return h.hexdigest()[:32]


class HostProblem:
    """Mesh + boundary conditions + material resolved to flat arrays (the C ABI structs)."""

    def __init__(self, geo, mat, bcs, effective_thermal_conductivity=None, heat_source=None):
        dim = int(geo.dim)
        self.dim = dim
        self.n_elems = int(geo.n_elems)
        self.sem = _i64(geo.side_elem_map)
        self.na = _f64(geo.normal_areas)
        self.vol = _f64(geo.elem_volumes)
        self.areas = _f64(geo.side_areas)
        self.internal = _i64(geo.internal)
        self.elem_nv = int(len(geo.elems[0]))
        # periodic (openbte/bte.py:100-110): every region named in bcs.periodic
        ps, pj = [], []
        for region, jump in bcs.periodic.items():
            sides = np.asarray(geo.periodic_sides[region], dtype=np.int64)
            ps.append(sides)
            pj.append(np.full(len(sides), float(jump)))
        self.per_sides = _i64(np.concatenate(ps)) if ps else _i64(np.zeros(0))
        self.per_jump = _f64(np.concatenate(pj)) if pj else _f64(np.zeros(0))
        # diffuse walls (openbte/bte.py:68-70)
        if len(bcs.diffuse) > 0:
            self.diffuse = _i64(geo.side_physical_regions[bcs.diffuse])
        else:
            self.diffuse = _i64(np.zeros(0))
        # mixed walls (openbte/bte.py:91-96)
        ms, mv = [], []
        for key, contact in bcs.mixed.items():
            sides = np.asarray(geo.side_physical_regions[key], dtype=np.int64)
            ms.append(sides)
            mv.append(np.full(len(sides), float(contact["value"])))
        self.mix_sides = _i64(np.concatenate(ms)) if ms else _i64(np.zeros(0))
        self.mix_value = _f64(np.concatenate(mv)) if mv else _f64(np.zeros(0))
        # contact (openbte/bte.py:132-158)
        ek = effective_thermal_conductivity
        self.contact_kind = _lib.CONTACT_NONE
        self.contact_sides = _i64(np.zeros(0))
        self.alpha = 0.0
        self.normalization = 0.0
        self.is_nanowire = int(bool(bcs.is_nanowire))
        if ek is not None:
            self.normalization = float(ek.normalization)
            if bcs.is_nanowire:
                self.contact_kind = _lib.CONTACT_NANOWIRE
            else:
                bc = bcs.get_bc_by_name(ek.contact)
                if bc == "Mixed":
                    self.contact_kind = _lib.CONTACT_MIXED
                    self.contact_sides = _i64(geo.side_physical_regions[ek.contact])
                    self.alpha = float(bcs.mixed[ek.contact]["value"])
                else:
                    self.contact_kind = _lib.CONTACT_PERIODIC
                    self.contact_sides = _i64(geo.periodic_sides[ek.contact])
                    self.alpha = float(bcs.periodic[ek.contact])
        self.heat_source = None
        if heat_source is not None:
            self.heat_source = _f64(heat_source.variables["Heat_Source"]["data"])
        # material (openbte/objects.py:500-509)
        self.mfps = _f64(mat.mfps)
        self.vmfp = _f64(mat.vmfp)
        self.sigma = _f64(mat.sigma)
        self.t_coeff = _f64(mat.t_coeff)
        self.n_mfp = int(self.mfps.shape[0])
        self.n_dir = int(self.vmfp.shape[0])
        if self.sigma.shape[:2] != (self.n_mfp, self.n_dir) or self.t_coeff.shape != (self.n_mfp, self.n_dir):
            raise ValueError("material arrays do not match (n_mfp, n_dir)")
        self.hs_coeff = float(getattr(mat, "heat_source_coeff", 0.0) or 0.0)

    def key(self) -> str:
        return fingerprint(self.dim, self.sem, self.na, self.vol, self.internal, self.per_sides, self.per_jump,
                           self.diffuse, self.mix_sides, self.mix_value, self.contact_kind, self.contact_sides,
                           self.alpha, self.normalization, self.is_nanowire, self.heat_source, self.mfps,
                           self.vmfp, self.sigma, self.t_coeff, self.hs_coeff)

    def c_structs(self):
        p = _lib.Problem()
        p.dim = self.dim
        p.n_elems = self.n_elems
        p.n_sides = self.sem.shape[0]
        p.elem_nv = self.elem_nv
        p.side_elem_map = ptr(self.sem, C.c_int64)
        p.normal_areas = ptr(self.na)
        p.elem_volumes = ptr(self.vol)
        p.side_areas = ptr(self.areas)
        p.n_internal = len(self.internal)
        p.internal = ptr(self.internal, C.c_int64)
        p.n_periodic = len(self.per_sides)
        p.periodic_sides = ptr(self.per_sides, C.c_int64)
        p.periodic_jump = ptr(self.per_jump)
        p.n_diffuse = len(self.diffuse)
        p.diffuse_sides = ptr(self.diffuse, C.c_int64)
        p.n_mixed = len(self.mix_sides)
        p.mixed_sides = ptr(self.mix_sides, C.c_int64)
        p.mixed_value = ptr(self.mix_value)
        p.contact_kind = self.contact_kind
        p.n_contact = len(self.contact_sides)
        p.contact_sides = ptr(self.contact_sides, C.c_int64)
        p.contact_alpha = self.alpha
        p.normalization = self.normalization
        p.is_nanowire = self.is_nanowire
        p.heat_source = ptr(self.heat_source) if self.heat_source is not None else None
        m = _lib.MaterialC()
        m.n_mfp = self.n_mfp
        m.n_dir = self.n_dir
        m.dim_dir = self.vmfp.shape[1]
        m.dim_sigma = self.sigma.shape[2]
        m.mfps = ptr(self.mfps)
        m.vmfp = ptr(self.vmfp)
        m.sigma = ptr(self.sigma)
        m.t_coeff = ptr(self.t_coeff)
        m.heat_source_coeff = self.hs_coeff
        return p, m


class Plan:
    """A device-resident sweep plan (orders, level sets, operator tables)."""

    def __init__(self, hp: HostProblem, device: int = 0, host_only: bool = False, stream=None):
        import threading
        self.lib = _lib.load()
        self.device = device
        self.lock = threading.Lock()      # one solve at a time per plan (its scratch is shared)
        self.ctx = None if host_only else context(device, stream)
        self.stream = None if host_only else (stream if stream is not None else
                                              _torch().cuda.current_stream(device).cuda_stream)
        self.hp = hp
        p, m = hp.c_structs()
        h = C.c_void_p()
        _lib.check(self.lib.obte_bte_plan_create(self.ctx, C.byref(p), C.byref(m), C.byref(h)), "obte_bte_plan_create")
        self.handle = h
        n, nd, nx = C.c_int64(), C.c_int64(), C.c_int64()
        _lib.check(self.lib.obte_bte_state_layout(h, C.byref(n), C.byref(nd), C.byref(nx)), "state_layout")
        self.n, self.nd, self.nx = n.value, nd.value, nx.value
        self.nu = self.n + self.nd + self.nx

    def set_stream(self, stream):
        """Issue this plan's later work on `stream` (a raw cudaStream_t handle)."""
        if int(stream or 0) != int(self.stream or 0):
            _lib.check(self.lib.obte_bte_plan_set_stream(self.handle, C.c_void_p(stream)), "set_stream")
            self.stream = stream

    def prepare(self, precision="fp32_refine", restart=30):
        """Upload the device tables `precision` uses and allocate the solver scratch ahead of a solve."""
        _lib.check(self.lib.obte_bte_plan_prepare(self.handle, _lib.PRECISION[precision], int(restart)), "prepare")

    def footprint(self, precision="fp64", restart=30):
        pb, sb = C.c_int64(), C.c_int64()
        _lib.check(self.lib.obte_bte_plan_footprint(self.handle, _lib.PRECISION[precision], restart, C.byref(pb),
                                                    C.byref(sb)), "footprint")
        return pb.value, sb.value

    def precond_bytes(self):
        """(bytes the built periodic-inflow preconditioner holds, upper bound of what building it would
        allocate; 0 once a build was tried)"""
        r, b = C.c_int64(), C.c_int64()
        _lib.check(self.lib.obte_bte_precond_bytes(self.handle, C.byref(r), C.byref(b)), "precond_bytes")
        return r.value, b.value

    def schedule(self, q):
        nl, ns = C.c_int64(), C.c_int64()
        _lib.check(self.lib.obte_bte_schedule(self.handle, q, None, None, C.byref(nl), C.byref(ns)), "schedule")
        order = np.zeros(self.n, dtype=np.int64)
        lp = np.zeros(nl.value + 1, dtype=np.int64)
        _lib.check(self.lib.obte_bte_schedule(self.handle, q, ptr(order, C.c_int64), ptr(lp, C.c_int64), C.byref(nl),
                                              C.byref(ns)), "schedule")
        return order, lp, ns.value

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.lib.obte_bte_plan_destroy(self.handle)
        except Exception:
            pass


_PLANS: "OrderedDict[str, Plan]" = OrderedDict()
PLAN_CACHE_SIZE = 8


def get_plan(hp: HostProblem, device: int = 0) -> Plan:
    key = (hp.key(), device)
    pl = _PLANS.get(key)
    if pl is not None:
        _PLANS.move_to_end(key)
        return pl
    pl = Plan(hp, device)
    _PLANS[key] = pl
    while len(_PLANS) > PLAN_CACHE_SIZE:
        _PLANS.popitem(last=False)
    return pl


def clear_plans():
    _PLANS.clear()
