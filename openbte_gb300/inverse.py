"""Inverse design on a periodic pixel grid: kappa_eff(rho) and dkappa_eff/drho on the GPU.

Mirrors the reference's inverse-design solver (openbte/inverse/bte.py:97-255): an n x n periodic
cell of pixel densities rho in [0, 1], a transmission-interface model on every pixel side
(t = harmonic mean of the two densities mapped to [1e-12, 1], openbte/inverse/bte.py:145-151; the
untransmitted part 1 - t is the pixel's own outgoing flux diffusely reflected back) and kappa_eff
along x or y from a unit periodic temperature jump.  The reference is gray (one Knudsen number);
here the material may be MFP-resolved (any isotropic 2D RTA material), with the gray case as the
special case ``Kn=...`` that reproduces the reference's numbers.

The solve is the transport path of this package (FP32 sweeps with FP64 refinement by default) on
the pixel grid as an unstructured quad mesh; the gradient comes from obte_bte_kappa_gradient, which
evaluates the adjoint from the same forward solution (the adjoint sweep of a direction is the
sweep of its reverse), then the chain rule through t(rho) runs here with torch on the device.

``KappaEff`` is a ``torch.autograd.Function`` (kappa_eff forward, dkappa/drho backward);
``get_solver(**options)`` returns ``func(rho) -> ((kappa, 1), jacobian)`` like the reference's
``bte(**options)`` (openbte/inverse/bte.py:201-250).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .material import lognormal_kappa
from .runtime import _torch, context, ptr

K0, K1 = 1e-12, 1.0


def pixel_grid(n: int, size: float = 1.0) -> dict:
    """Periodic n x n pixel grid in the reference's pixel order k = i*n + j
    (openbte/inverse/matinverse.py:494-546: i along +x, j along -y).

    Sides: for every pixel p an x side to (i+1, j) with unit normal (+1, 0), then for every pixel a
    y side to (i, j+1) with unit normal (0, -1); the side's first element is p.  The x sides of
    i = n-1 and the y sides of j = n-1 cross the periodic boundary."""
    h = size / n
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    p = (ii * n + jj).reshape(-1)
    e2x = (((ii + 1) % n) * n + jj).reshape(-1)
    e2y = (ii * n + (jj + 1) % n).reshape(-1)
    sem = np.stack([np.concatenate([p, p]), np.concatenate([e2x, e2y])], axis=1).astype(np.int64)
    normal = np.concatenate([np.tile([1.0, 0.0], (n * n, 1)), np.tile([0.0, -1.0], (n * n, 1))])
    per_x = np.concatenate([(ii == n - 1).reshape(-1), np.zeros(n * n, bool)])
    per_y = np.concatenate([np.zeros(n * n, bool), (jj == n - 1).reshape(-1)])
    return dict(n=n, size=size, h=h, n_elems=n * n, side_elem_map=np.ascontiguousarray(sem),
                normal_areas=np.ascontiguousarray(normal * h), side_areas=np.full(2 * n * n, h),
                elem_volumes=np.full(n * n, h * h), per_x=per_x, per_y=per_y)


def transmission(rho, grid):
    """t per side and dt/drho of its first and second pixel (openbte/inverse/bte.py:145-151)."""
    torch = _torch()
    sem = torch.as_tensor(grid["side_elem_map"], device=rho.device)
    r = K0 + rho * (K1 - K0)
    a, b = r[sem[:, 0]], r[sem[:, 1]]
    t = 2 * a * b / (a + b)
    return t, (K1 - K0) * 0.5 * (t / a) ** 2, (K1 - K0) * 0.5 * (t / b) ** 2


class IsotropicMaterial:
    """Isotropic 2D RTA material on directions s_q = (cos phi_q, sin phi_q), phi_q = 2 pi q / n_phi
    (openbte/inverse/bte.py:47-53): W_mq = 2 k_m / (n_phi L_m^2), t_coeff = W / sum W,
    sigma_mq = 2 k_m s_q / (n_phi L_m)."""

    def __init__(self, mfps, kappas, n_phi: int):
        self.mfps = np.ascontiguousarray(np.asarray(mfps, dtype=np.float64))
        self.kappas = np.asarray(kappas, dtype=np.float64)
        phi = 2 * np.pi * np.arange(n_phi) / n_phi
        self.vmfp = np.ascontiguousarray(np.stack([np.cos(phi), np.sin(phi)], axis=1))
        W = np.repeat((2 * self.kappas / (n_phi * self.mfps ** 2))[:, None], n_phi, axis=1)
        self.t_coeff = np.ascontiguousarray(W / W.sum())
        self.sigma = np.ascontiguousarray((2 * self.kappas / (n_phi * self.mfps))[:, None, None] * self.vmfp[None])
        self.kappa_bulk = float(self.kappas.sum())

    @staticmethod
    def gray(kn: float, n_phi: int, size: float = 1.0):
        """One MFP = kn x cell size and unit bulk conductivity: kappa_eff is the reference's normalised kappa."""
        return IsotropicMaterial([kn * size], [1.0], n_phi)

    @staticmethod
    def lognormal(n_mfp: int, n_phi: int, kappa_bulk=150.0, mfp_min=1.0, mfp_max=1.0e4, median=300.0, sigma_ln=1.0):
        """The synthetic MFP distribution of the transport benchmarks (MFPs in nm, log-spaced)."""
        mfps = np.logspace(math.log10(mfp_min), math.log10(mfp_max), n_mfp)
        return IsotropicMaterial(mfps, lognormal_kappa(mfps, kappa_bulk, median, sigma_ln), n_phi)

    def reversed(self):
        """The same material with every direction reversed (s_q -> -s_q, sigma -> -sigma): the adjoint
        problem of a direction set that is not closed under reversal."""
        r = IsotropicMaterial.__new__(IsotropicMaterial)
        r.mfps, r.kappas, r.kappa_bulk = self.mfps, self.kappas, self.kappa_bulk
        r.vmfp = np.ascontiguousarray(-self.vmfp)
        r.t_coeff = self.t_coeff
        r.sigma = np.ascontiguousarray(-self.sigma)
        return r

    def closed_under_reversal(self) -> bool:
        v = self.vmfp
        return all(np.min(np.abs(v + v[q]).max(axis=1)) < 1e-9 for q in range(len(v)))

    def c_struct(self):
        m = _lib.MaterialC()
        m.n_mfp, m.n_dir = len(self.mfps), self.vmfp.shape[0]
        m.dim_dir = m.dim_sigma = 2
        m.mfps, m.vmfp, m.sigma, m.t_coeff = ptr(self.mfps), ptr(self.vmfp), ptr(self.sigma), ptr(self.t_coeff)
        m.heat_source_coeff = 0.0
        return m


class PixelSolver:
    """kappa_eff and dkappa/drho of an n x n pixel cell.

    The plan (sweep order, slots, device tables) depends on the grid and the directions only: it is built on
    the first call and later density fields replace its transmissions (``obte_bte_plan_set_transmission``),
    as the reference recomputes only its density-dependent terms per field (openbte/inverse/bte.py:147-173)
    over the geometry of bte.py:116-140.  ``reuse_plan=False`` builds a new plan per field instead.
    ``warm_start=True`` starts each solve from the previous field's solution (the reference's x0 reuse,
    bte.py:234-236); the default starts from zero, so results do not depend on the call history."""

    def __init__(self, n: int, material: IsotropicMaterial, size: float = 1.0, direction=(1, 0), device: int = 0,
                 precision: str = "fp32_refine", rtol: float = 1e-8, restart: int = 100, max_sweeps: int = 3000,
                 reuse_plan: bool = True, warm_start: bool = False, dsa: int = 0):
        if tuple(direction) not in ((1, 0), (0, 1)):
            raise NotImplementedError("kappa along x ([1, 0]) or y ([0, 1])")
        self.lib = _lib.load()
        self.grid = pixel_grid(n, size)
        self.material = material
        self.device = device
        self.precision, self.rtol, self.restart, self.max_sweeps = precision, rtol, restart, max_sweeps
        g = self.grid
        jump_sides = g["per_x"] if tuple(direction) == (1, 0) else g["per_y"]
        self.internal = np.arange(2 * n * n, dtype=np.int64)
        self.per_sides = np.nonzero(g["per_x"] | g["per_y"])[0].astype(np.int64)
        self.per_jump = np.ascontiguousarray(jump_sides[self.per_sides].astype(np.float64))
        self.contact = np.nonzero(jump_sides)[0].astype(np.int64)
        self.empty = np.zeros(1, dtype=np.int64)
        self.last_info = None
        self.last_upload_bytes = 0
        self.reuse_plan, self.warm_start = reuse_plan, warm_start
        self.dsa = dsa            # diffusion-synthetic acceleration: 0 = the default (on here), 1 on, -1 off
        self._h = None
        # a direction set not closed under reversal takes its adjoint from a second plan with the reversed
        # directions (obte_bte_kappa_gradient_adjoint)
        self.paired = not material.closed_under_reversal()
        self._ha = None
        self.last_adjoint_info = None

    def _problem(self, t_host):
        g = self.grid
        p = _lib.Problem()
        p.dim, p.n_elems, p.n_sides, p.elem_nv = 2, g["n_elems"], g["side_elem_map"].shape[0], 4
        p.side_elem_map = ptr(g["side_elem_map"], C.c_int64)
        p.normal_areas, p.elem_volumes, p.side_areas = ptr(g["normal_areas"]), ptr(g["elem_volumes"]), ptr(g["side_areas"])
        p.n_internal, p.internal = len(self.internal), ptr(self.internal, C.c_int64)
        p.n_periodic, p.periodic_sides = len(self.per_sides), ptr(self.per_sides, C.c_int64)
        p.periodic_jump = ptr(self.per_jump)
        p.n_diffuse, p.diffuse_sides = 0, ptr(self.empty, C.c_int64)
        p.n_mixed, p.mixed_sides, p.mixed_value = 0, ptr(self.empty, C.c_int64), None
        p.contact_kind, p.n_contact = _lib.CONTACT_PERIODIC, len(self.contact)
        p.contact_sides = ptr(self.contact, C.c_int64)
        p.contact_alpha, p.normalization = 1.0, -1.0
        p.is_nanowire, p.heat_source = 0, None
        p.side_transmission, p.reflect_internal = ptr(t_host), 1
        return p

    def _plan(self, t_host):
        """The plan with side transmissions t_host: the cached one updated, or a new one (and the reversed
        directions' plan for a set that is not closed under reversal)."""
        if self._h is not None:
            nb = C.c_int64()
            _lib.check(self.lib.obte_bte_plan_set_transmission(self._h, ptr(t_host), C.byref(nb)),
                       "obte_bte_plan_set_transmission")
            self.last_upload_bytes = nb.value          # coefficients copied to the device
            if self._ha is not None:
                _lib.check(self.lib.obte_bte_plan_set_transmission(self._ha, ptr(t_host), C.byref(nb)),
                           "obte_bte_plan_set_transmission")
                self.last_upload_bytes += nb.value
            return self._h
        ctx = context(self.device)
        prob = self._problem(t_host)
        mat = self.material.c_struct()
        h = C.c_void_p()
        _lib.check(self.lib.obte_bte_plan_create(ctx, C.byref(prob), C.byref(mat), C.byref(h)), "obte_bte_plan_create")
        self._h = h
        if self.paired:
            rev = self.material.reversed()
            self._rev = rev                            # keeps the arrays the C struct points to alive
            ha = C.c_void_p()
            _lib.check(self.lib.obte_bte_plan_create(ctx, C.byref(prob), C.byref(rev.c_struct()), C.byref(ha)),
                       "obte_bte_plan_create")
            self._ha = ha
        pb, sb = C.c_int64(), C.c_int64()
        _lib.check(self.lib.obte_bte_plan_footprint(h, _lib.PRECISION[self.precision], self.restart, C.byref(pb),
                                                    C.byref(sb)), "obte_bte_plan_footprint")
        self.last_upload_bytes = pb.value              # device tables built from the host schedule (an upper bound)
        return h

    def close(self):
        """Release the cached plan(s)."""
        if self._h is not None:
            h, self._h = self._h, None
            self.lib.obte_bte_plan_destroy(h)
        if getattr(self, "_ha", None) is not None:
            h, self._ha = self._ha, None
            self.lib.obte_bte_plan_destroy(h)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def kappa_and_gradient(self, rho):
        """(kappa_eff, dkappa/drho as a float64 device tensor [n*n])."""
        torch = _torch()
        dev = torch.device("cuda", self.device)
        rho = torch.as_tensor(rho, dtype=torch.float64, device=dev).reshape(-1)
        t, da, db = transmission(rho, self.grid)
        t_host = np.ascontiguousarray(t.detach().cpu().numpy())
        h = self._plan(t_host)
        try:
            opts = _lib.SolveOpts(precision=_lib.PRECISION[self.precision], rtol=self.rtol, max_sweeps=self.max_sweeps,
                                  restart=self.restart, refine_steps=20, inner_rtol=1e-5,
                                  warm_start=1 if self.warm_start else 0, dsa=int(self.dsa))
            dT0 = torch.zeros(self.grid["n_elems"], dtype=torch.float64, device=dev)
            grad_t = torch.empty(self.grid["side_elem_map"].shape[0], dtype=torch.float64, device=dev)
            info = _lib.SolveInfo()
            if self._ha is not None:
                ainfo = _lib.SolveInfo()
                st = self.lib.obte_bte_kappa_gradient_adjoint(h, self._ha, C.byref(opts), C.c_void_p(dT0.data_ptr()),
                                                              C.c_void_p(grad_t.data_ptr()), C.byref(info),
                                                              C.byref(ainfo))
                self.last_adjoint_info = ainfo
                _lib.check(st, "obte_bte_kappa_gradient_adjoint")
            else:
                st = self.lib.obte_bte_kappa_gradient(h, C.byref(opts), C.c_void_p(dT0.data_ptr()),
                                                      C.c_void_p(grad_t.data_ptr()), C.byref(info))
                _lib.check(st, "obte_bte_kappa_gradient")
        finally:
            if not self.reuse_plan:
                self.close()
        self.last_info = info
        sem = torch.as_tensor(self.grid["side_elem_map"], device=dev)
        g = torch.zeros_like(rho)
        g.index_add_(0, sem[:, 0], grad_t * da)
        g.index_add_(0, sem[:, 1], grad_t * db)
        return float(info.kappa_eff), g


def _autograd_function():
    torch = _torch()

    class KappaEff(torch.autograd.Function):
        """kappa_eff(rho) with dkappa/drho from the adjoint (the solve runs once, in forward)."""

        @staticmethod
        def forward(ctx, rho, solver):
            k, g = solver.kappa_and_gradient(rho.detach())
            ctx.save_for_backward(g.to(rho.dtype).reshape(rho.shape))
            return torch.tensor(k, dtype=rho.dtype, device=rho.device)

        @staticmethod
        def backward(ctx, grad_out):
            (g,) = ctx.saved_tensors
            return grad_out * g, None

    return KappaEff


def kappa_eff(rho, solver: PixelSolver):
    """Differentiable kappa_eff(rho) (a torch scalar); backward gives dkappa/drho."""
    return _autograd_function().apply(rho, solver)


def get_solver(**options):
    """The reference's solver factory (openbte/inverse/bte.py:171-255): options ``grid`` (pixels per
    side), ``Kn`` (gray: MFP / cell size) or ``material`` (an IsotropicMaterial), ``n_phi``,
    ``directions`` (list of [1, 0] / [0, 1]), ``size``, ``precision``, ``rtol``, ``dsa`` (0: the default
    acceleration, -1 off).  Returns
    ``func(rho) -> ((kappa[n_directions], 1), jacobian[n_directions, grid**2])``."""
    n = int(options["grid"])
    size = float(options.get("size", 1.0))
    n_phi = int(options.get("n_phi", 48))
    mat = options.get("material")
    if mat is None:
        mat = IsotropicMaterial.gray(float(options["Kn"]), n_phi, size)
    directions = options.get("directions", [[1, 0]])
    solvers = [PixelSolver(n, mat, size, tuple(d), device=int(options.get("device", 0)),
                           precision=options.get("precision", "fp32_refine"), rtol=float(options.get("rtol", 1e-8)),
                           dsa=int(options.get("dsa", 0)))
               for d in directions]

    def func(rho):
        kappa = np.zeros(len(solvers))
        jac = np.zeros((len(solvers), n * n))
        for i, s in enumerate(solvers):
            k, g = s.kappa_and_gradient(rho)
            kappa[i], jac[i] = k, g.cpu().numpy()
        return (kappa, 1), jac

    return func
