"""Material builders with the reference's ordinate layout.

``synthetic_isotropic_2d`` is the seeded-free synthetic MFP-resolved material
used by the benchmark workloads; it follows the ``RTA2DSym`` layout
(openbte/material.py:105-189): directions ``phi_q = 2*pi*q/n_phi`` with
``s_q = (sin phi, cos phi)`` (openbte/material.py:117-119), ``sigma`` in
W/m/K/nm, ``mfps`` in nm, ``t_coeff = W / sum W``, ``grid = (n_mfp, n_phi)``.
At ``n_mfp = 1`` it reduces to ``Gray2D`` (openbte/material.py:217-247).

``synthetic_isotropic_3d`` uses the (theta, phi) midpoint grid and direction
convention of ``RTA3D`` (openbte/material.py:15-28) with solid-angle weights.
"""
from __future__ import annotations

import math

import numpy as np

from .objects import Material

__all__ = ["synthetic_isotropic_2d", "synthetic_isotropic_3d", "lognormal_kappa", "Gray2D", "load_rta", "RTA2DSym",
           "RTA3D"]


def _ndtr(x):
    return 0.5 * (1.0 + np.vectorize(math.erf)(np.asarray(x, dtype=np.float64) / math.sqrt(2.0)))


def lognormal_kappa(mfps, kappa_bulk=150.0, median=300.0, sigma_ln=1.0):
    """kappa_m = kappa_bulk x lognormal-CDF mass between geometric bin midpoints.

    The first and last bins absorb the tails, so sum(kappa_m) == kappa_bulk.
    """
    mfps = np.asarray(mfps, dtype=np.float64)
    edges = np.sqrt(mfps[:-1] * mfps[1:])
    cdf = _ndtr((np.log(edges) - math.log(median)) / sigma_ln)
    cdf = np.concatenate([[0.0], cdf, [1.0]])
    return kappa_bulk * np.diff(cdf)


def synthetic_isotropic_2d(n_mfp=30, n_phi=48, kappa_bulk=150.0, mfp_min=1.0, mfp_max=1.0e4,
                           median=300.0, sigma_ln=1.0) -> Material:
    """Isotropic 2D MFP-resolved material (RTA2DSym layout, see module docstring)."""
    mfps = np.logspace(math.log10(mfp_min), math.log10(mfp_max), n_mfp)
    kappa_m = lognormal_kappa(mfps, kappa_bulk, median, sigma_ln)
    phi = np.linspace(0.0, 2.0 * np.pi, n_phi, endpoint=False)
    s = np.stack([np.sin(phi), np.cos(phi)], axis=1)
    W = (2.0 * kappa_m / (n_phi * mfps ** 2))[:, None] * np.ones((1, n_phi))
    t_coeff = W / W.sum()
    sigma = (2.0 * kappa_m / (n_phi * mfps))[:, None, None] * s[None, :, :]
    kappa = np.einsum("mqi,mq,mqj->ij", sigma, 1.0 / W, sigma)
    return Material(kappa, sigma, s, t_coeff, mfps, (n_mfp, n_phi), 0.0, 1.0 / W.sum())


def synthetic_isotropic_3d(n_mfp=30, n_theta=16, n_phi=32, kappa_bulk=150.0, mfp_min=1.0,
                           mfp_max=1.0e4, median=300.0, sigma_ln=1.0) -> Material:
    """Isotropic 3D material on the RTA3D (theta, phi) midpoint grid.

    W_mq is proportional to the cell solid angle; the scale is fixed so that
    sum_mq sigma sigma^T / W has xx == kappa_bulk.
    """
    mfps = np.logspace(math.log10(mfp_min), math.log10(mfp_max), n_mfp)
    kappa_m = lognormal_kappa(mfps, kappa_bulk, median, sigma_ln)
    dphi = 2.0 * np.pi / n_phi
    phi = np.linspace(dphi / 2.0, 2.0 * np.pi - dphi / 2.0, n_phi)
    dth = np.pi / n_theta
    theta = np.linspace(dth / 2.0, np.pi - dth / 2.0, n_theta)
    polar = np.stack([np.sin(phi), np.cos(phi), np.ones(n_phi)], axis=1)
    azim = np.stack([np.sin(theta), np.sin(theta), np.cos(theta)], axis=1)
    s = np.einsum("lj,kj->lkj", azim, polar).reshape(n_theta * n_phi, 3)
    domega = (2.0 * np.sin(dth / 2.0) * np.sin(theta))[:, None] * dphi * np.ones((1, n_phi))
    w = (domega / domega.sum()).reshape(-1)
    # W_mq = c_m w_q / mfp^2, sigma_mq = W_mq * mfp * s_q; kappa_m,xx = c_m * sum_q w_q s_x^2
    sxx = float(np.sum(w * s[:, 0] ** 2))
    c = kappa_m / sxx
    W = (c / mfps ** 2)[:, None] * w[None, :]
    sigma = (W * mfps[:, None])[:, :, None] * s[None, :, :]
    t_coeff = W / W.sum()
    kappa = np.einsum("mqi,mq,mqj->ij", sigma, 1.0 / W, sigma)
    return Material(kappa, sigma, s, t_coeff, mfps, (n_mfp, n_theta, n_phi), 0.0, 1.0 / W.sum())


def Gray2D(**kwargs) -> Material:
    """Single-MFP 2D material (openbte/material.py:217-247)."""
    n_phi = kwargs.setdefault("n_phi", 96)
    MFP = kwargs["MFP"]
    phi = np.linspace(0, 2.0 * np.pi, n_phi, endpoint=False)
    polar = np.round(np.array([np.sin(phi), np.cos(phi)]).T, 4)
    kappa = kwargs.setdefault("kappa", 1) * np.eye(2)
    sigma = np.zeros((1, n_phi, 2))
    sigma[0] = 2 * kappa[0, 0] / MFP * polar / n_phi
    mfps = np.array([MFP])
    t_coeff = np.ones((1, n_phi)) / n_phi
    h = 4 / np.pi * kappa[0, 0] / mfps[0]
    heat_source_coeff = MFP * MFP * 0.5 / kappa[0, 0]
    return Material(kappa, sigma, polar, t_coeff, mfps, (1, n_phi), h, heat_source_coeff)


# ---- real materials: mode data binned onto the (MFP, direction) grid ------------------------------------

def load_rta(material: str, source: str = "database", path: str | None = None):
    """Mode data of `material` (openbte/utils.py:147-151, 260-279): a sqlitedict file `<material>.db` whose
    table `unnamed` maps the field names of `MaterialRTA` to pickled numpy arrays.

    source="database" reads it from the directory `path`, else from the directory named by the environment
    variable OBTE_MATERIAL_DB (this package ships no material data); source="local" reads ./<material>.db.
    Fields are matched by name, so the row order of the file does not matter.  A missing file raises
    FileNotFoundError (the reference prints a message and calls quit()).
    """
    import os
    import pickle
    import sqlite3
    from .objects import MaterialRTA
    if source == "local":
        folder = path or "."
    else:
        folder = path or os.environ.get("OBTE_MATERIAL_DB", "")
    fname = os.path.join(folder, material + ".db")
    if not os.path.isfile(fname):
        raise FileNotFoundError(f"{fname} does not exist")
    con = sqlite3.connect(f"file:{fname}?mode=ro", uri=True)
    try:
        rows = {k: pickle.loads(v) for k, v in con.execute("SELECT key, value FROM unnamed ORDER BY rowid")}
    finally:
        con.close()
    fields = {f: np.asarray(rows[f]) for f in MaterialRTA._fields if f in rows}
    missing = [f for f in ("heat_capacity", "scattering_time", "group_velocity") if f not in fields]
    if missing:
        raise ValueError(f"{fname}: missing fields {missing}")
    return MaterialRTA(**fields)


def _azimuth(v):
    """Angle of (x, y) measured from +y towards +x, in [0, 2 pi) (openbte/utils.py:323-337)."""
    a = np.arctan2(v[:, 0], v[:, 1])
    return np.where(a < 0, a + 2.0 * np.pi, a)


def _grid_weights(x, grid, bound):
    """Linear weights of each x on `grid` (increasing): (w_lo, w_hi, i_lo, i_hi) with x ~ w_lo g[i_lo] + w_hi g[i_hi].

    The interval is the one whose upper node is the first grid value >= x.  bound="extent": outside the grid
    the end intervals extrapolate linearly; bound="periodic" (angles, grid from 0 with constant spacing):
    x above the last node, or equal to the first, interpolates between the last node and 2 pi + the first.
    (The weights of openbte/utils.py:281-320 with these bounds.)
    """
    x = np.asarray(x, dtype=np.float64)
    n = len(grid)
    hi = np.searchsorted(grid, x, side="left")
    hi = np.where(hi == n, 0, hi)                 # no node >= x: treated like the first node, fixed below
    lo = hi - 1
    with np.errstate(divide="ignore", invalid="ignore"):
        w_hi = (x - grid[lo]) / (grid[hi] - grid[lo])
    if bound == "periodic":
        d = grid[-1] - grid[-2]
        wrap = hi == 0
        xw = np.where(x < d / 2, x + 2.0 * np.pi, x)
        lo = np.where(wrap, n - 1, lo)
        w_hi = np.where(wrap, (xw - grid[-1]) / d, w_hi)
    elif bound == "extent":
        below, above = x < grid[0], x > grid[-1]
        lo = np.where(below, 0, np.where(above, n - 2, lo))
        hi = np.where(below, 1, np.where(above, n - 1, hi))
        w_hi = np.where(below, (x - grid[0]) / (grid[1] - grid[0]),
                        np.where(above, (x - grid[-2]) / (grid[-1] - grid[-2]), w_hi))
    lo = np.where(lo < 0, lo + n, lo)
    return 1.0 - w_hi, w_hi, lo, hi


def _mode_arrays(data: "MaterialRTA", dim: int):
    tau = np.asarray(data.scattering_time, dtype=np.float64)
    cv = np.asarray(data.heat_capacity, dtype=np.float64)
    vg = np.asarray(data.group_velocity, dtype=np.float64)[:, :dim]
    sigma = cv[:, None] * vg
    mfp = vg * tau[:, None]
    inv_tau = np.divide(1.0, tau, out=np.zeros_like(tau), where=tau != 0)
    return sigma, mfp, cv * inv_tau


def _bin(shape, dim, idx_w, W, sigma):
    """W_s[m, q] and sigma_s[m, q, :] from per-mode corner indices (m, q) and weights."""
    n_mfp, n_ang = shape
    Ws = np.zeros(n_mfp * n_ang)
    Ss = np.zeros((n_mfp * n_ang, dim))
    for m, q, w in idx_w:
        flat = m * n_ang + q
        np.add.at(Ws, flat, w * W)
        np.add.at(Ss, flat, sigma * w[:, None])
    return Ws.reshape(n_mfp, n_ang), Ss.reshape(n_mfp, n_ang, dim)


def _finish(Ws, Ss):
    Winv = np.divide(1.0, Ws, out=np.zeros_like(Ws), where=Ws != 0)
    kappa = np.einsum("mqi,mq,mqj->ij", Ss, Winv, Ss)
    return kappa, Ws / Ws.sum()


def RTA2DSym(data: "MaterialRTA", **kwargs) -> Material:
    """2D material from mode data (openbte/material.py:105-189): the in-plane vectorial MFPs v tau of the
    modes are binned bilinearly onto n_mfp log-spaced MFPs x n_phi directions phi_q = 2 pi q / n_phi.

    Per mode: W = C / tau (the lattice-temperature weight) and sigma = C v; both are spread over the four
    surrounding (MFP, direction) nodes, kappa = sum sigma sigma^T / W over the nodes, t_coeff = W / sum W.
    The MFP grid runs from 0.9 of the smallest to 1.1 of the largest mode MFP above 1e-10 m (overridable
    with mfp_min / mfp_max in m), with the reference's start exponent log10(mfp_min) x 1.01.
    """
    n_phi = kwargs.get("n_phi", 48)
    n_mfp = kwargs.get("n_mfp", 50)
    phi = np.linspace(0.0, 2.0 * np.pi, n_phi, endpoint=False)
    dirs = np.stack([np.sin(phi), np.cos(phi)], axis=1)
    sigma, mfp, W = _mode_arrays(data, 2)
    r = np.linalg.norm(mfp, axis=1)
    keep = r > 1e-10
    sigma, mfp, W, r = sigma[keep], mfp[keep], W[keep], r[keep]
    ang = _azimuth(mfp)
    mfp_max = kwargs.get("mfp_max", r.max() * 1.1)
    mfp_min = kwargs.get("mfp_min", r.min() * 0.9)
    grid_m = np.logspace(np.log10(mfp_min) * 1.01, np.log10(mfp_max), n_mfp, endpoint=True)
    a1, a2, m1, m2 = _grid_weights(r, grid_m, "extent")
    b1, b2, p1, p2 = _grid_weights(ang, phi, "periodic")
    Ws, Ss = _bin((n_mfp, n_phi), 2, [(m1, p1, a1 * b1), (m1, p2, a1 * b2), (m2, p1, a2 * b1), (m2, p2, a2 * b2)],
                  W, sigma)
    kappa, t_coeff = _finish(Ws, Ss)
    h = 2.0 / 3.0 * np.sum(W * np.clip(mfp[:, 0], 0, None)) * 1e-9     # W/m/nm/K
    return Material(kappa, Ss * 1e-9, dirs, t_coeff, grid_m * 1e9, (n_mfp, n_phi), h, 1.0 / np.sum(W))


def RTA3D(data: "MaterialRTA", **kwargs) -> Material:
    """3D material from mode data (openbte/material.py:7-102): vectorial MFPs binned trilinearly onto
    n_mfp log-spaced MFPs x (n_theta x n_phi) midpoint directions (sin t sin p, sin t cos p, cos t), direction
    index t n_phi + p; polar angle with linear extrapolation at the ends, azimuth periodic."""
    n_phi = kwargs.get("n_phi", 24)
    n_mfp = kwargs.get("n_mfp", 50)
    n_theta = kwargs.get("n_theta", 24)
    dphi = 2.0 * np.pi / n_phi
    phi = np.linspace(dphi / 2.0, 2.0 * np.pi - dphi / 2.0, n_phi, endpoint=True)
    dth = np.pi / n_theta
    theta = np.linspace(dth / 2.0, np.pi - dth / 2.0, n_theta, endpoint=True)
    dirs = np.einsum("tj,pj->tpj", np.stack([np.sin(theta), np.sin(theta), np.cos(theta)], axis=1),
                     np.stack([np.sin(phi), np.cos(phi), np.ones(n_phi)], axis=1)).reshape(-1, 3)
    sigma, mfp, W = _mode_arrays(data, 3)
    r = np.linalg.norm(mfp, axis=1)
    keep = r > 1e-10
    sigma, mfp, W, r = sigma[keep], mfp[keep], W[keep], r[keep]
    ang = _azimuth(mfp)
    pol = np.arccos(mfp[:, 2] / r)
    grid_m = np.logspace(np.log10(r.min() * 0.9) * 1.01, np.log10(r.max() * 1.1), n_mfp, endpoint=True)
    a1, a2, m1, m2 = _grid_weights(r, grid_m, "extent")
    b1, b2, p1, p2 = _grid_weights(ang, phi, "periodic")
    c1, c2, t1, t2 = _grid_weights(pol, theta, "extent")
    corners = []
    for tt, cw in ((t1, c1), (t2, c2)):
        for pp, bw in ((p1, b1), (p2, b2)):
            for mm, aw in ((m1, a1), (m2, a2)):
                corners.append((mm, tt * n_phi + pp, aw * bw * cw))
    Ws, Ss = _bin((n_mfp, n_theta * n_phi), 3, corners, W, sigma)
    kappa, t_coeff = _finish(Ws, Ss)
    h = 2.0 / 3.0 * np.sum(W * np.clip(mfp[:, 0], 0, None)) * 1e-18
    return Material(kappa, Ss * 1e-9, dirs, t_coeff, grid_m * 1e9, (n_mfp, n_theta, n_phi), h, 1.0 / np.sum(W))
