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

__all__ = ["synthetic_isotropic_2d", "synthetic_isotropic_3d", "lognormal_kappa", "Gray2D"]


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
