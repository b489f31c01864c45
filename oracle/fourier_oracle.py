"""CPU oracle for the Fourier first guess — TEST INFRASTRUCTURE ONLY.

numpy/scipy restatement of the reference ``Fourier`` (openbte/fourier.py:15-185)
with ``Mesh.get_decomposed_directions`` (openbte/objects.py:312-319),
``Mesh.gradient`` (openbte/objects.py:322-405) and
``EffectiveThermalConductivity.get_diffusive`` (openbte/objects.py:139-172).
It is the checker for the device Fourier solver; only tests, the smoke check
and the benchmark's CPU-baseline leg use it.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

PIN = 10   # fourier.py:43 — element pinned to zero when no mixed BC exists


def decomposed_directions(geo, kappa):
    """objects.py:312-319."""
    na = geo.normal_areas
    v_orth = np.einsum("ki,ij,kj->k", na, kappa, na) / np.einsum("ki,ki->k", na, geo.dists)
    v_non = na @ kappa.T - geo.dists * v_orth[:, None]
    return v_orth, v_non


def side_slots(geo):
    """(elem, side) -> position of the side in the elem's side list (objects.py:335-336)."""
    esm = np.array([geo.elem_side_map[e] for e in range(geo.n_elems)])
    lut = {}
    for e in range(geo.n_elems):
        for r, s in enumerate(esm[e]):
            lut[(e, int(s))] = r
    return lut


def gradient(geo, bcs, T, lut=None):
    """Least-squares cell gradient (objects.py:322-405)."""
    lut = lut if lut is not None else side_slots(geo)
    nv = len(geo.elems[0])
    diff = np.zeros((geo.n_elems, nv))
    for s in geo.internal:
        i, j = geo.side_elem_map[s]
        d = T[j] - T[i]
        diff[i, lut[(i, int(s))]] = d
        diff[j, lut[(j, int(s))]] = -d
    for region, sides in geo.periodic_sides.items():
        jump = bcs.periodic[region]
        for s in sides:
            i, j = geo.side_elem_map[s]
            diff[i, lut[(i, int(s))]] += jump
            diff[j, lut[(j, int(s))]] -= jump
    for key, value in bcs.mixed.items():
        for s in geo.side_physical_regions[key]:
            i = geo.side_elem_map[s][0]
            diff[i, lut[(i, int(s))]] = value["value"] - T[i]
    return np.einsum("kjs,ks->kj", geo.gradient_weights, diff)


def fourier(geo, thermal_conductivity, bcs, effective_thermal_conductivity=None,
            fourier_max_iter=40, fourier_rtol=1e-8, verbose=False):
    """Returns (kappa_printed, T, J[n,dim] in W/m/nm, n_iter).

    ``kappa_printed`` is the value the reference prints each iteration; the
    reference *returns* 0 because of its while/else (fourier.py:179-180).
    """
    kappa = np.asarray(thermal_conductivity)[: geo.dim, : geo.dim]
    v_orth, v_non = decomposed_directions(geo, kappa)
    n = geo.n_elems
    internal = np.asarray(geo.internal)
    i = geo.side_elem_map[internal, 0]
    j = geo.side_elem_map[internal, 1]
    vi = geo.elem_volumes[i]
    vj = geo.elem_volumes[j]
    vo = v_orth[internal]
    # fourier.py:51-63
    rows = [i, i, j, j]
    cols = [i, j, j, i]
    vals = [vo / vi, -vo / vi, vo / vj, -vo / vj]
    B = np.zeros(n)
    for key, contact in bcs.mixed.items():                                  # fourier.py:70-86
        for s in geo.side_physical_regions[key]:
            e = geo.side_elem_map[s][0]
            h = contact["boundary_conductance"]
            tmp = v_orth[s] * h / (h + v_orth[s] / geo.side_areas[s])
            rows.append(np.array([e]))
            cols.append(np.array([e]))
            vals.append(np.array([tmp / geo.elem_volumes[e]]))
            B[e] = contact["value"] * tmp / geo.elem_volumes[e]
    for region, jump in bcs.periodic.items():                                # fourier.py:89-98
        for s in geo.periodic_sides[region]:
            a, b = geo.side_elem_map[s]
            B[a] += jump * v_orth[s] / geo.elem_volumes[a]
            B[b] -= jump * v_orth[s] / geo.elem_volumes[b]
    F = sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    if len(bcs.mixed) == 0:                                                  # fourier.py:115-118
        scale = np.ones(n)
        scale[PIN] = 0
        F.data = F.data * scale[F.indices]
        F = F.tolil()
        F[PIN, PIN] = 1
        F = F.tocsc()
        B[PIN] = 0                                                           # fourier.py:141-142
    lu = spla.splu(F)
    w = geo.interp_weights[internal]
    vnon = v_non[internal]
    lut = side_slots(geo)
    ek = effective_thermal_conductivity
    C = np.zeros(n)
    norm_C_old = 0.0
    error = 1.0
    n_iter = 0
    kappa_eff = 0.0
    T = np.zeros(n)
    grad = np.zeros((n, geo.dim))
    while error > fourier_rtol and n_iter < fourier_max_iter:               # fourier.py:149-178
        n_iter += 1
        T = lu.solve(B + C)
        if len(bcs.mixed) == 0:
            T = T - (np.max(T) + np.min(T)) * 0.5
        grad = gradient(geo, bcs, T, lut)
        C = np.zeros(n)
        F_ave = w[:, None] * grad[i] + (1 - w)[:, None] * grad[j]
        tmp = np.einsum("ki,ki->k", F_ave, vnon)
        np.add.at(C, i, tmp / vi)
        np.add.at(C, j, -tmp / vj)
        norm_C = np.linalg.norm(C)
        error = 0 if norm_C == 0 else abs(norm_C - norm_C_old) / norm_C
        norm_C_old = norm_C
        if ek is not None:
            kappa_eff = diffusive_kappa(geo, bcs, ek, T, kappa)
        if verbose:
            print("Kappa (Fourier): {:E}, Iterations {:n}, Error {:E}".format(kappa_eff, n_iter, error))
    J = -grad @ kappa.T                                                      # fourier.py:182
    return kappa_eff, T, J, n_iter


def diffusive_kappa(geo, bcs, ek, T, kappa):
    """objects.py:139-172."""
    bc = bcs.get_bc_by_name(ek.contact)
    v_orth, _ = decomposed_directions(geo, kappa)
    if bc == "Mixed":
        sides = np.asarray(geo.side_physical_regions[ek.contact])
        h = bcs.mixed[ek.contact]["boundary_conductance"]
        T2 = bcs.mixed[ek.contact]["value"]
        tmp = v_orth[sides] * h / (h + v_orth[sides] / geo.side_areas[sides])
        T1 = T[geo.side_elem_map[sides, 0]]
    else:
        sides = np.asarray(geo.periodic_sides[ek.contact])
        T1 = T[geo.side_elem_map[sides, 0]]
        T2 = T[geo.side_elem_map[sides, 1]] + bcs.periodic[ek.contact]
        tmp = v_orth[sides]
    return float(np.sum((T1 - T2) * tmp * ek.normalization))
