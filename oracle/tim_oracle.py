"""CPU oracle of the transmission-interface (TIM) BTE on a periodic pixel grid and of its gradient.

Test infrastructure only (used by tests and the CPU baseline, never by the product path).

The reference's inverse-design model (openbte/inverse/bte.py:97-168, grid from
openbte/inverse/matinverse.py:494-546) is gray: one Knudsen number, directions
s_q = (cos phi_q, sin phi_q), lattice temperature = mean over directions.  Each pixel face
transmits the fraction t = 2 rho_i rho_j / (rho_i + rho_j) of the incoming phonons from the
neighbour (rho mapped to [1e-12, 1]) and the rest, 1 - t, is the pixel's own outgoing flux
diffusely reflected back.  This module restates that model for an MFP-resolved material in the
conventions of the transport path of this package (the upwind FV rows of openbte/bte.py:183-218 and
the contact kappa of openbte/bte.py:132-158,222-243):

  r_mq(c) = X_mq(c) (1 + L_m D_q(c))
          + L_m sum_{f in(c,q)} g_qf [ t_f (X_mq(j_f) + J_f) + (1 - t_f) R_f ]
          - sum_{m'q'} tau_m'q' X_m'q'(c)                                     = 0

  g_qf = s_q . n_f / V_c (n_f outward area vector), D_q(c) = sum_f max(g_qf, 0),
  R_f  = sum_{m'q': g>0} w_m'q'f X_m'q'(c),  w = max(sigma . n_f, 0) / (-sum min(sigma . n_f, 0)),
  J_f  = +jump on the e1 side of a periodic x side, -jump on its e2 side, 0 elsewhere,
  kappa = nrm sum_{contact s} t_s sum_mq [max(sigma.n_s, 0) X(e1) + min(sigma.n_s, 0)(X(e2) + alpha)].

With one MFP and tau = 1/M this is the reference's operator (openbte/inverse/bte.py:155-163) and
kappa / kappa_bulk equals the reference's kappa (openbte/inverse/bte.py:27-40, divided by f).

Gradients: the explicit adjoint (A^T lam = dkappa/dX, dkappa/dt = d_t kappa - lam . d_t r), and the
same through the reflection identity used on the GPU: with weights V tau the operator is
symmetric up to reversing every direction, so lam_mq(c) = (nrm a / jump) V_c tau_mq X_m,qbar(c)
with sigma = a tau L s (the reference's G = -T[reflection], openbte/inverse/bte.py:33).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


# ---- grid (pixel order and side layout) ---------------------------------------------------------

def pixel_grid(n: int, size: float = 1.0):
    """Periodic n x n pixel grid in the reference's pixel order k = i*n + j (openbte/inverse/matinverse.py:494-546):
    i runs along +x, j along -y.  Sides: for every pixel p, an x side to (i+1, j) with unit normal
    (+1, 0) and a y side to (i, j+1) with unit normal (0, -1); e1 = p.  Periodic x sides are the x
    sides of i = n-1, periodic y sides the y sides of j = n-1."""
    h = size / n
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    p = (ii * n + jj).reshape(-1)
    px = (((ii + 1) % n) * n + jj).reshape(-1)
    py = (ii * n + (jj + 1) % n).reshape(-1)
    e1 = np.concatenate([p, p])
    e2 = np.concatenate([px, py])
    nrm = np.concatenate([np.tile([1.0, 0.0], (n * n, 1)), np.tile([0.0, -1.0], (n * n, 1))])
    per_x = np.concatenate([(ii == n - 1).reshape(-1), np.zeros(n * n, bool)])
    per_y = np.concatenate([np.zeros(n * n, bool), (jj == n - 1).reshape(-1)])
    return dict(n=n, h=h, size=size, n_elems=n * n, e1=e1, e2=e2, normal=nrm, area=np.full(2 * n * n, h),
                volume=np.full(n * n, h * h), per_x=per_x, per_y=per_y)


def transmission(rho, grid, k0=1e-12, k1=1.0):
    """Side transmission and its derivatives (openbte/inverse/bte.py:145-151)."""
    r = k0 + np.asarray(rho, dtype=np.float64) * (k1 - k0)
    a, b = r[grid["e1"]], r[grid["e2"]]
    t = 2 * a * b / (a + b)
    dt_da = (k1 - k0) * 0.5 * (t / a) ** 2
    dt_db = (k1 - k0) * 0.5 * (t / b) ** 2
    return t, dt_da, dt_db


def gray_material(kn: float, n_phi: int, size: float = 1.0, kappa_bulk: float = 1.0):
    """One MFP (kn x size), directions (cos phi, sin phi) (openbte/inverse/bte.py:47-53), tau = 1/M,
    sigma = 2 kappa s / (M L) (the 2D isotropic layout of the transport path)."""
    return material([kn * size], [kappa_bulk], n_phi)


def material(mfps, kappas, n_phi: int):
    """MFP-resolved isotropic 2D material: W_mq = 2 k_m / (M L_m^2), tau = W / sum W, sigma = 2 k_m s_q / (M L_m)."""
    mfps = np.asarray(mfps, dtype=np.float64)
    kappas = np.asarray(kappas, dtype=np.float64)
    phi = 2 * np.pi * np.arange(n_phi) / n_phi
    s = np.stack([np.cos(phi), np.sin(phi)], axis=1)
    W = np.repeat((2 * kappas / (n_phi * mfps ** 2))[:, None], n_phi, axis=1)
    tau = W / W.sum()
    sigma = (2 * kappas / (n_phi * mfps))[:, None, None] * s[None, :, :]
    refl = np.array([int(np.argmin(np.abs(s + s[q]).sum(axis=1))) for q in range(n_phi)])
    return dict(mfps=mfps, dirs=s, tau=tau, sigma=sigma, refl=refl, kappa_bulk=float(kappas.sum()))


# ---- operator ------------------------------------------------------------------------------------

def _faces(grid):
    """Directed faces: (owner c, neighbour j, outward area vector, side id, jump sign)."""
    ns = len(grid["e1"])
    c = np.concatenate([grid["e1"], grid["e2"]])
    j = np.concatenate([grid["e2"], grid["e1"]])
    av = (grid["normal"] * grid["area"][:, None])
    nv = np.concatenate([av, -av])
    side = np.concatenate([np.arange(ns), np.arange(ns)])
    jsign = np.concatenate([np.ones(ns), -np.ones(ns)]) * np.concatenate([grid["per_x"], grid["per_x"]])
    return c, j, nv, side, jsign


def assemble(grid, t, mat, jump=1.0):
    """Sparse A and f of the system A X = f, X ordered [m][q][c]."""
    nE = grid["n_elems"]
    V = grid["volume"]
    L = mat["mfps"]
    s = mat["dirs"]
    tau = mat["tau"]
    sig = mat["sigma"]
    nm, M = tau.shape
    c, j, nv, side, jsign = _faces(grid)
    tf = t[side]
    idx = lambda m, q, e: (m * M + q) * nE + e  # noqa: E731
    rows, cols, vals = [], [], []
    f = np.zeros(nm * M * nE)
    g = (nv @ s.T) / V[c][:, None]                       # [faces, q]
    D = np.zeros((nE, M))
    np.add.at(D, c, np.maximum(g, 0))
    # reflection weights per face over (m', q')
    sn = np.einsum("mqd,fd->fmq", sig, nv)               # sigma . n_f
    Z = -np.minimum(sn, 0).sum(axis=(1, 2))
    w = np.maximum(sn, 0) / Z[:, None, None]             # [faces, m', q']
    for m in range(nm):
        for q in range(M):
            r0 = idx(m, q, np.arange(nE))
            rows.append(r0); cols.append(r0); vals.append(1 + L[m] * D[:, q])
            inf = np.nonzero(g[:, q] < 0)[0]
            # transmitted inflow
            rows.append(idx(m, q, c[inf])); cols.append(idx(m, q, j[inf])); vals.append(L[m] * g[inf, q] * tf[inf])
            np.add.at(f, idx(m, q, c[inf]), -L[m] * g[inf, q] * tf[inf] * jump * jsign[inf])
            # reflected inflow: couples to the outgoing ordinates of the same pixel
            for fi in inf:
                mm, qq = np.nonzero(w[fi] > 0)
                rows.append(np.full(len(mm), idx(m, q, c[fi]))); cols.append(idx(mm, qq, c[fi]))
                vals.append(L[m] * g[fi, q] * (1 - tf[fi]) * w[fi, mm, qq])
            # lattice temperature
            for m2 in range(nm):
                for q2 in range(M):
                    rows.append(r0); cols.append(idx(m2, q2, np.arange(nE))); vals.append(np.full(nE, -tau[m2, q2]))
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(nm * M * nE,) * 2)
    A.sum_duplicates()
    return A, f


def _bordered_solve(A, b, left, right):
    """Solve A x = b on the complement of the null vector `right`, normalised by left . x = 0."""
    n = A.shape[0]
    B = sp.bmat([[A, sp.csr_matrix(right.reshape(-1, 1))], [sp.csr_matrix(left.reshape(1, -1)), None]], format="csc")
    x = spla.spsolve(B, np.concatenate([b, [0.0]]))
    return x[:n]


def solve(grid, t, mat, jump=1.0):
    A, f = assemble(grid, t, mat, jump)
    nm, M = mat["tau"].shape
    ell = (grid["volume"][None, None, :] * mat["tau"][:, :, None]).reshape(-1)
    X = _bordered_solve(A, f, ell, np.ones(A.shape[0]))
    return X.reshape(nm, M, grid["n_elems"]), A, f


def kappa_of(X, grid, t, mat, nrm=-1.0, alpha=1.0):
    """kappa = nrm sum_{periodic x sides} t_s sum_mq [max(sigma.n,0) X(e1) + min(sigma.n,0)(X(e2) + alpha)]."""
    cs = np.nonzero(grid["per_x"])[0]
    nv = grid["normal"][cs] * grid["area"][cs, None]
    sn = np.einsum("mqd,sd->mqs", mat["sigma"], nv)
    e1, e2 = grid["e1"][cs], grid["e2"][cs]
    K = (np.maximum(sn, 0) * X[:, :, e1] + np.minimum(sn, 0) * (X[:, :, e2] + alpha)) * t[cs][None, None, :]
    return nrm * K.sum()


def dkappa_dX(grid, t, mat, nrm=-1.0):
    nm, M = mat["tau"].shape
    b = np.zeros((nm, M, grid["n_elems"]))
    cs = np.nonzero(grid["per_x"])[0]
    nv = grid["normal"][cs] * grid["area"][cs, None]
    sn = np.einsum("mqd,sd->mqs", mat["sigma"], nv)
    np.add.at(b, (slice(None), slice(None), grid["e1"][cs]), nrm * np.maximum(sn, 0) * t[cs])
    np.add.at(b, (slice(None), slice(None), grid["e2"][cs]), nrm * np.minimum(sn, 0) * t[cs])
    return b.reshape(-1)


def reflected_temperature(X, grid, mat):
    """R_f for every directed face (faces ordered like _faces)."""
    c, j, nv, side, jsign = _faces(grid)
    sn = np.einsum("mqd,fd->fmq", mat["sigma"], nv)
    Z = -np.minimum(sn, 0).sum(axis=(1, 2))
    w = np.maximum(sn, 0) / Z[:, None, None]
    return np.einsum("fmq,mqf->f", w, X[:, :, c])


def dr_dt(X, grid, t, mat, jump=1.0):
    """d r / d t_s as a dense [n_sides, n_unknowns] array (small grids only)."""
    c, j, nv, side, jsign = _faces(grid)
    V = grid["volume"]
    s = mat["dirs"]
    L = mat["mfps"]
    nm, M = mat["tau"].shape
    nE = grid["n_elems"]
    R = reflected_temperature(X, grid, mat)
    g = (nv @ s.T) / V[c][:, None]
    out = np.zeros((len(grid["e1"]), nm, M, nE))
    for fi in range(len(c)):
        for q in np.nonzero(g[fi] < 0)[0]:
            out[side[fi], :, q, c[fi]] += L * g[fi, q] * (X[:, q, j[fi]] + jump * jsign[fi] - R[fi])
    return out.reshape(len(grid["e1"]), -1)


def dkappa_dt_explicit(X, grid, t, mat, nrm=-1.0, alpha=1.0):
    g = np.zeros(len(grid["e1"]))
    cs = np.nonzero(grid["per_x"])[0]
    nv = grid["normal"][cs] * grid["area"][cs, None]
    sn = np.einsum("mqd,sd->mqs", mat["sigma"], nv)
    e1, e2 = grid["e1"][cs], grid["e2"][cs]
    g[cs] = nrm * (np.maximum(sn, 0) * X[:, :, e1] + np.minimum(sn, 0) * (X[:, :, e2] + alpha)).sum(axis=(0, 1))
    return g


def gradient_adjoint(X, A, grid, t, mat, nrm=-1.0, alpha=1.0, jump=1.0):
    """dkappa/dt per side through an explicit adjoint solve."""
    b = dkappa_dX(grid, t, mat, nrm)
    ell = (grid["volume"][None, None, :] * mat["tau"][:, :, None]).reshape(-1)
    lam = _bordered_solve(A.T.tocsr(), b, np.ones(A.shape[0]), ell)
    return dkappa_dt_explicit(X, grid, t, mat, nrm, alpha) - dr_dt(X, grid, t, mat, jump) @ lam


def flux_scale(mat):
    """a with sigma_mq = a tau_mq L_m s_q (isotropic materials; a = sum W)."""
    a = np.einsum("mqd,qd->mq", mat["sigma"], mat["dirs"]) / (mat["tau"] * mat["mfps"][:, None])
    assert np.allclose(a, a.flat[0], rtol=1e-12, atol=0)
    return float(a.flat[0])


def gradient_reflection(X, grid, t, mat, nrm=-1.0, alpha=1.0, jump=1.0):
    """dkappa/dt per side through lam_mq(c) = (nrm a / jump) V_c tau_mq X_m,qbar(c) (a = flux_scale):
    per directed face E_f = sum_{q in(f)} (s_q . n_f) sum_m tau_mq L_m X_m,qbar(c) (X_mq(j) + J_f - R_f)."""
    c, j, nv, side, jsign = _faces(grid)
    s = mat["dirs"]
    tl = mat["tau"] * mat["mfps"][:, None]
    R = reflected_temperature(X, grid, mat)
    Xb = X[:, mat["refl"], :]
    sn = nv @ s.T                                            # [faces, q]
    E = np.zeros(len(c))
    for fi in range(len(c)):
        qs = np.nonzero(sn[fi] < 0)[0]
        E[fi] = np.sum(sn[fi, qs][None, :] * tl[:, qs] * Xb[:, qs, c[fi]] *
                       (X[:, qs, j[fi]] + jump * jsign[fi] - R[fi]))
    G = np.zeros(len(grid["e1"]))
    np.add.at(G, side, E)
    return dkappa_dt_explicit(X, grid, t, mat, nrm, alpha) - (nrm * flux_scale(mat) / jump) * G


def kappa_and_gradient(rho, grid, mat, nrm=-1.0, method="reflection"):
    """kappa_eff and dkappa/drho (chain rule through the harmonic-mean transmission)."""
    t, da, db = transmission(rho, grid)
    X, A, f = solve(grid, t, mat)
    k = kappa_of(X, grid, t, mat, nrm)
    gt = gradient_reflection(X, grid, t, mat, nrm) if method == "reflection" else gradient_adjoint(X, A, grid, t, mat, nrm)
    grad = np.zeros(grid["n_elems"])
    np.add.at(grad, grid["e1"], gt * da)
    np.add.at(grad, grid["e2"], gt * db)
    return k, grad, X


def kappa_fd(rho, grid, mat, pixels, h=1e-6, nrm=-1.0):
    """Central finite differences of kappa_eff in the given pixels."""
    out = []
    for p in pixels:
        r1 = np.array(rho, dtype=np.float64); r1[p] += h
        r2 = np.array(rho, dtype=np.float64); r2[p] -= h
        k1 = kappa_of(solve(grid, transmission(r1, grid)[0], mat)[0], grid, transmission(r1, grid)[0], mat, nrm)
        k2 = kappa_of(solve(grid, transmission(r2, grid)[0], mat)[0], grid, transmission(r2, grid)[0], mat, nrm)
        out.append((k1 - k2) / (2 * h))
    return np.array(out)
