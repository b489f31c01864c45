"""CPU oracle for the BTE source iteration — TEST INFRASTRUCTURE ONLY.

A numpy/scipy restatement of the reference solver ``BTE_RTA``
(openbte/bte.py:19-271). It is the checker for the GPU solver: only the
tests, the smoke check and the benchmark's CPU-baseline leg may import it.
The product path never calls it.

Same algorithm as the reference: per-ordinate sparse LU of
``A_mq = I + mfp_m (diag D_q + offdiag Gm_q)`` (scipy SuperLU), Jacobi source
iteration on (DeltaT, T_B), reductions to DeltaT, T_B, J, K, S, the
``|‖ΔT‖-‖ΔT_old‖|/‖ΔT‖`` stopping test. It is pinned against golden vectors
produced by running the unmodified reference (tests/golden/make_golden.py).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def _n_angles(mat):
    g = mat.grid
    if isinstance(g, (tuple, list)) and len(g) == 3:
        return g[1] * g[2]
    return g[1] if isinstance(g, (tuple, list)) else int(g)


def setup_operators(geo, mat, bcs):
    """Directed-face operator, diffuse-wall and periodic-jump terms (openbte/bte.py:47-119)."""
    n_angles = _n_angles(mat)
    dim = geo.dim
    i = geo.side_elem_map[:, 0]
    j = geo.side_elem_map[:, 1]
    internal = np.asarray(geo.internal)
    # bte.py:48-54 directed internal faces (both orientations)
    dk1 = geo.normal_areas[internal] / geo.elem_volumes[i[internal]][:, None]
    dk2 = -geo.normal_areas[internal] / geo.elem_volumes[j[internal]][:, None]
    k_mat = np.vstack((dk1, dk2))
    i_mat = np.hstack((i[internal], j[internal]))
    j_mat = np.hstack((j[internal], i[internal]))
    vmfp = np.asarray(mat.vmfp)
    # bte.py:58-62
    G = vmfp[:, :dim] @ k_mat.T
    Gp = G.clip(min=0)
    Gm = G.clip(max=0)
    D = np.zeros((n_angles, geo.n_elems))
    np.add.at(D.T, i_mat, Gp.T)

    out = dict(i_mat=i_mat, j_mat=j_mat, Gm=Gm, D=D, n_angles=n_angles)
    # bte.py:68-87 diffuse walls
    if len(bcs.diffuse) > 0:
        s_diffuse = np.asarray(geo.side_physical_regions[bcs.diffuse])
        i_diffuse = i[s_diffuse]
        db = geo.normal_areas[s_diffuse] / geo.elem_volumes[i_diffuse][:, None]
        Gb = np.einsum("mqj,sj->mqs", mat.sigma[:, :, :dim], db)
        Gbp = Gb.clip(min=0)
        Gbm = Gb.clip(max=0)
        tmp = Gbm.sum(axis=0).sum(axis=0)
        R = np.divide(1, tmp, out=np.zeros_like(tmp), where=tmp != 0)
        GG = Gbp * R[None, None, :]
        tmp = vmfp[:, :dim] @ db.T
        Gbp2 = tmp.clip(min=0)
        Gbm2 = tmp.clip(max=0)
        np.add.at(D.T, i_diffuse, Gbp2.T)
        out.update(i_diffuse=i_diffuse, GG=GG, Gbm2=Gbm2)
    else:
        out.update(i_diffuse=np.empty(0, dtype=np.int64), GG=None, Gbm2=None)

    # bte.py:90-96 thermalising (mixed) walls
    RHS_ISO = np.zeros((n_angles, geo.n_elems))
    for key, contact in bcs.mixed.items():
        sides = np.asarray(geo.side_physical_regions[key])
        tmp = geo.normal_areas[sides] / geo.elem_volumes[i[sides]][:, None]
        tmp = vmfp @ tmp.T
        np.add.at(RHS_ISO.T, i[sides], -(tmp.clip(max=0) * contact["value"]).T)
        np.add.at(D.T, i[sides], tmp.clip(min=0).T)

    # bte.py:99-110 periodic jump source
    P = np.zeros((n_angles, geo.n_elems))
    for region, jump in bcs.periodic.items():
        sides = np.asarray(geo.periodic_sides[region])
        tmp = geo.normal_areas[sides] / geo.elem_volumes[i[sides]][:, None]
        tmp = vmfp @ tmp.T
        np.add.at(P.T, i[sides], -(tmp.clip(max=0) * jump).T)
        tmp = -geo.normal_areas[sides] / geo.elem_volumes[j[sides]][:, None]
        tmp = vmfp @ tmp.T
        np.add.at(P.T, j[sides], (tmp.clip(max=0) * jump).T)

    # bte.py:113-119
    P_nano = -vmfp[:, 2] if bcs.is_nanowire else np.zeros(n_angles)
    out["perturbation"] = P + RHS_ISO + P_nano[:, None]
    return out


def contact_terms(geo, mat, bcs, ek):
    """kappa_eff contact preparation (openbte/bte.py:132-158)."""
    if bcs.is_nanowire:
        return dict(is_nanowire=True, alpha=0.0, e1=np.arange(geo.n_elems), e2=np.empty(0, dtype=np.int64),
                    sigma_normal=np.einsum("ml,c->mlc", mat.sigma[:, :, 2], geo.elem_volumes),
                    side_areas=None, normalization=ek.normalization)
    bc = bcs.get_bc_by_name(ek.contact)
    if bc == "Mixed":
        sides = np.asarray(geo.side_physical_regions[ek.contact])
        e1 = geo.side_elem_map[sides][:, 0]
        e2 = np.empty(0, dtype=np.int64)
        alpha = bcs.mixed[ek.contact]["value"]
    else:
        sides = np.asarray(geo.periodic_sides[ek.contact])
        e1 = geo.side_elem_map[sides][:, 0]
        e2 = geo.side_elem_map[sides][:, 1]
        alpha = bcs.periodic[ek.contact]
    sigma_normal = np.einsum("mli,ci->mlc", mat.sigma, geo.normal_areas[sides])
    side_areas = np.linalg.norm(geo.normal_areas[sides], axis=1)
    return dict(is_nanowire=False, alpha=alpha, e1=e1, e2=e2, sigma_normal=sigma_normal,
                side_areas=side_areas, normalization=ek.normalization)


class OrdinateSolver:
    """Per-ordinate LU cache (openbte/bte.py:181-185)."""

    def __init__(self, geo, mfps, ops):
        n = geo.n_elems
        self.n = n
        self.mfps = mfps
        self.ops = ops
        self.im = np.concatenate((ops["i_mat"], np.arange(n)))
        self.jm = np.concatenate((ops["j_mat"], np.arange(n)))
        self.cache = {}

    def matrix(self, q, m):
        ops = self.ops
        d = np.concatenate((self.mfps[m] * ops["Gm"][q], self.mfps[m] * ops["D"][q] + 1.0))
        return sp.csc_matrix((d, (self.im, self.jm)), shape=(self.n, self.n), dtype=np.float64)

    def solve(self, q, m, B):
        key = (q, m)
        lu = self.cache.get(key)
        if lu is None:
            lu = spla.splu(self.matrix(q, m))
            self.cache[key] = lu
        return lu.solve(B)


def bte_rta(geo, mat, bcs, fourier=None, effective_thermal_conductivity=None, heat_source=None,
            bte_max_iter=100, bte_rtol=1e-4, verbose=False, history=None):
    """Source iteration with exact per-ordinate solves (openbte/bte.py:19-271).

    Returns (kappa_eff, DeltaT, J[n, dim_vmfp] in W/m/nm (x1e9 = W/m^2), K, S, n_iter).
    """
    mfps = np.asarray(mat.mfps, dtype=np.float64)
    t_coeff = np.asarray(mat.t_coeff)
    n_mfp = mat.grid[0] if isinstance(mat.grid, (tuple, list)) else 1
    ops = setup_operators(geo, mat, bcs)
    n_angles = ops["n_angles"]
    n = geo.n_elems
    if fourier is None:
        DeltaT = np.zeros(n)
    else:
        DeltaT = np.array(fourier.variables["Temperature_Fourier"]["data"], dtype=np.float64)
    hs = np.zeros(n) if heat_source is None else heat_source.variables["Heat_Source"]["data"]
    ek = effective_thermal_conductivity
    ct = contact_terms(geo, mat, bcs, ek) if ek is not None else None

    i_diffuse = ops["i_diffuse"]
    n_diffuse = len(i_diffuse)
    TB = DeltaT[i_diffuse].copy() if n_diffuse > 0 else np.empty(0)
    K = np.zeros((n_mfp, n_angles))
    S = np.zeros_like(K)
    J = np.zeros((n, np.asarray(mat.vmfp).shape[1]))
    solver = OrdinateSolver(geo, mfps, ops)
    pert = ops["perturbation"]

    norm_old = np.linalg.norm(DeltaT)
    error = 1.0
    n_iter = 0
    while error > bte_rtol and n_iter < bte_max_iter:          # bte.py:196
        n_iter += 1
        boundary = -TB[None, :] * ops["Gbm2"] if n_diffuse > 0 else None   # bte.py:200
        pT = np.zeros(n)
        pTB = np.zeros(n_diffuse)
        pJ = np.zeros_like(J)
        pK = np.zeros_like(K)
        pS = np.zeros_like(S)
        for q in range(n_angles):
            for m, mfp in enumerate(mfps):
                B = DeltaT + mfp * pert[q] + hs * mat.heat_source_coeff     # bte.py:211
                if n_diffuse > 0:
                    np.add.at(B, i_diffuse, mfp * boundary[q])               # bte.py:214
                T = solver.solve(q, m, B)                                    # bte.py:218
                pT += t_coeff[m, q] * T                                      # bte.py:223
                if n_diffuse > 0:
                    pTB -= T[i_diffuse] * ops["GG"][m, q]                    # bte.py:227
                pJ += np.outer(T - DeltaT, mat.sigma[m, q])                  # bte.py:230
                if ct is not None:                                           # bte.py:232-243
                    sn = ct["sigma_normal"][m, q]
                    nrm = ct["normalization"]
                    if ct["is_nanowire"]:
                        pK[m, q] = np.dot(T[ct["e1"]], sn) * nrm
                    else:
                        pK[m, q] = np.dot(T[ct["e1"]], sn.clip(min=0)) * nrm
                        pS[m, q] = np.dot(T[ct["e1"]], ct["side_areas"]) * nrm
                    if len(ct["e2"]) > 0:
                        pK[m, q] += np.dot(T[ct["e2"]], sn.clip(max=0)) * nrm
                    pK[m, q] += ct["alpha"] * np.sum(sn.clip(max=0)) * nrm
        DeltaT, TB, J, K, S = pT, pTB, pJ, pK, pS                          # bte.py:245-249
        norm = np.linalg.norm(DeltaT)                                       # bte.py:252-254
        error = abs(norm - norm_old) / norm
        norm_old = norm
        if history is not None:
            history.append((float(np.sum(K)), float(error)))
        if verbose:
            print("Kappa (BTE): {:E}, Iterations {:n}, Error {:E}".format(np.sum(K), n_iter, error))
    return float(np.sum(K)), DeltaT, J, K, S, n_iter


def cut_ordinate_solve(solver, faces, q, m, B, x_src, src, order):
    """One transport solve with the periodic inflow given instead of solved for.

    The reference's operator A_mq = I + mfp_m (diag D_q + offdiag Gm_q) (openbte/bte.py:181-185) couples
    the two sides of every kept periodic side inside one solve.  Here its entries on the directed faces
    that cross the periodic boundary (``faces`` from ``sweep_order.directed_faces``, flag ``cut``) move
    to the right-hand side, where they multiply given inflow values: ``x_src[k]`` is the temperature of
    ordinate (m, q) at periodic source element ``src[k]`` (sorted), read across every cut inflow face
    from that element.  With x_src equal to the exact periodic solution at those elements this returns
    the reference's exact solve; for any x_src it is the transport solve a sweep evaluates.

    The cut operator has an acyclic upwind graph, so in a topological ``order`` it is lower triangular;
    it is solved by sparse triangular substitution after the order is checked to make it so (an order
    that is not topological raises).
    """
    row, nb, _, cut = faces
    ops = solver.ops
    n = solver.n
    mfp = solver.mfps[m]
    gm = np.asarray(ops["Gm"][q])
    keep = ~cut
    d = np.concatenate((mfp * gm[keep], mfp * ops["D"][q] + 1.0))
    im = np.concatenate((ops["i_mat"][keep], np.arange(n)))
    jm = np.concatenate((ops["j_mat"][keep], np.arange(n)))
    A = sp.csr_matrix((d, (im, jm)), shape=(n, n), dtype=np.float64)
    A.eliminate_zeros()   # outflow faces carry Gm = 0
    rhs = np.array(B, dtype=np.float64, copy=True)
    cf = np.nonzero(cut & (gm < 0))[0]
    if len(cf):
        pos = np.searchsorted(src, nb[cf])
        if np.any(pos >= len(src)) or np.any(src[np.minimum(pos, len(src) - 1)] != nb[cf]):
            raise ValueError("a cut inflow face reads an element outside the periodic source list")
        np.add.at(rhs, row[cf], -mfp * gm[cf] * np.asarray(x_src)[pos])
    order = np.asarray(order)
    Ap = A[order][:, order].tocsr()
    if sp.triu(Ap, k=1).nnz:
        raise ValueError("the order does not make the cut operator lower triangular")
    T = np.empty(n)
    T[order] = spla.spsolve_triangular(Ap, rhs[order], lower=True)
    return T


def solve_ordinate(geo, mat, bcs, q, m, B):
    """One exact transport solve A_mq T = B (the reference's per-ordinate splu)."""
    ops = setup_operators(geo, mat, bcs)
    s = OrdinateSolver(geo, np.asarray(mat.mfps, dtype=np.float64), ops)
    return s.solve(q, m, B)


def _one_pass(ops, solver, mat, ct, dT, TB, with_source, hs=None, dirs=None):
    """The reference's per-ordinate solves and reductions at the state (DeltaT, T_B) (openbte/bte.py:199-249);
    with_source=False leaves out the periodic-jump and heat sources (the linear part of the map).  dirs: only
    these directions (one worker's share of the ordinates, openbte/utils.py:209; the reductions are then
    that worker's partial sums, which the reference adds over workers, openbte/objects.py:86-101)."""
    n = len(dT)
    mfps = np.asarray(mat.mfps, dtype=np.float64)
    t_coeff = np.asarray(mat.t_coeff)
    n_mfp = len(mfps)
    idf = ops["i_diffuse"]
    nd = len(idf)
    boundary = -TB[None, :] * ops["Gbm2"] if nd > 0 else None
    pT, pTB = np.zeros(n), np.zeros(nd)
    pJ = np.zeros((n, np.asarray(mat.vmfp).shape[1]))
    pK = np.zeros((n_mfp, ops["n_angles"]))
    pS = np.zeros_like(pK)
    for q in (range(ops["n_angles"]) if dirs is None else dirs):
        for m, mfp in enumerate(mfps):
            B = dT.copy()
            if with_source:
                B += mfp * ops["perturbation"][q]
                if hs is not None:
                    B += hs * mat.heat_source_coeff
            if nd > 0:
                np.add.at(B, idf, mfp * boundary[q])
            T = solver.solve(q, m, B)
            pT += t_coeff[m, q] * T
            if nd > 0:
                pTB -= T[idf] * ops["GG"][m, q]
            pJ += np.outer(T - dT, mat.sigma[m, q])
            if ct is not None and with_source:
                sn = ct["sigma_normal"][m, q]
                nrm = ct["normalization"]
                if ct["is_nanowire"]:
                    pK[m, q] = np.dot(T[ct["e1"]], sn) * nrm
                else:
                    pK[m, q] = np.dot(T[ct["e1"]], sn.clip(min=0)) * nrm
                    pS[m, q] = np.dot(T[ct["e1"]], ct["side_areas"]) * nrm
                if len(ct["e2"]) > 0:
                    pK[m, q] += np.dot(T[ct["e2"]], sn.clip(max=0)) * nrm
                pK[m, q] += ct["alpha"] * np.sum(sn.clip(max=0)) * nrm
    return pT, pTB, pJ, pK, pS


def bte_rta_krylov(geo, mat, bcs, effective_thermal_conductivity=None, rtol=1e-12, restart=80, max_matvec=800):
    """The fixed point of the reference's source iteration (openbte/bte.py:193-256), found by restarted GMRES on
    (I - K) u = f, u = (DeltaT, T_B), with the same exact per-ordinate solves and reductions.

    For materials whose plain iteration is too slow to converge (long or very short MFPs).  The fixed point is
    defined up to a uniform shift of every temperature (which the reference's iteration fixes by its starting
    point): compare kappa, J and the volume-mean-free DeltaT.  Returns (kappa_eff, DeltaT, J, K, S, n_matvec).
    """
    ops = setup_operators(geo, mat, bcs)
    n = geo.n_elems
    nd = len(ops["i_diffuse"])
    ek = effective_thermal_conductivity
    ct = contact_terms(geo, mat, bcs, ek) if ek is not None else None
    solver = OrdinateSolver(geo, np.asarray(mat.mfps, dtype=np.float64), ops)

    def F(u, src):
        pT, pTB, *_ = _one_pass(ops, solver, mat, None, u[:n], u[n:], src)
        return np.concatenate([pT, pTB])

    f = F(np.zeros(n + nd), True)
    fn = np.linalg.norm(f)
    x = np.zeros(n + nd)
    mv = 0
    while mv < max_matvec:
        r = f - (x - F(x, False)) if mv else f.copy()
        mv += 1 if mv else 0
        beta = np.linalg.norm(r)
        if beta <= rtol * fn:
            break
        V = [r / beta]
        H = np.zeros((restart + 1, restart))
        g = np.zeros(restart + 1)
        g[0] = beta
        y = np.zeros(0)
        for j in range(restart):
            w = V[j] - F(V[j], False)
            mv += 1
            for _ in range(2):                       # Gram-Schmidt twice
                for i in range(j + 1):
                    h = V[i] @ w
                    H[i, j] += h
                    w = w - h * V[i]
            H[j + 1, j] = np.linalg.norm(w)
            V.append(w / H[j + 1, j] if H[j + 1, j] > 0 else w)
            y, *_ = np.linalg.lstsq(H[:j + 2, :j + 1], g[:j + 2], rcond=None)
            res = np.linalg.norm(g[:j + 2] - H[:j + 2, :j + 1] @ y)
            if res <= rtol * fn or H[j + 1, j] == 0 or mv >= max_matvec:
                break
        x = x + sum(y[k] * V[k] for k in range(len(y)))
        if res <= rtol * fn:
            break
    pT, pTB, pJ, pK, pS = _one_pass(ops, solver, mat, ct, x[:n], x[n:], True)
    return float(np.sum(pK)), pT, pJ, pK, pS, mv
