"""FP64 restatement of the reference's alignment caller (numpy over the oracle).

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` as the checker of
``pointint_gb300.align``; the product never imports it.

Restates PoIntInt ``cpp/app/align``:
  * ``similarity`` — similarity_measure.cpp:9-157 (Ochiai / Jaccard / Dice,
    gradient and Gauss-Newton Hessian of -log(similarity)), on the volume
    matrix, gradients and hessian_ij of ``oracle.volume_matrix`` (the
    restatement of compute_intersection_volume_multi_object.cpp:31-292);
  * ``optimize_alignment`` — optimizer.cpp:8-133;
  * ``compute_moments`` / ``compute_warm_start`` — warm_start.cpp:8-243.
Eigenvectors follow numpy's ``eigh`` (ascending eigenvalues), each made to
have its largest-magnitude component positive — the same canonical choice as
the product, since the reference leaves their signs to Eigen's solver.
"""
from __future__ import annotations

import numpy as np

from . import oracle as orc

OCHIAI, JACCARD, DICE = 0, 1, 2
FUNC_ONLY, GRADIENT, HESSIAN, ALL = 1, 2, 4, 7
IDENTITY = orc.IDENTITY_AFFINE


def similarity(geom1, geom2, dofs2, kgrid, measure: int, V1: float, flags: int = FUNC_ONLY | GRADIENT) -> dict:
    """geom = (geom_type, elems).  similarity_measure.cpp:9-157."""
    need_g, need_h = bool(flags & GRADIENT), bool(flags & HESSIAN)
    objs = [orc.Obj(geom1[0], geom1[1], orc.DOF_AFFINE, IDENTITY.copy()),
            orc.Obj(geom2[0], geom2[1], orc.DOF_AFFINE, np.asarray(dofs2, dtype=np.float64).copy())]
    vf = orc.VOLUME_ONLY | (orc.GRADIENT if need_g else 0) | (orc.HESSIAN if need_h else 0)
    V, grad, hess = orc.volume_matrix(objs, kgrid, vf)
    Vint, V2 = V[0, 1], V[1, 1]
    gI = grad[1][0] if need_g else np.zeros(12)
    g2 = 2.0 * grad[1][1] if need_g else np.zeros(12)
    HI = np.zeros((12, 12))  # hessian_jj[0][1]: zero in the Gauss-Newton form
    H2 = (hess[1][1] + hess[1][1].T) if need_h else np.zeros((12, 12))  # + hessian_ii + hessian_jj (zero)
    if measure == OCHIAI:
        inv = 1.0 / np.sqrt(V1 * V2)
        s = inv * Vint
        gs = inv * gI + (-0.5 * inv ** 3 * Vint * V1) * g2
        Hs = (inv * HI - 0.5 * inv * Vint / V2 * H2 + 0.75 * inv * Vint / V2 ** 2 * np.outer(g2, g2)
              - 0.5 * inv / V2 * (np.outer(gI, g2) + np.outer(g2, gI)))
    elif measure == JACCARD:
        den = V1 + V2 - Vint
        s = Vint / den
        dD = g2 - gI
        gs = gI / den - Vint / den ** 2 * dD
        Hs = (HI / den - Vint / den ** 2 * (H2 - HI) - (np.outer(gI, dD) + np.outer(dD, gI)) / den ** 2
              + 2.0 * Vint / den ** 3 * np.outer(dD, dD))
    else:
        den = V1 + V2
        s = 2.0 * Vint / den
        inv, coeff = 2.0 / den, -2.0 * Vint / den ** 2
        gs = inv * gI + coeff * g2
        Hs = (inv * HI + coeff * H2 - inv / den * (np.outer(gI, g2) + np.outer(g2, gI))
              - 2.0 * coeff / den * np.outer(g2, g2))
    ss = max(s, 1e-10)
    out = {"similarity": s, "value": -np.log(ss), "gradient": None, "hessian": None}
    if need_g:
        out["gradient"] = -gs / ss
    if need_h:
        out["hessian"] = np.outer(gs, gs) / ss ** 2 - Hs / ss
    return out


def optimize_alignment(geom1, geom2, initial_dofs, kgrid, measure, V1, tolerance=1e-6, max_iterations=50,
                       damping=0.1, first_step_only=False) -> dict:
    """optimizer.cpp:8-133.  Returns the final state and the Newton direction
    of the first iteration."""
    dofs = np.asarray(initial_dofs, dtype=np.float64).copy()
    st = {"converged": False, "status": "", "iteration": 0, "first_delta": None}
    for it in range(max_iterations):
        st["iteration"] = it
        r = similarity(geom1, geom2, dofs, kgrid, measure, V1, ALL)
        st["similarity"], st["similarity_loss"] = r["similarity"], r["value"]
        g, H = r["gradient"], r["hessian"]
        if np.linalg.norm(g) < tolerance:
            st["converged"], st["status"] = True, "Converged (gradient norm < tolerance)"
            break
        lam, Qm = np.linalg.eigh(H)
        Hf = Qm @ np.diag(np.maximum(lam, 0.0)) @ Qm.T + damping * np.eye(12)
        delta = np.linalg.solve(Hf, -g)
        if st["first_delta"] is None:
            st["first_delta"] = delta.copy()
            if first_step_only:
                break
        descent = -delta @ g
        f0, alpha = r["value"], 1.0
        f_new = similarity(geom1, geom2, dofs + alpha * delta, kgrid, measure, V1, FUNC_ONLY)["value"]
        ls = 0
        while f_new > f0 - 0.1 * alpha * descent and alpha > 1e-10 and ls < 20:
            alpha *= 0.5
            f_new = similarity(geom1, geom2, dofs + alpha * delta, kgrid, measure, V1, FUNC_ONLY)["value"]
            ls += 1
        if alpha <= 1e-10:
            st["status"] = "Line search failed (step size too small)"
            break
        dofs = dofs + alpha * delta
    if not st["converged"]:
        st["status"] = "Reached max iterations"
    st["dofs"] = dofs
    return st


def _affine(dofs):
    d = np.asarray(dofs, dtype=np.float64)
    return d[3:].reshape(3, 3), d[:3]


def compute_moments(geom_type: int, elems: np.ndarray, dofs=IDENTITY):
    """warm_start.cpp:8-131 -> (volume, centroid, covariance)."""
    A, t = _affine(dofs)
    if geom_type == orc.GEOM_TRIANGLE:
        a0 = elems["a"]
        a = a0 @ A.T + t
        b = (a0 + elems["e1"]) @ A.T + t
        c = (a0 + elems["e2"]) @ A.T + t
        vt = np.einsum("ij,ij->i", a, np.cross(b - a, c - a)) / 6.0
        ct = (a + b + c) / 4.0
        V = vt.sum()
        if abs(V) <= 1e-10:
            return 0.0, np.zeros(3), np.zeros((3, 3))
        cen = (vt[:, None] * ct).sum(0) / V
        return V, cen, np.einsum("i,ij,ik->jk", vt, ct, ct) / V - np.outer(cen, cen)
    disk = geom_type == orc.GEOM_DISK
    V = orc.self_volume(orc.Obj(geom_type, elems, orc.DOF_AFFINE, np.asarray(dofs, dtype=np.float64)))
    c = elems["c"] @ A.T + t
    wt = elems["area"] if disk else elems["w"]
    W = wt.sum()
    cen = (wt[:, None] * c).sum(0) / W if W > 1e-10 else np.zeros(3)
    d = c - cen
    cov = np.einsum("i,ij,ik->jk", wt, d, d)
    if not disk:
        cov = cov + (wt * elems["sigma"] ** 2).sum() * np.eye(3)
    if W > 1e-10:
        cov = cov / W
    return V, cen, cov


def _canonical_eigh(C):
    lam, P = np.linalg.eigh(C)
    for k in range(3):
        i = np.argmax(np.abs(P[:, k]))
        if P[i, k] < 0:
            P[:, k] = -P[:, k]
    return lam, P


def compute_warm_start(geom1, geom2) -> np.ndarray:
    """warm_start.cpp:133-243.  geom = (geom_type, elems)."""
    v1, c1, C1 = compute_moments(*geom1)
    v2, c2, C2 = compute_moments(*geom2)
    l1, P1 = _canonical_eigh(C1)
    l2, P2 = _canonical_eigh(C2)
    for P in (P1, P2):
        if np.linalg.det(P) < 0:
            P[:, 2] = -P[:, 2]
    U, _, Vt = np.linalg.svd(P1 @ P2.T)
    R = U @ Vt
    if np.linalg.det(R) < 0:
        U[:, 2] = -U[:, 2]
        R = U @ Vt
    if abs(v2) > 1e-10:
        s = np.cbrt(v1 / v2)
    else:
        r = [np.sqrt(l1[i] / l2[i]) for i in range(3) if l2[i] > 1e-6]
        s = np.mean(r) if r else 1.0
    s = min(10.0, max(0.1, s))
    A = s * R
    return np.concatenate([c1 - A @ c2, A.reshape(-1)])
