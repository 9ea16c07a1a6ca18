"""Reference elements: quadrature rules, shape functions and the per-type
tables the CUDA kernels read.

Element types follow the reference's strings (``element/element_type.py``):
``"triangle"`` (P1, 3 nodes), ``"triangle6"`` (P2, 6 nodes), ``"tetra"``
(P1, 4 nodes), ``"tetra10"`` (P2, 10 nodes).  Node order is vertices first,
then one node per edge in the order ``Triangle.edge`` = [[1,2],[0,2],[0,1]]
(``element/element.py:1684``) and ``Tetrahedron.edge`` =
[[2,3],[1,3],[1,2],[0,3],[0,2],[0,1]] (``element/element.py:1949``).

Shape functions are written in barycentric form (lambda_0 = 1 - sum xi,
lambda_k = xi_k): vertex ``i`` has ``lambda_i (2 lambda_i - 1)`` and edge
``(a,b)`` has ``4 lambda_a lambda_b`` for P2.  The reference obtains the
same polynomials by inverting a monomial Vandermonde matrix
(``element/element.py:557-659``); the two agree to rounding.

Quadrature tables are the reference's decimal tables for orders 1-4
(``element/quadrature.py:68-166``), kept identical so that both sides
integrate with the same nodes and weights.
"""
from dataclasses import dataclass
from functools import lru_cache
from typing import Dict, Tuple

import numpy as np

TRI_QUAD = {
    1: ([0.5], [[0.3333333333333333, 0.3333333333333333]]),
    2: ([0.16666666666666666] * 3,
        [[0.16666666666666666, 0.16666666666666666], [0.6666666666666666, 0.16666666666666666],
         [0.16666666666666666, 0.6666666666666666]]),
    3: ([-0.28125, 0.260416666666667, 0.260416666666667, 0.260416666666667],
        [[0.333333333333333, 0.333333333333333], [0.2, 0.6], [0.6, 0.2], [0.2, 0.2]]),
    4: ([0.111690794839006, 0.054975871827661, 0.111690794839006,
         0.054975871827661, 0.111690794839006, 0.054975871827661],
        [[0.445948490915965, 0.10810301816807], [0.0915762135097699, 0.816847572980459],
         [0.10810301816807, 0.445948490915965], [0.816847572980459, 0.091576213509771],
         [0.445948490915965, 0.445948490915965], [0.091576213509771, 0.0915762135097699]]),
}
_A, _B = 0.5854101966249685, 0.1381966011250105
_S6 = 0.1666666666666667
_T1, _T2 = 0.7857142857142857, 0.0714285714285714
_U1, _U2 = 0.1005964238332008, 0.3994035761667992
TET_QUAD = {
    1: ([0.16666666666666666], [[0.25, 0.25, 0.25]]),
    2: ([0.041666666666666664] * 4,
        [[_A, _B, _B], [_B, _B, _B], [_B, _B, _A], [_B, _A, _B]]),
    3: ([-0.13333333333333333, 0.075, 0.075, 0.075, 0.075],
        [[0.25, 0.25, 0.25], [0.5, _S6, _S6], [_S6, _S6, _S6], [_S6, _S6, 0.5], [_S6, 0.5, _S6]]),
    4: ([-0.01315555555555555] + [0.007622222222222217] * 4 + [0.02488888888888888] * 6,
        [[0.25, 0.25, 0.25], [_T1, _T2, _T2], [_T2, _T2, _T2], [_T2, _T2, _T1], [_T2, _T1, _T2],
         [_U1, _U2, _U2], [_U2, _U1, _U2], [_U2, _U2, _U1], [_U2, _U1, _U1], [_U1, _U2, _U1],
         [_U1, _U1, _U2]]),
}

TRI_EDGES = ((1, 2), (0, 2), (0, 1))
TET_EDGES = ((2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1))


@dataclass(frozen=True)
class ElementInfo:
    name: str
    code: int        # element-type code of the C ABI (TM_TRI3 ...)
    dim: int
    order: int
    n_basis: int


ELEMENTS: Dict[str, ElementInfo] = {
    "triangle": ElementInfo("triangle", 0, 2, 1, 3),
    "tetra": ElementInfo("tetra", 1, 3, 1, 4),
    "triangle6": ElementInfo("triangle6", 2, 2, 2, 6),
    "tetra10": ElementInfo("tetra10", 3, 3, 2, 10),
}
# element_type2dimension / element_type2order of the reference, for the
# types this package assembles
element_type2dimension = {k: v.dim for k, v in ELEMENTS.items()}
element_type2order = {k: v.order for k, v in ELEMENTS.items()}


def element_info(etype: str) -> ElementInfo:
    if etype not in ELEMENTS:
        raise NotImplementedError(
            f"element type {etype!r} is not assembled by tensormesh_gb300 "
            f"(supported: {sorted(ELEMENTS)})")
    return ELEMENTS[etype]


def quadrature(etype: str, order: int) -> Tuple[np.ndarray, np.ndarray]:
    info = element_info(etype)
    table = TRI_QUAD if info.dim == 2 else TET_QUAD
    if order not in table:
        raise NotImplementedError(f"quadrature order {order} is not tabulated (orders {sorted(table)})")
    w, p = table[order]
    return np.array(w, dtype=np.float64), np.array(p, dtype=np.float64)


def _barycentric(xi: np.ndarray):
    """lambda [Q, D+1] and d lambda / d xi [D, D+1]."""
    Q, D = xi.shape
    lam = np.concatenate([1.0 - xi.sum(1, keepdims=True), xi], axis=1)
    dlam = np.concatenate([-np.ones((D, 1)), np.eye(D)], axis=1)
    return lam, dlam


def shape_functions(etype: str, xi: np.ndarray):
    """phi [Q, B] and dphi [Q, D, B] (dphi[q, i, b] = d phi_b / d xi_i)."""
    info = element_info(etype)
    lam, dlam = _barycentric(np.asarray(xi, dtype=np.float64))
    Q, D = xi.shape
    if info.order == 1:
        phi = lam
        dphi = np.broadcast_to(dlam, (Q, D, D + 1)).copy()
        return phi, dphi
    edges = TRI_EDGES if D == 2 else TET_EDGES
    nv = D + 1
    B = nv + len(edges)
    phi = np.zeros((Q, B))
    dphi = np.zeros((Q, D, B))
    for i in range(nv):
        phi[:, i] = lam[:, i] * (2.0 * lam[:, i] - 1.0)
        dphi[:, :, i] = (4.0 * lam[:, i] - 1.0)[:, None] * dlam[None, :, i]
    for k, (a, b) in enumerate(edges):
        phi[:, nv + k] = 4.0 * lam[:, a] * lam[:, b]
        dphi[:, :, nv + k] = 4.0 * (lam[:, a][:, None] * dlam[None, :, b]
                                    + lam[:, b][:, None] * dlam[None, :, a])
    return phi, dphi


@lru_cache(maxsize=None)
def element_tables(etype: str, qorder: int) -> Dict[str, np.ndarray]:
    """Everything the kernels need about one (element type, quadrature
    order): weights, phi, dphi at the quadrature points, the reference mass
    matrix sum_q w phi_a phi_b and load vector sum_q w phi_a."""
    w, xi = quadrature(etype, qorder)
    phi, dphi = shape_functions(etype, xi)
    mass_hat = np.einsum("q,qa,qb->ab", w, phi, phi)
    load_hat = np.einsum("q,qa->a", w, phi)
    return {"w": w, "xi": xi, "phi": phi, "dphi": dphi, "mass_hat": mass_hat,
            "load_hat": load_hat, "wsum": np.array([w.sum()])}


def packed_tables(etype: str, qorder: int) -> np.ndarray:
    """Tables in the flat float64 layout of ``tm_element_tables``:
    [w(Q) | phi(Q*B) | dphi(Q*D*B) | mass_hat(B*B) | load_hat(B) | wsum]."""
    t = element_tables(etype, qorder)
    return np.concatenate([t["w"].ravel(), t["phi"].ravel(), t["dphi"].ravel(),
                           t["mass_hat"].ravel(), t["load_hat"].ravel(), t["wsum"]]).astype(np.float64)
