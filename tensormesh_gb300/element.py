"""Reference elements: quadrature rules, shape functions and the per-type
tables the CUDA kernels read.

Element types follow the reference's strings (``element/element_type.py``):
``"triangle"`` (P1, 3 nodes), ``"triangle6"`` (P2, 6 nodes), ``"tetra"``
(P1, 4 nodes), ``"tetra10"`` (P2, 10 nodes), ``"quad"`` (Q1, 4 nodes) and
``"quad9"`` (Q2, 9 nodes).  Simplex node order is vertices first, then one
node per edge in the order ``Triangle.edge`` = [[1,2],[0,2],[0,1]]
(``element/element.py:1684``) and ``Tetrahedron.edge`` =
[[2,3],[1,3],[1,2],[0,3],[0,2],[0,1]] (``element/element.py:1949``).
Quadrilaterals live on [0,1]^2 with the vertices in lexicographic order
(0,0), (1,0), (0,1), (1,1), then for Q2 the mid-points of
``Quadrilateral.edge`` = [[0,1],[0,2],[1,3],[2,3]] and the centre
(``element/element.py:1801-1816``, ``element/basis.py:697-748``); their
rule is the tensor product of the Gauss-Legendre line rule of the same
order (``element/quadrature.py:169-203``: points x fastest).

Shape functions are written in barycentric form for simplices (lambda_0 =
1 - sum xi, lambda_k = xi_k): vertex ``i`` has ``lambda_i (2 lambda_i - 1)``
and edge ``(a,b)`` has ``4 lambda_a lambda_b`` for P2; quadrilaterals use
products of the 1-D Lagrange polynomials on the nodes 0, 1 (and 1/2).  The
reference obtains the same polynomials by inverting a monomial Vandermonde
matrix (``element/element.py:557-659``); the two agree to rounding.

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
QUAD_EDGES = ((0, 1), (0, 2), (1, 3), (2, 3))
# reference coordinates of the quadrilateral nodes (element/basis.py:697-748)
QUAD_NODES = {
    1: ((0.0, 0.0), (1.0, 0.0), (0.0, 1.0), (1.0, 1.0)),
    2: ((0.0, 0.0), (1.0, 0.0), (0.0, 1.0), (1.0, 1.0),
        (0.5, 0.0), (0.0, 0.5), (1.0, 0.5), (0.5, 1.0), (0.5, 0.5)),
}


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
    "quad": ElementInfo("quad", 4, 2, 1, 4),
    "quad9": ElementInfo("quad9", 5, 2, 2, 9),
}
QUADRILATERALS = ("quad", "quad9")
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
    if etype in QUADRILATERALS:
        w1, p1 = line_quadrature(order)
        wx, wy = np.meshgrid(w1, w1, indexing="xy")
        px, py = np.meshgrid(p1[:, 0], p1[:, 0], indexing="xy")
        return (wx * wy).ravel(), np.stack([px.ravel(), py.ravel()], 1)
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


def _lagrange_1d(order: int, node: float, s: np.ndarray):
    """The 1-D Lagrange polynomial of ``node`` on the nodes {0, 1} (order 1)
    or {0, 1, 1/2} (order 2) and its derivative, at s."""
    if order == 1:
        return (s, np.ones_like(s)) if node == 1.0 else (1.0 - s, -np.ones_like(s))
    if node == 0.0:
        return (1.0 - s) * (1.0 - 2.0 * s), 4.0 * s - 3.0
    if node == 1.0:
        return s * (2.0 * s - 1.0), 4.0 * s - 1.0
    return 4.0 * s * (1.0 - s), 4.0 - 8.0 * s


def _quad_shape_functions(order: int, xi: np.ndarray):
    Q = xi.shape[0]
    nodes = QUAD_NODES[order]
    phi = np.zeros((Q, len(nodes)))
    dphi = np.zeros((Q, 2, len(nodes)))
    for b, (nx, ny) in enumerate(nodes):
        lx, dx = _lagrange_1d(order, nx, xi[:, 0])
        ly, dy = _lagrange_1d(order, ny, xi[:, 1])
        phi[:, b] = lx * ly
        dphi[:, 0, b] = dx * ly
        dphi[:, 1, b] = lx * dy
    return phi, dphi


def shape_functions(etype: str, xi: np.ndarray):
    """phi [Q, B] and dphi [Q, D, B] (dphi[q, i, b] = d phi_b / d xi_i)."""
    info = element_info(etype)
    if etype in QUADRILATERALS:
        return _quad_shape_functions(info.order, np.asarray(xi, dtype=np.float64))
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


# ---------------------------------------------------------------------------
# Facets (boundary integrals, assemble/facet_assembler.py)
#
# The facets of an element are its edges (2-D) or faces (3-D).  A facet is
# integrated as a simplex of its own: its nodes in facet-local order
# (vertices, then, for P2, the midpoint of facet edge [[1,2],[0,2],[0,1]]),
# its own Lagrange basis -- the element's basis restricted to the facet --
# and the measure sqrt(det(F^T F)) of its map from the reference facet.
# Line facets use Gauss-Legendre on [0, 1] (element/quadrature.py:13-66),
# triangle facets the triangle rule above.

# Gauss-Legendre nodes on [-1, 1] and weights, orders 1-7: the decimal
# values of element/quadrature.py:36-53, mapped to [0, 1] below
_GL = {
    1: ([2.0], [0.0]),
    2: ([1.0, 1.0], [-0.57735026918962576451, 0.57735026918962576451]),
    3: ([0.55555555555555555556, 0.88888888888888888889, 0.55555555555555555556],
        [-0.77459666924148337704, 0.0, 0.77459666924148337704]),
    4: ([0.34785484513745385737, 0.65214515486254614263, 0.65214515486254614263, 0.34785484513745385737],
        [-0.8611363115940526, -0.3399810435848563, 0.3399810435848563, 0.8611363115940526]),
    5: ([0.23692688505618908751, 0.47862867049936646804, 0.56888888888888888889, 0.47862867049936646804,
         0.23692688505618908751],
        [-0.9061798459386640, -0.5384693101056831, 0.0, 0.5384693101056831, 0.9061798459386640]),
    6: ([0.17132449237917034504, 0.36076157304813860757, 0.46791393457269104739, 0.46791393457269104739,
         0.36076157304813860757, 0.17132449237917034504],
        [-0.9324695142031521, -0.6612093864662645, -0.2386191860831969, 0.2386191860831969,
         0.6612093864662645, 0.9324695142031521]),
    7: ([0.12948496616886969327, 0.27970539148927666790, 0.38183005050511894495, 0.41795918367346938776,
         0.38183005050511894495, 0.27970539148927666790, 0.12948496616886969327],
        [-0.9491079123427585, -0.7415311855993945, -0.4058451513773972, 0.0, 0.4058451513773972,
         0.7415311855993945, 0.9491079123427585]),
}


def line_quadrature(order: int) -> Tuple[np.ndarray, np.ndarray]:
    """Gauss-Legendre rule on [0, 1]: weights (sum 1) and points [Q, 1]."""
    if order not in _GL:
        raise NotImplementedError(f"line quadrature order {order} is not tabulated (orders 1-7)")
    w, p = _GL[order]
    return np.array(w, dtype=np.float64) / 2.0, ((np.array(p, dtype=np.float64) + 1.0) / 2.0)[:, None]


def _edge_node(a: int, b: int, edges, base: int) -> int:
    for k, (x, y) in enumerate(edges):
        if {x, y} == {a, b}:
            return base + k
    raise ValueError((a, b))


def _facet_nodes(etype: str):
    """Local node lists of the element's facets, each in facet-local order."""
    if etype == "triangle":
        return [(0, 1), (1, 2), (2, 0)]
    if etype == "tetra":
        return [(0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)]
    if etype == "triangle6":
        return [(a, b, _edge_node(a, b, TRI_EDGES, 3)) for a, b in [(0, 1), (1, 2), (2, 0)]]
    if etype == "tetra10":
        out = []
        for a, b, c in [(0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)]:
            out.append((a, b, c, _edge_node(b, c, TET_EDGES, 4), _edge_node(a, c, TET_EDGES, 4),
                        _edge_node(a, b, TET_EDGES, 4)))
        return out
    if etype == "quad":
        return list(QUAD_EDGES)
    if etype == "quad9":
        return [(a, b, 4 + k) for k, (a, b) in enumerate(QUAD_EDGES)]
    raise NotImplementedError(f"facets of {etype!r}")


# facet code of the C ABI: (facet dimension, facet order) -> TM_FACET_*
FACET_CODES = {(1, 1): 0, (1, 2): 1, (2, 1): 2, (2, 2): 3}


@dataclass(frozen=True)
class FacetInfo:
    element: str
    facet_dim: int     # 1 (lines, in 2-D) or 2 (triangles, in 3-D)
    order: int
    n_basis: int       # nodes per facet
    code: int          # TM_FACET_*
    nodes: tuple       # local node lists of the element's facets


def facet_info(etype: str) -> FacetInfo:
    info = element_info(etype)
    fd = info.dim - 1
    nodes = tuple(_facet_nodes(etype))
    return FacetInfo(etype, fd, info.order, len(nodes[0]), FACET_CODES[(fd, info.order)], nodes)


def facet_shape_functions(facet_dim: int, order: int, t: np.ndarray):
    """psi [Q, Bf] and dpsi [Q, facet_dim, Bf] of the facet's own Lagrange
    basis at facet-local points t [Q, facet_dim]."""
    t = np.asarray(t, dtype=np.float64)
    if facet_dim == 1:
        s = t[:, 0]
        lam = np.stack([1.0 - s, s], 1)
        dlam = np.array([[-1.0, 1.0]])
        if order == 1:
            return lam, np.broadcast_to(dlam, (len(s), 1, 2)).copy()
        psi = np.stack([lam[:, 0] * (2 * lam[:, 0] - 1), lam[:, 1] * (2 * lam[:, 1] - 1), 4 * lam[:, 0] * lam[:, 1]], 1)
        d = np.stack([(4 * lam[:, 0] - 1) * dlam[0, 0], (4 * lam[:, 1] - 1) * dlam[0, 1],
                      4 * (lam[:, 0] * dlam[0, 1] + lam[:, 1] * dlam[0, 0])], 1)
        return psi, d[:, None, :]
    return shape_functions("triangle" if order == 1 else "triangle6", t)


@lru_cache(maxsize=None)
def facet_tables(etype: str, qorder: int) -> Dict[str, np.ndarray]:
    """Weights, psi and dpsi of the facets of ``etype`` at the facet
    quadrature of order ``qorder``."""
    fi = facet_info(etype)
    if fi.facet_dim == 1:
        w, t = line_quadrature(qorder)
    else:
        w, t = quadrature("triangle", qorder)
    psi, dpsi = facet_shape_functions(fi.facet_dim, fi.order, t)
    return {"w": w, "t": t, "psi": psi, "dpsi": dpsi}


def packed_facet_tables(etype: str, qorder: int) -> np.ndarray:
    """[w(Q) | psi(Q*Bf) | dpsi(Q*(D-1)*Bf)] float64, the layout of
    ``tm_facet_tables``."""
    t = facet_tables(etype, qorder)
    return np.concatenate([t["w"].ravel(), t["psi"].ravel(), t["dpsi"].ravel()]).astype(np.float64)
