"""Oracle for the tensorized-assembly path -- TEST INFRASTRUCTURE ONLY.

A CPU restatement, in plain torch/numpy FP64, of the reference's assembly
algorithm (TensorMesh).  It follows the reference's own op sequence --
gather of element coordinates, transposed-Jacobian einsum, batched
``torch.inverse``, gradient einsum, ``|det J| * w``, the integrand, the
quadrature contraction and the ``index_add_`` scatter -- so that it can be
compared with the reference on the golden fixtures and then used as the
checker of the CUDA path.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module.  The product (``tensormesh_gb300``) never
does: it has no CPU path.
"""
from typing import Dict, Optional, Sequence, Tuple

import hashlib
import numpy as np
import scipy.sparse
import scipy.sparse.linalg
import torch

DT = torch.float64

# ---------------------------------------------------------------------------
# Quadrature rules (element/quadrature.py:68-166).  Same decimal tables as the
# reference for orders 1-4, so that the oracle reproduces its rounding.
# ---------------------------------------------------------------------------
_TRI_W = {
    1: [0.5],
    2: [0.16666666666666666] * 3,
    3: [-0.28125, 0.260416666666667, 0.260416666666667, 0.260416666666667],
    4: [0.111690794839006, 0.054975871827661, 0.111690794839006,
        0.054975871827661, 0.111690794839006, 0.054975871827661],
}
_TRI_P = {
    1: [[0.3333333333333333, 0.3333333333333333]],
    2: [[0.16666666666666666, 0.16666666666666666], [0.6666666666666666, 0.16666666666666666],
        [0.16666666666666666, 0.6666666666666666]],
    3: [[0.333333333333333, 0.333333333333333], [0.2, 0.6], [0.6, 0.2], [0.2, 0.2]],
    4: [[0.445948490915965, 0.10810301816807], [0.0915762135097699, 0.816847572980459],
        [0.10810301816807, 0.445948490915965], [0.816847572980459, 0.091576213509771],
        [0.445948490915965, 0.445948490915965], [0.091576213509771, 0.0915762135097699]],
}
_TET_W = {
    1: [0.16666666666666666],
    2: [0.041666666666666664] * 4,
    3: [-0.13333333333333333, 0.075, 0.075, 0.075, 0.075],
    4: [-0.01315555555555555] + [0.007622222222222217] * 4 + [0.02488888888888888] * 6,
}
_TET_P = {
    1: [[0.25, 0.25, 0.25]],
    2: [[0.5854101966249685, 0.1381966011250105, 0.1381966011250105],
        [0.1381966011250105, 0.1381966011250105, 0.1381966011250105],
        [0.1381966011250105, 0.1381966011250105, 0.5854101966249685],
        [0.1381966011250105, 0.5854101966249685, 0.1381966011250105]],
    3: [[0.25, 0.25, 0.25], [0.5, 0.1666666666666667, 0.1666666666666667],
        [0.1666666666666667, 0.1666666666666667, 0.1666666666666667],
        [0.1666666666666667, 0.1666666666666667, 0.5],
        [0.1666666666666667, 0.5, 0.1666666666666667]],
    4: [[0.25, 0.25, 0.25], [0.7857142857142857, 0.0714285714285714, 0.0714285714285714],
        [0.0714285714285714, 0.0714285714285714, 0.0714285714285714],
        [0.0714285714285714, 0.0714285714285714, 0.7857142857142857],
        [0.0714285714285714, 0.7857142857142857, 0.0714285714285714],
        [0.1005964238332008, 0.3994035761667992, 0.3994035761667992],
        [0.3994035761667992, 0.1005964238332008, 0.3994035761667992],
        [0.3994035761667992, 0.3994035761667992, 0.1005964238332008],
        [0.3994035761667992, 0.1005964238332008, 0.1005964238332008],
        [0.1005964238332008, 0.3994035761667992, 0.1005964238332008],
        [0.1005964238332008, 0.1005964238332008, 0.3994035761667992]],
}

ELEMENT = {  # type -> (dim, order, n_basis)   (element/element_type.py:57-87)
    "triangle": (2, 1, 3), "triangle6": (2, 2, 6),
    "tetra": (3, 1, 4), "tetra10": (3, 2, 10),
    "quad": (2, 1, 4), "quad9": (2, 2, 9),
}
_QUADS = ("quad", "quad9")
_QUAD_VERTS = [[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0]]  # element.py:1811
_QUAD_EDGE = [[0, 1], [0, 2], [1, 3], [2, 3]]                   # element.py:1813
_TRI_EDGE = [[1, 2], [0, 2], [0, 1]]                          # element.py:1684
_TET_EDGE = [[2, 3], [1, 3], [1, 2], [0, 3], [0, 2], [0, 1]]  # element.py:1949


def quadrature(etype: str, order: int) -> Tuple[torch.Tensor, torch.Tensor]:
    if etype in _QUADS:
        return quad_quadrature(order)
    dim = ELEMENT[etype][0]
    w, p = (_TRI_W, _TRI_P) if dim == 2 else (_TET_W, _TET_P)
    return torch.tensor(w[order], dtype=DT), torch.tensor(p[order], dtype=DT)


def quad_quadrature(order: int) -> Tuple[torch.Tensor, torch.Tensor]:
    """element/quadrature.py:169-203: the line rule on [0, 1] in each
    direction, torch.meshgrid(..., indexing='xy') flattened (x fastest)."""
    w1, p1 = _facet_rule(2, order)
    wx, wy = torch.meshgrid(w1, w1, indexing="xy")
    px, py = torch.meshgrid(p1[:, 0], p1[:, 0], indexing="xy")
    return (wx * wy).flatten(), torch.stack([px.flatten(), py.flatten()], -1)


def n_vertices(etype: str) -> int:
    return 4 if etype in _QUADS else ELEMENT[etype][0] + 1


def basis_nodes(etype: str) -> torch.Tensor:
    """Reference-element nodes: vertices, then edge mid-points in the
    element's edge order (element/basis.py:639-695, 750-860); for
    quadrilaterals the lexicographic vertices, the mid-points of their edges
    and the centre (element/basis.py:697-748)."""
    dim, order, _ = ELEMENT[etype]
    if etype in _QUADS:
        verts = torch.tensor(_QUAD_VERTS, dtype=DT)
        if order == 1:
            return verts
        mids = torch.stack([(verts[a] + verts[b]) / 2 for a, b in _QUAD_EDGE])
        return torch.cat([verts, mids, verts.mean(0, keepdim=True)], 0)
    verts = torch.cat([torch.zeros(1, dim, dtype=DT), torch.eye(dim, dtype=DT)], 0)
    if order == 1:
        return verts
    edges = _TRI_EDGE if dim == 2 else _TET_EDGE
    mids = torch.stack([(verts[a] + verts[b]) / 2 for a, b in edges])
    return torch.cat([verts, mids], 0)


def _monomials(dim: int, order: int, tensor: bool = False):
    """Exponents by total degree (element/polynomial.py): complete
    polynomials of degree ``order`` for simplices, every exponent up to
    ``order`` in each variable for the tensor-product (quadrilateral) space."""
    exps = []
    for tot in range((dim if tensor else 1) * order + 1):
        if dim == 2:
            for a in range(tot, -1, -1):
                if not tensor or (a <= order and tot - a <= order):
                    exps.append((a, tot - a))
        else:
            for a in range(tot, -1, -1):
                for b in range(tot - a, -1, -1):
                    exps.append((a, b, tot - a - b))
    return exps


def element_monomials(etype: str):
    dim, order, _ = ELEMENT[etype]
    return _monomials(dim, order, tensor=etype in _QUADS)


def _eval_monomials(exps, pts: torch.Tensor) -> torch.Tensor:
    return torch.stack([torch.prod(pts ** torch.tensor(e, dtype=DT), -1) for e in exps], -1)


def _eval_monomial_grads(exps, pts: torch.Tensor) -> torch.Tensor:
    """[Q, dim, n_mono] derivatives of the monomials."""
    out = []
    dim = pts.shape[-1]
    for d in range(dim):
        cols = []
        for e in exps:
            if e[d] == 0:
                cols.append(torch.zeros(pts.shape[0], dtype=DT))
            else:
                e2 = list(e)
                e2[d] -= 1
                cols.append(e[d] * torch.prod(pts ** torch.tensor(e2, dtype=DT), -1))
        out.append(torch.stack(cols, -1))
    return torch.stack(out, 1)


def shape_tables(etype: str, qorder: int):
    """(w [Q], phi [Q,B], dphi [Q,D,B]) via the inverse monomial Vandermonde
    matrix at the basis nodes (element/element.py:557-716, 804-872)."""
    dim, order, nb = ELEMENT[etype]
    w, q = quadrature(etype, qorder)
    exps = element_monomials(etype)
    V = _eval_monomials(exps, basis_nodes(etype))        # [B, n_mono]
    coef = torch.linalg.inv(V).T                          # element.py:657
    phi = _eval_monomials(exps, q) @ coef.T               # [Q, B]
    dphi = torch.einsum("qdm,bm->qdb", _eval_monomial_grads(exps, q), coef)
    return w, phi, dphi


# ---------------------------------------------------------------------------
# Geometry: element.py:875-968 and transformation.py:1219-1276
# ---------------------------------------------------------------------------
def shape_grad_jxw(points: torch.Tensor, conn: torch.Tensor, etype: str, qorder: int = 2):
    w, _, dphi = shape_tables(etype, qorder)
    X = points[conn]                                                 # transformation.py:219
    J = torch.einsum("ebj,qib->eqij", X, dphi)                        # element.py:962
    Jinv = torch.inverse(J)                                          # element.py:964
    grad = torch.einsum("qib,eqji->eqbj", dphi, Jinv)                 # element.py:966
    jxw = torch.einsum("q,eq->eq", w, torch.linalg.det(J).abs())      # transformation.py:1272
    return grad, jxw


# ---------------------------------------------------------------------------
# Sparsity pattern and slot map: element_assembler.py:811-830
# ---------------------------------------------------------------------------
def element_pattern(conn: torch.Tensor, n_points: int):
    """Return (edges int32 [2,nnz], slot map int64 [E*B*B])."""
    c = conn.cpu().numpy().astype(np.int64)
    E, B = c.shape
    eu = np.repeat(c[:, :, None], B, axis=2).reshape(-1)
    ev = np.repeat(c[:, None, :], B, axis=1).reshape(-1)
    tmp = scipy.sparse.coo_matrix((np.ones_like(eu), (eu, ev)),
                                  shape=(n_points, n_points)).tocsr().tocoo()
    edge_u, edge_v = tmp.row, tmp.col
    eids = scipy.sparse.coo_matrix((np.arange(len(edge_u)), (edge_u, edge_v)),
                                   shape=(n_points, n_points)).tocsr()
    slot = np.asarray(eids[eu, ev]).ravel().astype(np.int64)
    edges = np.stack([edge_u, edge_v], 0).astype(np.int32)
    return torch.from_numpy(edges), torch.from_numpy(slot)


def reduce_project(indices: torch.Tensor, x: torch.Tensor, to_size: int) -> torch.Tensor:
    """projector.py:95-123: zeros(to).index_add_(0, indices, x)."""
    x = x.reshape(indices.shape[0], *x.shape[indices.dim():]) if x.dim() > 1 else x
    out = torch.zeros(to_size, *x.shape[1:], dtype=x.dtype)
    return out.index_add_(0, indices, x)


def layout_hash(row: torch.Tensor, col: torch.Tensor) -> str:
    """sparse/matrix.py:82-86."""
    return hashlib.sha256(row.detach().cpu().numpy().tobytes()
                          + col.detach().cpu().numpy().tobytes()).hexdigest()


def block_coo_indices(row: torch.Tensor, col: torch.Tensor, H: int):
    """sparse/matrix.py:332-381: row*H+a, col*H+b in [edge, a, b] order."""
    a = torch.arange(H).repeat_interleave(H)
    b = torch.arange(H).repeat(H)
    return ((row.long()[:, None] * H + a).reshape(-1), (col.long()[:, None] * H + b).reshape(-1))


# ---------------------------------------------------------------------------
# Forms (element_assembler.py:390-445 with the integrands of builtin.py)
# ---------------------------------------------------------------------------
def _chunks(E: int, chunk: int):
    for s in range(0, E, chunk):
        yield s, min(E, s + chunk)


def element_locals_diffusion(points, conn, etype, kappa=None, qorder=2):
    """K_e[i,j] = kappa_e sum_q jxw gradu_i . gradv_j  (builtin.py:61-62)."""
    grad, jxw = shape_grad_jxw(points, conn, etype, qorder)
    integ = torch.einsum("eqid,eqjd->eqij", grad, grad)
    if kappa is not None:
        integ = kappa[:, None, None, None] * integ
    return torch.einsum("eqij,eq->eij", integ, jxw)                  # element_assembler.py:199


def element_locals_mass(points, conn, etype, qorder=2):
    """M_e[i,j] = sum_q jxw phi_i phi_j  (builtin.py:99-100, 'qij,eq->eij')."""
    _, phi, _ = shape_tables(etype, qorder)
    _, jxw = shape_grad_jxw(points, conn, etype, qorder)
    integ = phi[:, :, None] * phi[:, None, :]
    return torch.einsum("qij,eq->eij", integ, jxw)                   # element_assembler.py:208


def voigt_B(grad: torch.Tensor) -> torch.Tensor:
    """functional/elasticity.py:132-200: rows [xx,yy,(zz),(yz,xz),xy]."""
    D = grad.shape[-1]
    z = torch.zeros_like(grad[..., 0])
    g = [grad[..., d] for d in range(D)]
    if D == 2:
        rows = [[g[0], z], [z, g[1]], [g[1], g[0]]]
    else:
        rows = [[g[0], z, z], [z, g[1], z], [z, z, g[2]],
                [z, g[2], g[1]], [g[2], z, g[0]], [g[1], g[0], z]]
    return torch.stack([torch.stack(r, -1) for r in rows], -2)       # [..., 3|6, D]


def voigt_C(E: torch.Tensor, nu: float, D: int) -> torch.Tensor:
    """functional/elasticity.py:202-284 for a batch of Young's moduli."""
    mu = E / (2. * (1. + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    n = 3 if D == 2 else 6
    C = torch.zeros(E.shape[0], n, n, dtype=DT)
    for k in range(n):
        C[:, k, k] = mu
    for a in range(D):
        for b in range(D):
            C[:, a, b] = C[:, a, b] + lam
        C[:, a, a] = C[:, a, a] + mu
    return C


def element_locals_elasticity(points, conn, etype, E, nu=0.3, qorder=2):
    """Block [i,j,a,b] = sum_q jxw (B_i^T C B_j)[a,b]  (builtin.py:172-178)."""
    grad, jxw = shape_grad_jxw(points, conn, etype, qorder)
    D = grad.shape[-1]
    if not torch.is_tensor(E):
        E = torch.full((conn.shape[0],), float(E), dtype=DT)
    Bm = voigt_B(grad)                                               # [e,q,b,k,a]
    C = voigt_C(E, nu, D)
    integ = torch.einsum("eqika,ekl,eqjlb->eqijab", Bm, C, Bm)
    return torch.einsum("eqijab,eq->eijab", integ, jxw)


def assemble_matrix(points, conn, n_points, local_fn, chunk=1 << 15, **kw):
    """Run ``local_fn`` over element chunks and scatter with the slot map."""
    edges, slot = element_pattern(conn, n_points)
    nnz = edges.shape[1]
    out = None
    B = conn.shape[1]
    for s, e in _chunks(conn.shape[0], chunk):
        kwc = {k: (v[s:e] if torch.is_tensor(v) and v.dim() > 0 and v.shape[0] == conn.shape[0] else v)
               for k, v in kw.items()}
        loc = local_fn(points, conn[s:e], **kwc)
        flat = loc.reshape((e - s) * B * B, *loc.shape[3:])
        part = reduce_project(slot[s * B * B:e * B * B], flat, nnz)
        out = part if out is None else out + part
    return edges, slot, out


def assemble_mixed(points, cells, n_points, local_fns):
    """A matrix over a mesh with several element types: the pattern of every
    type's local pairs together (element_assembler.py:811-830 with all types'
    pairs), and the sum over types, in type order, of each type's locals
    reduced onto it (the projectors of element_assembler.py:832-856 summed
    as __call__ sums them).  ``local_fns[et](points, conn)`` gives a type's
    locals.  Returns (edges int32 [2, nnz], values)."""
    keys = []
    for et, conn in cells.items():
        c = conn.cpu().numpy().astype(np.int64)
        B = c.shape[1]
        keys.append((np.repeat(c[:, :, None], B, 2) * n_points + np.repeat(c[:, None, :], B, 1)).reshape(-1))
    union = np.unique(np.concatenate(keys))
    edges = torch.from_numpy(np.stack([union // n_points, union % n_points]).astype(np.int32))
    out = None
    for (et, conn), k in zip(cells.items(), keys):
        loc = local_fns[et](points, conn)
        slot = torch.from_numpy(np.searchsorted(union, k))
        part = reduce_project(slot, loc.reshape(slot.shape[0], *loc.shape[3:]), union.shape[0])
        out = part if out is None else out + part
    return edges, out


def assemble_load(points, conn, etype, n_points, f_nodes=None, const=None, func=None, qorder=2,
                  chunk=1 << 16):
    """b_i = sum_e sum_q jxw phi_i(q) f(q)  (node_assembler.py:368-409):
    ``f_nodes`` nodal values interpolated with phi (:389), ``const`` a
    constant (builtin.py:730-771), ``func`` a function of the quadrature
    point coordinates (builtin.py:773-813)."""
    _, phi, _ = shape_tables(etype, qorder)
    out = None
    for s, e in _chunks(conn.shape[0], chunk):
        c = conn[s:e]
        _, jxw = shape_grad_jxw(points, c, etype, qorder)
        if f_nodes is not None:
            fq = torch.einsum("eb...,qb->eq...", f_nodes[c], phi)
        elif func is not None:
            xq = torch.einsum("ebd,qb->eqd", points[c], phi)
            fq = func(xq)
        else:
            fq = torch.full(jxw.shape, float(1.0 if const is None else const), dtype=DT)
        integ = phi[None, :, :] * fq[..., None] if fq.dim() == 2 else phi[None, :, :, None] * fq[:, :, None, :]
        loc = torch.einsum("eqb...,eq->eb...", integ, jxw)
        part = reduce_project(c.reshape(-1), loc.reshape(-1, *loc.shape[2:]), n_points)
        out = part if out is None else out + part
    return out


# ---------------------------------------------------------------------------
# Boundary facets (assemble/facet_assembler.py:123-277, 367-515)
# ---------------------------------------------------------------------------
# Gauss-Legendre on [-1, 1] (element/quadrature.py:36-53), mapped to [0, 1]
_GL_W = {1: [2.0], 2: [1.0, 1.0],
         3: [0.55555555555555555556, 0.88888888888888888889, 0.55555555555555555556],
         4: [0.34785484513745385737, 0.65214515486254614263, 0.65214515486254614263, 0.34785484513745385737],
         5: [0.23692688505618908751, 0.47862867049936646804, 0.56888888888888888889, 0.47862867049936646804,
             0.23692688505618908751],
         6: [0.17132449237917034504, 0.36076157304813860757, 0.46791393457269104739, 0.46791393457269104739,
             0.36076157304813860757, 0.17132449237917034504],
         7: [0.12948496616886969327, 0.27970539148927666790, 0.38183005050511894495, 0.41795918367346938776,
             0.38183005050511894495, 0.27970539148927666790, 0.12948496616886969327]}
_GL_P = {1: [0.0], 2: [-0.57735026918962576451, 0.57735026918962576451],
         3: [-0.77459666924148337704, 0.0, 0.77459666924148337704],
         4: [-0.8611363115940526, -0.3399810435848563, 0.3399810435848563, 0.8611363115940526],
         5: [-0.9061798459386640, -0.5384693101056831, 0.0, 0.5384693101056831, 0.9061798459386640],
         6: [-0.9324695142031521, -0.6612093864662645, -0.2386191860831969, 0.2386191860831969,
             0.6612093864662645, 0.9324695142031521],
         7: [-0.9491079123427585, -0.7415311855993945, -0.4058451513773972, 0.0, 0.4058451513773972,
             0.7415311855993945, 0.9491079123427585]}
_FACET_VERTS = {2: [[0, 1], [1, 2], [2, 0]], 3: [[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]]}


def facet_vertices(etype):
    """Vertex lists of the element's facets (quadrilaterals: its edges,
    element.py:1813)."""
    return _QUAD_EDGE if etype in _QUADS else _FACET_VERTS[ELEMENT[etype][0]]


def _facet_rule(dim, qorder):
    """Facet-local weights [Qf] and points [Qf, dim-1]: lines [0, 1]
    (element/quadrature.py:13-66), triangles the element rule."""
    if dim == 2:
        w = torch.tensor(_GL_W[qorder], dtype=DT) / 2
        return w, ((torch.tensor(_GL_P[qorder], dtype=DT) + 1) / 2)[:, None]
    return quadrature("triangle", qorder)


def facet_nodes(etype):
    """Local nodes of each facet: its vertices, then (P2) the element's edge
    nodes whose two ends are both facet vertices."""
    dim, order, _ = ELEMENT[etype]
    edges = _QUAD_EDGE if etype in _QUADS else (_TRI_EDGE if dim == 2 else _TET_EDGE)
    nv = n_vertices(etype)
    out = []
    for vs in facet_vertices(etype):
        nodes = list(vs)
        if order == 2:
            nodes += [nv + k for k, (a, b) in enumerate(edges) if a in vs and b in vs]
        out.append(nodes)
    return out


def assemble_facet_load(points, conn, etype, boundary, n_points, qorder=2, f_nodes=None, const=None, func=None):
    """b_i = sum over the selected (element, facet) pairs of
    sum_q w_q |F_q| g(x_q) phi_i(xi_q), in the element's frame as the
    reference writes it (facet_assembler.py:123-277): a facet of an element
    is selected when all its nodes are boundary nodes (:367-515); xi_q is the
    facet quadrature point mapped into the element's reference coordinates,
    phi the cell basis, |F| = sqrt(det(F^T F)) with F = J G, J the cell
    Jacobian at xi_q and G the facet map's gradient (element.py:1295-1408),
    and every cell node receives its value.  ``f_nodes`` nodal values
    [N] or [N, W] interpolated with phi, ``const`` a scalar or a vector of
    length W, ``func`` a function of x_q."""
    dim, order, nb = ELEMENT[etype]
    conn = conn.long()
    verts = basis_nodes(etype)[:n_vertices(etype)]       # reference vertex coordinates
    exps = element_monomials(etype)
    coef = torch.linalg.inv(_eval_monomials(exps, basis_nodes(etype))).T
    wf, tf = _facet_rule(dim, qorder)
    width = 1
    if f_nodes is not None and f_nodes.dim() == 2:
        width = f_nodes.shape[1]
    if const is not None and torch.as_tensor(const).dim() == 1:
        width = torch.as_tensor(const).numel()
    out = torch.zeros(n_points, width, dtype=DT)
    for k, (vs, fnodes) in enumerate(zip(facet_vertices(etype), facet_nodes(etype))):
        sel = boundary[conn[:, fnodes]].all(1)
        if not bool(sel.any()):
            continue
        c = conn[sel]
        G = torch.stack([verts[vs[j]] - verts[vs[0]] for j in range(1, dim)], 1)   # [dim, dim-1]
        xi = verts[vs[0]][None, :] + tf @ G.T                                        # [Qf, dim]
        phi = _eval_monomials(exps, xi) @ coef.T                                     # [Qf, B]
        dphi = torch.einsum("qdm,bm->qdb", _eval_monomial_grads(exps, xi), coef)    # [Qf, dim, B]
        X = points[c]                                                                # [E, B, dim]
        J = torch.einsum("qib,ebj->eqji", dphi, X)                                   # [E, Qf, dim(x), dim(xi)]
        F = J @ G                                                                    # [E, Qf, dim, dim-1]
        detF = torch.sqrt(torch.linalg.det(F.transpose(-1, -2) @ F))                # [E, Qf]
        if f_nodes is not None:
            fv = f_nodes.reshape(n_points, -1)[c]                                    # [E, B, W]
            g = torch.einsum("ebw,qb->eqw", fv, phi)
        elif func is not None:
            g = func(torch.einsum("ebd,qb->eqd", X, phi)).reshape(c.shape[0], len(wf), -1)
        else:
            cv = torch.as_tensor(1.0 if const is None else const, dtype=DT).reshape(1, 1, -1)
            g = cv.expand(c.shape[0], len(wf), width)
        loc = torch.einsum("q,eq,eqw,qb->ebw", wf, detF, g, phi)
        out.index_add_(0, c.reshape(-1), loc.reshape(-1, width))
    return out[:, 0] if width == 1 and (f_nodes is None or f_nodes.dim() == 1) and \
        (const is None or torch.as_tensor(const).dim() == 0) else out


# ---------------------------------------------------------------------------
# Dirichlet condensation (operator/condense.py:182-296) and a direct solve
# ---------------------------------------------------------------------------
def condense(values, row, col, n, mask, rhs, value=None):
    row = row.long()
    col = col.long()
    inner = ~mask
    ie = inner[row] & inner[col]
    oe = inner[row] & mask[col]
    loc = torch.full((n,), -1, dtype=torch.long)
    loc[inner] = torch.arange(int(inner.sum()))
    loc[mask] = torch.arange(int(mask.sum()))
    ni, no = int(inner.sum()), int(mask.sum())
    Kii = scipy.sparse.coo_matrix((values[ie].numpy(), (loc[row[ie]].numpy(), loc[col[ie]].numpy())),
                                  shape=(ni, ni)).tocsr()
    uo = torch.zeros(no, dtype=DT) if value is None else value
    Kio = scipy.sparse.coo_matrix((values[oe].numpy(), (loc[row[oe]].numpy(), loc[col[oe]].numpy())),
                                  shape=(ni, no)).tocsr()
    rhs_i = rhs[inner].numpy() - Kio @ uo.numpy()
    return Kii, rhs_i, inner


def solve_dirichlet(values, row, col, n, mask, rhs):
    Kii, ri, inner = condense(values, row, col, n, mask, rhs)
    ui = scipy.sparse.linalg.spsolve(Kii.tocsc(), ri)
    u = torch.zeros(n, dtype=DT)
    u[inner] = torch.from_numpy(np.asarray(ui))
    return u


def checksum(values: torch.Tensor) -> Dict[str, float]:
    """Size-independent fingerprints of an assembled value array: the
    Frobenius norm and two positively weighted sums (weights in [0.5,1.5)
    from a multiplicative hash of the flat index, so no cancellation)."""
    v = values.reshape(-1).to(DT)
    i = torch.arange(v.shape[0], dtype=torch.int64)
    w1 = ((i * 2654435761) % 4294967296).to(DT) / 4294967296.0 + 0.5
    w2 = ((i * 40503 + 12345) % 65536).to(DT) / 65536.0 + 0.5
    return {"fro": float(torch.linalg.vector_norm(v)), "w1": float((w1 * v).sum()),
            "w2": float((w2 * v).sum()), "abs": float(v.abs().sum()), "n": int(v.shape[0])}


# ---------------------------------------------------------------------------
# Random sign sketches: a relative-Frobenius comparison with a value array
# that is too large to store.  Sketch k of v is s_k = sum_i r_k[i] v_i with
# Rademacher signs r_k[i] = 1 - 2 * bit k of splitmix64(i) (Vigna's
# SplitMix64 finaliser, computed with wrapping int64 arithmetic in torch, so
# that the signs are the same on every machine and device).  For a
# difference d = a - b, E[(s_k(a) - s_k(b))^2] = ||d||^2 for every k, so
# sqrt(mean_k (s_k(a) - s_k(b))^2) estimates ||a - b||_F from the 64 stored
# numbers of b alone; with 64 sketches the estimate stays within a factor of
# about two of the true norm (chi-square-like with 64 degrees of freedom,
# relative spread ~0.18), and no cancellation can hide an error, unlike
# positively weighted sums.  The sums run in float64 over blocks; their own
# rounding (~1e-16 ||v|| for random signs) is far below the 1e-12 bar.
# ---------------------------------------------------------------------------
N_SKETCH = 64
_U64 = 1 << 64


def _s64(c: int) -> int:
    return c - _U64 if c >= 1 << 63 else c


def _srl(x: torch.Tensor, s: int) -> torch.Tensor:
    """Logical right shift of int64 values (torch shifts arithmetically)."""
    return (x >> s) & ((1 << (64 - s)) - 1)


def splitmix64(i: torch.Tensor) -> torch.Tensor:
    """SplitMix64 output for state increments i (int64, wrapping)."""
    z = i + _s64(0x9E3779B97F4A7C15)
    z = (z ^ _srl(z, 30)) * _s64(0xBF58476D1CE4E5B9)
    z = (z ^ _srl(z, 27)) * _s64(0x94D049BB133111EB)
    return z ^ _srl(z, 31)


def splitmix64_py(i: int) -> int:
    """The same function on Python integers (to check the tensor version)."""
    z = (i + 0x9E3779B97F4A7C15) % _U64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) % _U64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) % _U64
    return z ^ (z >> 31)


def sketch(values: torch.Tensor, n: int = N_SKETCH, block: int = 1 << 18) -> list:
    """The n sign sketches of the flat float64 value array (on its device)."""
    v = values.detach().reshape(-1).to(DT)
    dev = v.device
    ks = torch.arange(n, device=dev, dtype=torch.int64)
    acc = torch.zeros(n, dtype=DT, device=dev)
    for b0 in range(0, v.shape[0], block):
        b1 = min(v.shape[0], b0 + block)
        h = splitmix64(torch.arange(b0, b1, device=dev, dtype=torch.int64))
        signs = 1.0 - 2.0 * ((h[:, None] >> ks[None, :]) & 1).to(DT)
        acc += v[b0:b1] @ signs
    return [float(x) for x in acc.cpu()]


def sketch_rel_error(got: Sequence[float], ref: Sequence[float], ref_fro: float) -> float:
    """Estimated ||a - b||_F / ||b||_F from the sketches of a and b."""
    d = np.asarray(got, dtype=np.float64) - np.asarray(ref, dtype=np.float64)
    return float(np.sqrt(np.mean(d * d)) / ref_fro)


def slot_hash(slot: torch.Tensor) -> str:
    """SHA-256 of a slot map's entries as little-endian int32 bytes."""
    s = slot.detach().reshape(-1).cpu().numpy()
    return hashlib.sha256(s.astype("<i4").tobytes()).hexdigest()


# ---------------------------------------------------------------------------
# The reference's per-call work for the diffusion + mass benchmark, restated
# op for op (element_assembler.py:390-445 with builtin.py:61-62 / :99-100 and
# sparse/matrix.py:76-86), given the slot map of ``from_mesh``.  Used as the
# reference arm of the benchmark, on the host cores and on the GPU.
# ---------------------------------------------------------------------------
def reference_call_diffusion_mass(points, conn, kappa, slot, edges, etype="tetra", qorder=2,
                                  with_hash=True):
    w, phi, dphi = shape_tables(etype, qorder)
    w, phi, dphi = w.to(points.device), phi.to(points.device), dphi.to(points.device)
    nnz = edges.shape[1]
    X = points[conn]
    J = torch.einsum("ebj,qib->eqij", X, dphi)
    grad = torch.einsum("qib,eqji->eqbj", dphi, torch.inverse(J))
    jxw = torch.einsum("q,eq->eq", w, torch.linalg.det(J).abs())
    integ = kappa[:, None, None, None] * torch.einsum("eqid,eqjd->eqij", grad, grad)
    Ke = torch.einsum("eqij,eq->eij", integ, jxw)
    K = torch.zeros(nnz, dtype=points.dtype, device=points.device).index_add_(0, slot, Ke.reshape(-1))
    # mass: the reference recomputes the geometry for every assembler call
    J2 = torch.einsum("ebj,qib->eqij", X, dphi)
    jxw2 = torch.einsum("q,eq->eq", w, torch.linalg.det(J2).abs())
    Me = torch.einsum("qij,eq->eij", phi[:, :, None] * phi[:, None, :], jxw2)
    M = torch.zeros(nnz, dtype=points.dtype, device=points.device).index_add_(0, slot, Me.reshape(-1))
    hashes = []
    if with_hash:
        for _ in range(2):                       # one SparseMatrix per assembled form
            r, c = edges[0], edges[1]
            r.long(), c.long()
            hashes.append(layout_hash(r, c))
    return K, M, hashes


# ---------------------------------------------------------------------------
# The reference's per-call work for the P2-tet elasticity benchmark, restated
# op for op: element_assembler.py:390-445 with the integrand of
# builtin.py:172-178 (Ba^T C Bb per basis pair and quadrature point), the
# quadrature contraction (element_assembler.py:199), the reduce projection
# into [n_edge, D, D] (projector.py:95-123) and SparseMatrix.from_block_coo's
# expansion and layout hash (sparse/matrix.py:76-86, :332-381).  A
# per-element Young's modulus scales C element by element.
# ---------------------------------------------------------------------------
def reference_call_elasticity(points, conn, E, slot, edges, nu=0.3, etype="tetra10", qorder=2,
                              with_hash=True):
    dev = points.device
    w, _, dphi = shape_tables(etype, qorder)
    w, dphi = w.to(dev), dphi.to(dev)
    D = points.shape[1]
    nnz = edges.shape[1]
    X = points[conn]
    J = torch.einsum("ebj,qib->eqij", X, dphi)
    grad = torch.einsum("qib,eqji->eqbj", dphi, torch.inverse(J))
    jxw = torch.einsum("q,eq->eq", w, torch.linalg.det(J).abs())
    Bm = voigt_B(grad)                                               # [e,q,b,k,a]
    C1 = voigt_C(torch.ones(1, dtype=DT), nu, D)[0].to(dev)           # unit-E stiffness
    integ = torch.einsum("eqika,kl,eqjlb->eqijab", Bm, C1, Bm) * E[:, None, None, None, None, None]
    Ke = torch.einsum("eqijab,eq->eijab", integ, jxw)
    K = torch.zeros(nnz, D, D, dtype=points.dtype, device=dev).index_add_(0, slot, Ke.reshape(-1, D, D))
    h = None
    if with_hash:
        i, j = torch.meshgrid(torch.arange(D, device=dev), torch.arange(D, device=dev), indexing="ij")
        r = (edges[0][:, None].repeat(1, D * D) * D + i.flatten()).flatten()
        c = (edges[1][:, None].repeat(1, D * D) * D + j.flatten()).flatten()
        h = layout_hash(r, c)
    return K, h


# ---------------------------------------------------------------------------
# The reference's per-mesh solve path, restated on any device: from_mesh's
# SciPy pattern and slot map (element_assembler.py:811-851), the diffusion
# and load assembly op sequences (element_assembler.py:390-445,
# node_assembler.py:242-409), the Condenser's layout and gathers
# (operator/condense.py:182-296) and the in-tree conjugate gradient cg_py
# (sparse/solve/torch_solve.py:70-127: torch CSR product, one host check of
# sqrt(r.r) < atol per iteration).  The per-mesh baseline of the batched
# benchmark.
# ---------------------------------------------------------------------------
def reference_cg(values, row, col, n, b, atol, max_iter=100000):
    """cg_py: CG on the CSR operator, stopping when ||r|| < atol."""
    A = torch.sparse_coo_tensor(torch.stack([row.long(), col.long()]), values, (n, n)).coalesce()
    A = A.to_sparse_csr()
    x = torch.zeros_like(b)
    r = b - A @ x
    p = r.clone()
    rs_old = torch.dot(r, r)
    it = 0
    for it in range(max_iter):
        Ap = A @ p
        alpha = rs_old / torch.dot(p, Ap)
        x = x + alpha * p
        r = r - alpha * Ap
        rs_new = torch.dot(r, r)
        if torch.sqrt(rs_new) < atol:
            break
        p = r + (rs_new / rs_old) * p
        rs_old = rs_new
    return x, it + 1


def reference_bicgstab(values, row, col, n, b, atol, max_iter=10000):
    """bicgstab_py (sparse/solve/torch_solve.py:130-248), restated: Jacobi
    (right) preconditioning by 1 / diag, a missing or |d| < 1e-12 diagonal
    taken as 1; stop when ||r|| < atol; breakdown when |r0^ . v| < 1e-12;
    x += alpha p^ and stop when ||s|| < atol; omega = 0 when t . t < 1e-12,
    and stop after that update.  Returns (x, iterations)."""
    A = torch.sparse_coo_tensor(torch.stack([row.long(), col.long()]), values, (n, n)).coalesce().to_sparse_csr()
    d = torch.ones(n, dtype=values.dtype, device=values.device)
    diag = row.long() == col.long()
    d[row.long()[diag]] = values[diag]
    d = torch.where(d.abs() < 1e-12, torch.ones_like(d), d)
    minv = 1.0 / d
    x = torch.zeros_like(b)
    r = b - A @ x
    r0 = r.clone()
    rho = torch.dot(r0, r)
    p = r.clone()
    it = 0
    for it in range(max_iter):
        if torch.norm(r) < atol:
            break
        ph = minv * p
        v = A @ ph
        den = torch.dot(r0, v)
        if den.abs() < 1e-12:
            break
        alpha = rho / den
        s = r - alpha * v
        if torch.norm(s) < atol:
            x = x + alpha * ph
            break
        sh = minv * s
        t = A @ sh
        tt = torch.dot(t, t)
        omega = 0.0 if tt.abs() < 1e-12 else torch.dot(t, s) / tt
        x = x + alpha * ph + omega * sh
        r = s - omega * t
        if torch.norm(r) < atol:
            break
        rho_new = torch.dot(r0, r)
        if omega == 0:
            break
        p = r + (rho_new / rho) * (alpha / omega) * (p - omega * v)
        rho = rho_new
    return x, it + 1


def reference_per_mesh_solve(points, conn, boundary, kappa, f, etype="triangle", qorder=2, rel=1e-10):
    """One mesh through the reference's path on the device of ``points``:
    pattern and slot map on the host, K(kappa) and b = int f v assembled by
    the reference's op sequence, the Dirichlet rows condensed (zero boundary
    values), CG to ||r|| < rel ||b_i||.  Returns (u [N], iterations)."""
    dev = points.device
    n = points.shape[0]
    edges, slot = element_pattern(conn, n)
    edges, slot = edges.to(dev), slot.to(dev)
    w, phi, dphi = (t.to(dev) for t in shape_tables(etype, qorder))
    X = points[conn]
    J = torch.einsum("ebj,qib->eqij", X, dphi)
    grad = torch.einsum("qib,eqji->eqbj", dphi, torch.inverse(J))
    jxw = torch.einsum("q,eq->eq", w, torch.linalg.det(J).abs())
    Ke = torch.einsum("eqij,eq->eij", kappa[:, None, None, None] * torch.einsum("eqid,eqjd->eqij", grad, grad), jxw)
    K = torch.zeros(edges.shape[1], dtype=points.dtype, device=dev).index_add_(0, slot, Ke.reshape(-1))
    fq = torch.einsum("eb,qb->eq", f[conn], phi)
    be = torch.einsum("eq,qb,eq->eb", fq, phi, jxw)
    b = torch.zeros(n, dtype=points.dtype, device=dev).index_add_(0, conn.reshape(-1), be.reshape(-1))
    # Condenser: inner/outer masks over the pattern, local numbering
    row, col = edges[0].long(), edges[1].long()
    inner = ~boundary
    ie = inner[row] & inner[col]
    oe = inner[row] & boundary[col]
    loc = torch.full((n,), -1, dtype=torch.long, device=dev)
    ni, no = int(inner.sum()), int(boundary.sum())
    loc[inner] = torch.arange(ni, device=dev)
    loc[boundary] = torch.arange(no, device=dev)
    uo = torch.zeros(no, dtype=points.dtype, device=dev)
    Kio = torch.sparse_coo_tensor(torch.stack([loc[row[oe]], loc[col[oe]]]), K[oe], (ni, no))
    bi = b[inner] - Kio @ uo
    ui, iters = reference_cg(K[ie], loc[row[ie]], loc[col[ie]], ni, bi, rel * float(bi.norm()))
    u = torch.zeros(n, dtype=points.dtype, device=dev)
    u[inner] = ui
    return u, iters
