"""Mesh container and structured mesh generators.

The assemblers only need what the reference's ``Mesh`` exposes on the
assembly path (``tensormesh/mesh/mesh.py``): ``points`` (:86-145),
``elements()`` (:403-486), ``default_element_type`` (:654), ``n_points``
(:601), ``dtype`` / ``device`` (:671-692) and ``boundary_mask`` (:633).
Any object with those members (including the reference's own ``Mesh``)
can be handed to ``ElementAssembler.from_mesh`` / ``NodeAssembler.from_mesh``.

The reference builds its meshes with gmsh, which this project does not
use; the generators below produce the structured meshes the benchmark
workloads are defined on:

* ``gen_unit_square(n)``: an (n+1)x(n+1) grid on [0,1]^2, every cell split
  into two triangles along its (0,0)-(1,1) diagonal, or kept as one
  quadrilateral (``cell="quad"``).
* ``gen_unit_cube(n)``: an (n+1)^3 grid on [0,1]^3, every cube split into
  six tetrahedra that share the cube's main diagonal (Kuhn split).
* ``order=2`` adds the edge mid-points in the reference's node order:
  vertices first, then one node per edge in the order of
  ``Triangle.edge`` = [[1,2],[0,2],[0,1]] (``element/element.py:1684``) and
  ``Tetrahedron.edge`` = [[2,3],[1,3],[1,2],[0,3],[0,2],[0,1]]
  (``element/element.py:1949``). Mid-points are numbered on the grid of
  half the spacing, so a P2 mesh on n cells per side has the node set of
  a P1 grid on 2n cells per side.

Random perturbations use ``numpy.random.default_rng(seed)`` so that the same
seed gives the same mesh on every platform.
"""
from typing import Dict, Optional, Union

import numpy as np
import torch

# vertex offsets of the unit cube, v0..v7 = 000,100,110,010,001,101,111,011
_CUBE_VERTS = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                        [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=np.int64)
# six tetrahedra around the 0-6 diagonal
_KUHN_TETS = np.array([[0, 1, 2, 6], [0, 2, 3, 6], [0, 3, 7, 6],
                       [0, 7, 4, 6], [0, 4, 5, 6], [0, 5, 1, 6]], dtype=np.int64)
_TRI_EDGES = np.array([[1, 2], [0, 2], [0, 1]], dtype=np.int64)
_QUAD_EDGES = ((0, 1), (0, 2), (1, 3), (2, 3))
_TET_EDGES = np.array([[2, 3], [1, 3], [1, 2], [0, 3], [0, 2], [0, 1]], dtype=np.int64)

ELEMENT_DIM = {"triangle": 2, "triangle6": 2, "tetra": 3, "tetra10": 3, "quad": 2, "quad9": 2}


class Mesh:
    """Nodes, per-type connectivity and nodal fields of an unstructured mesh.

    Parameters
    ----------
    points : torch.Tensor
        ``[N, D]`` node coordinates.
    cells : dict
        ``{element_type: LongTensor[E, B]}``; element types are the
        reference's strings ``"triangle"``, ``"triangle6"``, ``"tetra"``,
        ``"tetra10"``, ``"quad"``, ``"quad9"``.
    point_data : dict, optional
        Nodal fields; ``"is_boundary"`` is what ``boundary_mask`` returns.
    element_groups : array of int, optional
        ``[G+1]`` element offsets of independent groups (several meshes
        concatenated into one): the assemblers order elements by Morton code
        within each group and keep the groups in sequence, so that a chunk
        of elements stays within one group even where the groups overlap in
        space.
    """

    def __init__(self, points: torch.Tensor, cells: Dict[str, torch.Tensor],
                 point_data: Optional[Dict[str, torch.Tensor]] = None, element_groups=None):
        self.points = points
        self.cells = {k: v.long() for k, v in cells.items()}
        self.point_data = dict(point_data or {})
        self.element_groups = None if element_groups is None else np.asarray(element_groups, dtype=np.int64)
        dims = {k: ELEMENT_DIM[k] for k in self.cells}
        top = max(dims.values())
        types = [k for k, d in dims.items() if d == top]
        self.default_eletyp = types[0] if len(types) == 1 else types

    # -- members used by the assemblers -------------------------------------
    @property
    def default_element_type(self):
        return self.default_eletyp

    def elements(self, element_type: Optional[Union[str, int]] = None):
        if element_type == "all":
            return dict(self.cells)
        if element_type is None:
            if isinstance(self.default_eletyp, str):
                return self.cells[self.default_eletyp]
            return {k: self.cells[k] for k in self.default_eletyp}
        if isinstance(element_type, str):
            return self.cells[element_type]
        return {k: self.cells[k] for k in element_type}

    @property
    def n_points(self) -> int:
        return int(self.points.shape[0])

    @property
    def n_elements(self) -> int:
        if isinstance(self.default_eletyp, str):
            return int(self.cells[self.default_eletyp].shape[0])
        return sum(int(self.cells[k].shape[0]) for k in self.default_eletyp)

    @property
    def dim(self) -> int:
        return int(self.points.shape[1])

    @property
    def dtype(self) -> torch.dtype:
        return self.points.dtype

    @property
    def device(self) -> torch.device:
        return self.points.device

    @property
    def boundary_mask(self) -> torch.Tensor:
        if "is_boundary" in self.point_data:
            return self.point_data["is_boundary"]
        if "boundary_mask" in self.point_data:
            return self.point_data["boundary_mask"]
        raise KeyError("'boundary_mask' or 'is_boundary' is not found in point_data")

    def to(self, device=None, dtype=None) -> "Mesh":
        pts = self.points.to(device=device) if device is not None else self.points
        if dtype is not None:
            pts = pts.to(dtype)
        cells = {k: v.to(device) if device is not None else v for k, v in self.cells.items()}
        pd = {k: v.to(device) if device is not None else v for k, v in self.point_data.items()}
        return Mesh(pts, cells, pd, self.element_groups)

    def __repr__(self):
        sizes = ", ".join(f"{k}:{tuple(v.shape)}" for k, v in self.cells.items())
        return f"Mesh(n_points={self.n_points}, dim={self.dim}, cells=[{sizes}])"


def _grid_points(m: int, dim: int) -> np.ndarray:
    """Points of an (m+1)^dim grid on the unit box, x fastest."""
    t = np.arange(m + 1, dtype=np.float64) / m
    if dim == 2:
        y, x = np.meshgrid(t, t, indexing="ij")
        return np.stack([x.ravel(), y.ravel()], axis=1)
    z, y, x = np.meshgrid(t, t, t, indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)


def _boundary(points: np.ndarray) -> np.ndarray:
    """Boundary nodes by exact coordinate equality with the box faces."""
    return np.any((points == 0.0) | (points == 1.0), axis=1)


def _jitter(points: np.ndarray, boundary: np.ndarray, amount: float, h: float,
            seed: int) -> np.ndarray:
    if amount <= 0:
        return points
    rng = np.random.default_rng(seed)
    d = rng.uniform(-amount * h, amount * h, size=points.shape)
    d[boundary] = 0.0
    return points + d


def gen_unit_square(n: int, order: int = 1, jitter: float = 0.0, seed: int = 0,
                    dtype: torch.dtype = torch.float64, device="cpu", cell: str = "triangle") -> Mesh:
    """Unit square with ``n`` cells per side, triangulated (``cell=
    "triangle"``) or as quadrilaterals (``cell="quad"``).

    Cell (i, j) with corners a=(i,j), b=(i+1,j), c=(i+1,j+1), d=(i,j+1)
    becomes the triangles (a,b,c) and (a,c,d), or the quadrilateral
    (a,b,d,c) in the reference's lexicographic vertex order (for ``order=2``
    followed by the mid-points of its edges [[0,1],[0,2],[1,3],[2,3]] and
    its centre: types ``"quad"`` / ``"quad9"``).  ``jitter`` moves interior
    nodes by U(-jitter*h, jitter*h) per coordinate (h = 1/(order*n)).
    """
    s = order                      # node grid has s*n cells per side
    m = s * n
    pts = _grid_points(m, 2)
    idx = lambda i, j: j * (m + 1) + i
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    i, j = i.ravel() * s, j.ravel() * s
    if cell == "quad":
        h = s // 2
        corners = [(i, j), (i + s, j), (i, j + s), (i + s, j + s)]
        conn = [idx(x, y) for x, y in corners]
        etype = "quad"
        if order == 2:
            for (p, q) in _QUAD_EDGES:
                conn.append(idx((corners[p][0] + corners[q][0]) // 2, (corners[p][1] + corners[q][1]) // 2))
            conn.append(idx(i + h, j + h))
            etype = "quad9"
        conn = np.stack(conn, axis=1)
        bnd = _boundary(pts)
        pts = _jitter(pts, bnd, jitter, 1.0 / m, seed)
        return Mesh(torch.tensor(pts, dtype=dtype, device=device),
                    {etype: torch.from_numpy(conn).to(device)},
                    {"is_boundary": torch.from_numpy(bnd).to(device)})
    if cell != "triangle":
        raise ValueError(f"cell must be 'triangle' or 'quad', got {cell!r}")
    a, b, c, d = (np.array([i, j]), np.array([i + s, j]),
                  np.array([i + s, j + s]), np.array([i, j + s]))
    tris = []
    for t in ((a, b, c), (a, c, d)):
        tris.append(np.stack(t, axis=0))           # [3 verts, 2 coords, ncell]
    verts = np.stack(tris, axis=1)                  # [3, 2 tri, 2, ncell]
    verts = verts.transpose(3, 1, 0, 2).reshape(-1, 3, 2)   # [ncell*2, 3, 2] cell-major
    conn = [idx(verts[:, k, 0], verts[:, k, 1]) for k in range(3)]
    etype = "triangle"
    if order == 2:
        for (p, q) in _TRI_EDGES:
            mid = (verts[:, p, :] + verts[:, q, :]) // 2
            conn.append(idx(mid[:, 0], mid[:, 1]))
        etype = "triangle6"
    conn = np.stack(conn, axis=1)
    bnd = _boundary(pts)
    pts = _jitter(pts, bnd, jitter, 1.0 / m, seed)
    return Mesh(torch.tensor(pts, dtype=dtype, device=device),
                {etype: torch.from_numpy(conn).to(device)},
                {"is_boundary": torch.from_numpy(bnd).to(device)})


def gen_unit_square_mixed(n: int, jitter: float = 0.0, seed: int = 0, dtype: torch.dtype = torch.float64,
                          device="cpu") -> Mesh:
    """Unit square with ``n`` cells per side and two element types: cells
    whose left edge lies in the left half are quadrilaterals (``"quad"``),
    the others are split into the triangles (a,b,c), (a,c,d) of
    ``gen_unit_square`` (``"triangle"``).  The quadrilaterals are listed
    first.  Same nodes, jitter and boundary flags as ``gen_unit_square``."""
    q = gen_unit_square(n, jitter=jitter, seed=seed, dtype=dtype, cell="quad")
    t = gen_unit_square(n, jitter=jitter, seed=seed, dtype=dtype, cell="triangle")
    i = np.tile(np.arange(n), n)                   # cell column, cells x fastest in both generators
    left = i < (n + 1) // 2
    quads = q.cells["quad"].numpy()[left]
    tris = t.cells["triangle"].numpy().reshape(n * n, 2, 3)[~left].reshape(-1, 3)
    return Mesh(q.points.to(device), {"quad": torch.from_numpy(quads).to(device),
                                      "triangle": torch.from_numpy(tris).to(device)},
                {"is_boundary": q.point_data["is_boundary"].to(device)})


def gen_unit_cube(n: int, order: int = 1, jitter: float = 0.0, seed: int = 0,
                  dtype: torch.dtype = torch.float64, device="cpu") -> Mesh:
    """Kuhn-split unit cube with ``n`` cubes per side (6 tetrahedra per cube).

    Cubes are visited x fastest, then y, then z; each contributes the six
    tetrahedra (0,1,2,6), (0,2,3,6), (0,3,7,6), (0,7,4,6), (0,4,5,6),
    (0,5,1,6) over its vertices v0..v7 = 000,100,110,010,001,101,111,011.
    """
    s = order
    m = s * n
    pts = _grid_points(m, 3)
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1) * s      # [ncube, 3]
    corners = base[:, None, :] + s * _CUBE_VERTS[None, :, :]              # [ncube, 8, 3]
    verts = corners[:, _KUHN_TETS, :].reshape(-1, 4, 3)                   # [ncube*6, 4, 3]
    idx = lambda g: (g[..., 2] * (m + 1) + g[..., 1]) * (m + 1) + g[..., 0]
    conn = [idx(verts[:, v, :]) for v in range(4)]
    etype = "tetra"
    if order == 2:
        for (p, q) in _TET_EDGES:
            conn.append(idx((verts[:, p, :] + verts[:, q, :]) // 2))
        etype = "tetra10"
    conn = np.stack(conn, axis=1)
    bnd = _boundary(pts)
    pts = _jitter(pts, bnd, jitter, 1.0 / m, seed)
    return Mesh(torch.tensor(pts, dtype=dtype, device=device),
                {etype: torch.from_numpy(conn).to(device)},
                {"is_boundary": torch.from_numpy(bnd).to(device)})
