"""Quadrilateral meshes of gen_unit_square(cell="quad"): their node order is
the reference's lexicographic one (element/element.py:1801-1816), checked
through the geometry itself, which a wrong order would twist: every
quadrature point has a positive Jacobian determinant, the mass matrix
integrates 1 to the area of the unit square, and the stiffness matrix
passes the patch test (interior rows annihilate linear fields) -- on
straight and on jittered (Q2: curved) meshes, with the oracle."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from oracle import fem_oracle as O


@pytest.mark.parametrize("order,n,jitter", [(1, 5, 0.0), (1, 6, 0.2), (2, 3, 0.0), (2, 4, 0.1)])
def test_quad_geometry_area_and_patch(order, n, jitter):
    mesh = tg.gen_unit_square(n, order=order, jitter=jitter, seed=131, cell="quad")
    et = mesh.default_element_type
    assert et == ("quad" if order == 1 else "quad9")
    pts, conn = mesh.points, mesh.elements()
    # lexicographic corners: (x0,y0) (x1,y0) (x0,y1) (x1,y1) on straight meshes
    if jitter == 0.0:
        c = pts[conn[:, :4]]
        assert torch.all(c[:, 0, 1] == c[:, 1, 1]) and torch.all(c[:, 2, 1] == c[:, 3, 1])
        assert torch.all(c[:, 0, 0] == c[:, 2, 0]) and torch.all(c[:, 1, 0] == c[:, 3, 0])
        assert torch.all(c[:, 1, 0] > c[:, 0, 0]) and torch.all(c[:, 2, 1] > c[:, 0, 1])
    w, phi, dphi = O.shape_tables(et, 3)
    X = pts[conn]
    J = torch.einsum("ebj,qib->eqij", X, dphi)
    assert bool((torch.linalg.det(J) > 0).all()), "a quadrilateral is twisted or inverted"
    _, _, M = O.assemble_matrix(pts, conn, mesh.n_points, lambda p, c: O.element_locals_mass(p, c, et, 3))
    assert abs(float(M.sum()) - 1.0) <= 1e-12
    edges, _, K = O.assemble_matrix(pts, conn, mesh.n_points,
                                    lambda p, c: O.element_locals_diffusion(p, c, et, None, 3))
    Kd = torch.zeros(mesh.n_points, mesh.n_points, dtype=torch.float64)
    Kd.index_put_((edges[0].long(), edges[1].long()), K, accumulate=True)
    u = pts[:, 0] + 2.0 * pts[:, 1]
    r = Kd @ u
    interior = ~mesh.boundary_mask
    assert float(r[interior].abs().max()) <= 1e-11 * float(Kd.abs().max())
