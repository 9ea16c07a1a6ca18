"""Reference-element tables of the product (closed-form shape functions,
quadrature) against the oracle's Vandermonde construction and the
reference's own known answers."""
import numpy as np
import pytest
import torch

from tensormesh_gb300.element import ELEMENTS, element_tables, quadrature, shape_functions, packed_tables
from oracle import fem_oracle as O


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_quadrature_weights_sum_to_reference_measure(order):
    # tests/quadrature/test_tri.py:18-25, test_tetra.py:17-21
    assert abs(quadrature("triangle", order)[0].sum() - 0.5) < 1e-6
    assert abs(quadrature("tetra", order)[0].sum() - 1.0 / 6.0) < 1e-6


@pytest.mark.parametrize("etype", list(ELEMENTS))
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_shape_tables_match_vandermonde_construction(etype, order):
    t = element_tables(etype, order)
    w, phi, dphi = O.shape_tables(etype, order)
    np.testing.assert_allclose(t["w"], w.numpy(), rtol=0, atol=0)
    np.testing.assert_allclose(t["phi"], phi.numpy(), rtol=0, atol=5e-15)
    np.testing.assert_allclose(t["dphi"], dphi.numpy(), rtol=0, atol=5e-14)
    np.testing.assert_allclose(t["phi"].sum(1), 1.0, atol=1e-14)      # partition of unity
    np.testing.assert_allclose(t["dphi"].sum(2), 0.0, atol=1e-13)


@pytest.mark.parametrize("etype", list(ELEMENTS))
def test_kronecker_property_at_nodes(etype):
    nodes = O.basis_nodes(etype).numpy()
    phi, _ = shape_functions(etype, nodes)
    np.testing.assert_allclose(phi, np.eye(len(nodes)), atol=1e-15)


def test_p2_triangle_closed_form():
    # tests/element/test_transformation.py:66-98: internal order, nodes 3,4,5 on edges (1,2),(0,2),(0,1)
    xi = np.array([[0.2, 0.3], [0.1, 0.7]])
    phi, _ = shape_functions("triangle6", xi)
    x, y = xi[:, 0], xi[:, 1]
    l0 = 1 - x - y
    ref = np.stack([l0 * (2 * l0 - 1), x * (2 * x - 1), y * (2 * y - 1), 4 * x * y, 4 * l0 * y, 4 * l0 * x], 1)
    np.testing.assert_allclose(phi, ref, atol=1e-15)


def test_voigt_pins():
    # tests/functional/test_elasticity.py:19-60
    g = torch.tensor([[1., 2., 3.]], dtype=torch.float64)
    B = O.voigt_B(g)[0]
    expected = torch.tensor([[1., 0., 0.], [0., 2., 0.], [0., 0., 3.], [0., 3., 2.], [3., 0., 1.], [2., 1., 0.]],
                            dtype=torch.float64)
    assert torch.equal(B, expected)
    C = O.voigt_C(torch.tensor([70.0], dtype=torch.float64), 0.3, 3)[0]
    mu, lam = 70 / (2 * 1.3), 70 * 0.3 / (1.3 * 0.4)
    assert abs(C[0, 0] - (lam + 2 * mu)) < 1e-12 and abs(C[0, 1] - lam) < 1e-12 and abs(C[3, 3] - mu) < 1e-12


def test_packed_layout():
    t = element_tables("tetra10", 3)
    p = packed_tables("tetra10", 3)
    Q, B, D = 5, 10, 3
    assert p.shape[0] == Q + Q * B + Q * D * B + B * B + B + 1
    np.testing.assert_array_equal(p[Q:Q + Q * B], t["phi"].ravel())
    assert p[-1] == t["w"].sum()
