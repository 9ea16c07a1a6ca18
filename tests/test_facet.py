"""Boundary-facet loads on CPU: the oracle's restatement of the reference's
FacetAssembler against the reference's own outputs (golden fixtures; the
reference evaluates its facet quadrature rule in float32, so the bound is
1e-6 relative, and 1e-14 for order-1 triangle edges, whose rule float32
holds exactly; its quadrilateral edge maps round in float32 even there),
and the facet selection of the package against the oracle's."""
import math

import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import fem_oracle as O
from tensormesh_gb300.element import facet_info, facet_tables
from tensormesh_gb300.facet import FacetAssembler

ET = {"tri3": "triangle", "tri6": "triangle6", "tet4": "tetra", "tet10": "tetra10", "quad": "quad",
      "quad9": "quad9"}
# the quadrilateral cases live in their own fixture file
FIXTURE = {name: ("facet_quad" if name.startswith("quad") else "facet") for name in ET}


def _func(x):
    return torch.sin(math.pi * x[..., 0]) * (1 + x[..., 1])


@pytest.mark.parametrize("name", list(ET))
def test_oracle_matches_reference_facets(name):
    g = load_golden(FIXTURE[name])
    et = ET[name]
    P = torch.from_numpy(g[f"{name}_points"])
    Cn = torch.from_numpy(g[f"{name}_conn"])
    B = torch.from_numpy(g[f"{name}_boundary"])
    N = P.shape[0]
    for qo in g[f"{name}_qorders"]:
        qo = int(qo)
        tol = 1e-14 if (name == "tri3" and qo == 1) else 1e-6
        got = {
            "unit": O.assemble_facet_load(P, Cn, et, B, N, qo),
            "nodal": O.assemble_facet_load(P, Cn, et, B, N, qo, f_nodes=torch.from_numpy(g[f"{name}_f"])),
            "func": O.assemble_facet_load(P, Cn, et, B, N, qo, func=_func),
            "traction": O.assemble_facet_load(P, Cn, et, B, N, qo,
                                              const=torch.from_numpy(g[f"{name}_traction"])).reshape(-1),
        }
        for key, val in got.items():
            ref = g[f"{name}_q{qo}_{key}"]
            assert np.linalg.norm(val.numpy() - ref) <= tol * np.linalg.norm(ref), (name, qo, key)


@pytest.mark.parametrize("name", list(ET))
def test_selection_matches_oracle(name):
    g = load_golden(FIXTURE[name])
    et = ET[name]
    conn = g[f"{name}_conn"].astype(np.int64)
    bnd = g[f"{name}_boundary"].astype(bool)
    items = FacetAssembler._select(conn, bnd, et)
    expect = []
    for nodes in O.facet_nodes(et):
        sel = bnd[conn[:, nodes]].all(1)
        expect += [tuple(sorted(r)) for r in conn[sel][:, nodes]]
    assert sorted(tuple(sorted(r)) for r in items) == sorted(expect)
    assert items.shape[1] == facet_info(et).n_basis


@pytest.mark.parametrize("et", list(ET.values()))
@pytest.mark.parametrize("qo", [1, 2, 3, 4])
def test_facet_tables_integrate_exactly(et, qo):
    """psi sums to 1 and the rule integrates the facet monomials of its
    degree exactly on the reference facet."""
    t = facet_tables(et, qo)
    np.testing.assert_allclose(t["psi"].sum(1), 1.0, atol=1e-14)
    np.testing.assert_allclose(t["dpsi"].sum(2), 0.0, atol=1e-13)
    if facet_info(et).facet_dim == 1:
        for k in range(2 * qo):
            assert abs((t["w"] * t["t"][:, 0] ** k).sum() - 1.0 / (k + 1)) < 1e-14
    else:
        assert abs(t["w"].sum() - 0.5) < 1e-14
