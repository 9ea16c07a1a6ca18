"""Boundary-facet loads on the GPU (tm_assemble_facet_vector through the
FacetAssembler built-ins) against the oracle's restatement (1e-12 relative)
and the reference's outputs (golden fixtures, 1e-6 relative: the reference
evaluates its facet quadrature rule in float32; 1e-14 for order-1
triangle edges), on all six element types, scalar and vector loads;
multi-chunk determinism and float32."""
import math

import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import load_golden, rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu
ET = {"tri3": "triangle", "tri6": "triangle6", "tet4": "tetra", "tet10": "tetra10", "quad": "quad",
      "quad9": "quad9"}
FIXTURE = {name: ("facet_quad" if name.startswith("quad") else "facet") for name in ET}


def _func(x):
    return torch.sin(math.pi * x[..., 0]) * (1 + x[..., 1])


@pytest.mark.parametrize("name", list(ET))
def test_facet_loads_match_oracle_and_reference(name, cuda):
    g = load_golden(FIXTURE[name])
    et = ET[name]
    P = torch.from_numpy(g[f"{name}_points"])
    Cn = torch.from_numpy(g[f"{name}_conn"])
    B = torch.from_numpy(g[f"{name}_boundary"])
    N = P.shape[0]
    mesh = tg.Mesh(P, {et: Cn}, {"is_boundary": B}).to(cuda)
    f = torch.from_numpy(g[f"{name}_f"])
    t = torch.from_numpy(g[f"{name}_traction"])
    for qo in g[f"{name}_qorders"]:
        qo = int(qo)
        tol_ref = 1e-14 if (name == "tri3" and qo == 1) else 1e-6
        ours = {
            "unit": tg.const_facet_assembler(1.0).from_mesh(mesh, quadrature_order=qo)(mesh.points),
            "nodal": tg.LoadFacetAssembler.from_mesh(mesh, quadrature_order=qo)(
                mesh.points, point_data={"f": f.to(cuda)}),
            "func": tg.func_facet_assembler(_func).from_mesh(mesh, quadrature_order=qo)(mesh.points),
            "traction": tg.const_facet_assembler(t).from_mesh(mesh, quadrature_order=qo)(mesh.points),
        }
        oracle = {
            "unit": O.assemble_facet_load(P, Cn, et, B, N, qo),
            "nodal": O.assemble_facet_load(P, Cn, et, B, N, qo, f_nodes=f),
            "func": O.assemble_facet_load(P, Cn, et, B, N, qo, func=_func),
            "traction": O.assemble_facet_load(P, Cn, et, B, N, qo, const=t).reshape(-1),
        }
        for key in ours:
            assert ours[key].shape == oracle[key].shape, key
            assert rel_fro(ours[key], oracle[key]) <= 1e-12, (name, qo, key)
            ref = torch.from_numpy(g[f"{name}_q{qo}_{key}"])
            assert rel_fro(ours[key], ref) <= tol_ref, (name, qo, key)


def test_facet_multichunk_deterministic_and_float32(cuda):
    mesh = tg.gen_unit_cube(20, jitter=0.2, seed=121)
    dm = mesh.to(cuda)
    fa = tg.LoadFacetAssembler.from_mesh(dm)
    assert fa.n_items > 4 * 256                       # several chunks, shared nodes
    fv = torch.from_numpy(np.random.default_rng(122).uniform(-1, 1, (mesh.n_points, 3)))
    b1 = fa(dm.points, point_data={"f": fv.to(cuda)})
    b2 = fa(dm.points, point_data={"f": fv.to(cuda)})
    assert torch.equal(b1, b2)
    ref = O.assemble_facet_load(mesh.points, mesh.elements(), "tetra", mesh.boundary_mask, mesh.n_points, 2,
                                f_nodes=fv).reshape(-1)
    assert rel_fro(b1, ref) <= 1e-12
    m32 = dm.to(dtype=torch.float32)
    b32 = tg.LoadFacetAssembler.from_mesh(m32)(m32.points, point_data={"f": fv.float().to(cuda)})
    assert b32.dtype == torch.float32
    assert rel_fro(b32.double(), ref) <= 1e-5
    with pytest.raises(NotImplementedError):
        tg.FacetAssembler.from_mesh(dm)(dm.points)


FGRAD_MESHES = {
    "triangle": lambda: tg.gen_unit_square(5, jitter=0.2, seed=131),
    "triangle6": lambda: tg.gen_unit_square(3, order=2, jitter=0.1, seed=132),
    "quad9": lambda: tg.gen_unit_square(3, order=2, jitter=0.1, seed=133, cell="quad"),
    "tetra": lambda: tg.gen_unit_cube(3, jitter=0.2, seed=134),
    "tetra10": lambda: tg.gen_unit_cube(2, order=2, jitter=0.1, seed=135),
}


@pytest.mark.parametrize("etype", list(FGRAD_MESHES))
@pytest.mark.parametrize("kind", ["const", "nodal", "func"])
def test_facet_load_gradients(etype, kind, cuda):
    """dL/dpoints (through the facet measure, tm_facet_adjoint, and for a
    function source through x_q) and dL/dsource of L = w . b_facet, against
    the oracle's facet load under autograd (1e-10)."""
    mesh = FGRAD_MESHES[etype]()
    gm = mesh.to(cuda)
    rng = np.random.default_rng(136)
    N = mesh.n_points
    c0 = torch.tensor([0.7, -1.1], dtype=torch.float64)
    f0 = torch.from_numpy(rng.uniform(-1.0, 1.0, N))
    a0 = torch.tensor(1.4, dtype=torch.float64)
    width = 2 if kind == "const" else 1
    W = torch.from_numpy(rng.uniform(-1.0, 1.0, N * width))
    P = gm.points.clone().requires_grad_(True)
    if kind == "const":
        c = c0.clone().requires_grad_(True)
        b = tg.const_facet_assembler(c).from_mesh(gm)(P)
        src = c
    elif kind == "nodal":
        f = f0.clone().to(cuda).requires_grad_(True)
        b = tg.LoadFacetAssembler.from_mesh(gm)(P, point_data={"f": f})
        src = f
    else:
        a = a0.clone().to(cuda).requires_grad_(True)
        b = tg.func_facet_assembler(lambda x: a * torch.sin(2.0 * x[..., 0]) * (1 + x[..., 1] ** 2)).from_mesh(gm)(P)
        src = a
    (b * W.to(cuda)).sum().backward()

    Po = mesh.points.clone().requires_grad_(True)
    conn = mesh.elements()
    if kind == "const":
        so = c0.clone().requires_grad_(True)
        bo = O.assemble_facet_load(Po, conn, etype, mesh.boundary_mask, N, 2, const=so).reshape(-1)
    elif kind == "nodal":
        so = f0.clone().requires_grad_(True)
        bo = O.assemble_facet_load(Po, conn, etype, mesh.boundary_mask, N, 2, f_nodes=so)
    else:
        so = a0.clone().requires_grad_(True)
        bo = O.assemble_facet_load(Po, conn, etype, mesh.boundary_mask, N, 2,
                                   func=lambda x: so * torch.sin(2.0 * x[..., 0]) * (1 + x[..., 1] ** 2))
    assert rel_fro(b.detach().cpu(), bo.detach()) <= 1e-12
    (bo * W).sum().backward()
    assert rel_fro(P.grad.cpu(), Po.grad) <= 1e-10
    assert rel_fro(src.grad.detach().cpu().reshape(-1), so.grad.reshape(-1)) <= 1e-10
