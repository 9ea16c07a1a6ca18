"""Gradients of load vectors b_a = sum_q w_q |det J_q| phi_a(q) f(q) on every
element type (``LoadAssembly``: the load term of ``tm_adjoint_general`` /
``tm_adjoint_p1`` for dL/dpoints; the load of the nodal source lam for
dL/df), for nodal (scalar and 2-component) and constant (scalar and vector)
sources, against autograd through the oracle's restatement of the
reference's linear-form assembly (node_assembler.py:368-409), within 1e-10
relative."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu

MESHES = {
    "triangle": lambda: tg.gen_unit_square(6, jitter=0.2, seed=71),
    "tetra": lambda: tg.gen_unit_cube(3, jitter=0.2, seed=72),
    "triangle6": lambda: tg.gen_unit_square(3, order=2, jitter=0.1, seed=73),
    "tetra10": lambda: tg.gen_unit_cube(2, order=2, jitter=0.1, seed=74),
    "quad": lambda: tg.gen_unit_square(4, jitter=0.2, seed=75, cell="quad"),
    "quad9": lambda: tg.gen_unit_square(3, order=2, jitter=0.1, seed=76, cell="quad"),
}


@pytest.mark.parametrize("etype", list(MESHES))
@pytest.mark.parametrize("width", [1, 2])
def test_nodal_source_gradients(etype, width, cuda):
    mesh = MESHES[etype]()
    rng = np.random.default_rng(77)
    shape = (mesh.n_points,) if width == 1 else (mesh.n_points, width)
    f0 = torch.from_numpy(rng.uniform(-1.0, 2.0, shape))
    W = torch.from_numpy(rng.uniform(-1.0, 1.0, mesh.n_points * width))
    gm = mesh.to(cuda)
    src = tg.LoadNodeAssembler.from_mesh(gm)
    P = gm.points.clone().requires_grad_(True)
    f = f0.clone().to(cuda).requires_grad_(True)
    b = src(P, point_data={"f": f})
    (b * W.to(cuda)).sum().backward()
    Po = mesh.points.clone().requires_grad_(True)
    fo = f0.clone().requires_grad_(True)
    bo = O.assemble_load(Po, mesh.elements().long(), etype, mesh.n_points, f_nodes=fo).reshape(-1)
    assert rel_fro(b.detach().cpu(), bo.detach()) <= 1e-12
    (bo * W).sum().backward()
    assert rel_fro(P.grad.cpu(), Po.grad) <= 1e-10
    assert rel_fro(f.grad.cpu(), fo.grad) <= 1e-10


@pytest.mark.parametrize("etype", list(MESHES))
@pytest.mark.parametrize("vector", [False, True])
def test_constant_source_gradients(etype, vector, cuda):
    mesh = MESHES[etype]()
    rng = np.random.default_rng(78)
    c0 = torch.tensor([0.7, -1.3], dtype=torch.float64) if vector else torch.tensor(1.9, dtype=torch.float64)
    width = 2 if vector else 1
    W = torch.from_numpy(rng.uniform(-1.0, 1.0, mesh.n_points * width))
    gm = mesh.to(cuda)
    c = c0.clone().requires_grad_(True)
    src = tg.const_node_assembler(c).from_mesh(gm)
    P = gm.points.clone().requires_grad_(True)
    b = src(P)
    (b * W.to(cuda)).sum().backward()
    Po = mesh.points.clone().requires_grad_(True)
    co = c0.clone().requires_grad_(True)
    b1 = O.assemble_load(Po, mesh.elements().long(), etype, mesh.n_points, const=1.0)     # [N]
    bo = (b1[:, None] * co.reshape(1, -1)).reshape(-1)
    assert rel_fro(b.detach().cpu(), bo.detach()) <= 1e-12
    (bo * W).sum().backward()
    assert rel_fro(P.grad.cpu(), Po.grad) <= 1e-10
    assert rel_fro(c.grad, co.grad) <= 1e-10


def test_source_gradient_alone(cuda):
    """Only the nodal source requires grad (fixed coordinates)."""
    mesh = MESHES["quad9"]()
    gm = mesh.to(cuda)
    rng = np.random.default_rng(79)
    f0 = torch.from_numpy(rng.uniform(0.0, 1.0, mesh.n_points))
    f = f0.clone().to(cuda).requires_grad_(True)
    b = tg.LoadNodeAssembler.from_mesh(gm)(gm.points, point_data={"f": f})
    (b ** 2).sum().backward()
    fo = f0.clone().requires_grad_(True)
    bo = O.assemble_load(mesh.points, mesh.elements().long(), "quad9", mesh.n_points, f_nodes=fo)
    (bo ** 2).sum().backward()
    assert rel_fro(f.grad.cpu(), fo.grad) <= 1e-10


@pytest.mark.parametrize("etype", ["triangle", "tetra", "triangle6", "quad9"])
def test_function_source_gradients(etype, cuda):
    """A source given as a function of the quadrature-point coordinates and
    of a nodal field and a captured tensor: dL/dpoints (through x_q and the
    measure), dL/dnodal field and dL/dcaptured, against the oracle's
    restatement under autograd."""
    mesh = MESHES[etype]()
    rng = np.random.default_rng(86)
    a0 = torch.tensor(1.3, dtype=torch.float64)
    h0 = torch.from_numpy(rng.uniform(0.5, 1.5, mesh.n_points))
    W = torch.from_numpy(rng.uniform(-1.0, 1.0, mesh.n_points))
    gm = mesh.to(cuda)
    a = a0.clone().to(cuda).requires_grad_(True)

    class Src(tg.NodeAssembler):
        def forward(self, x, v, h):
            return a * torch.sin(3.0 * x[..., 0]) * (1.0 + x[..., 1] ** 2) * h * v

    P = gm.points.clone().requires_grad_(True)
    h = h0.clone().to(cuda).requires_grad_(True)
    b = Src.from_mesh(gm)(P, point_data={"h": h})
    (b * W.to(cuda)).sum().backward()

    Po = mesh.points.clone().requires_grad_(True)
    ao = a0.clone().requires_grad_(True)
    ho = h0.clone().requires_grad_(True)
    conn = mesh.elements().long()
    # the oracle integrates func(x_q) * v; the nodal field enters as h(x_q)
    _, phi, _ = O.shape_tables(etype, 2)
    hq = torch.einsum("eb,qb->eq", ho[conn], phi)
    xq = torch.einsum("ebd,qb->eqd", Po[conn], phi)
    fq = ao * torch.sin(3.0 * xq[..., 0]) * (1.0 + xq[..., 1] ** 2) * hq
    _, jxw = O.shape_grad_jxw(Po, conn, etype, 2)
    loc = torch.einsum("qb,eq,eq->eb", phi, fq, jxw)
    bo = O.reduce_project(conn.reshape(-1), loc.reshape(-1), mesh.n_points)
    assert rel_fro(b.detach().cpu(), bo.detach()) <= 1e-12
    (bo * W).sum().backward()
    assert rel_fro(P.grad.cpu(), Po.grad) <= 1e-10
    assert rel_fro(h.grad.cpu(), ho.grad) <= 1e-10
    assert abs(float(a.grad) - float(ao.grad)) <= 1e-10 * abs(float(ao.grad))
