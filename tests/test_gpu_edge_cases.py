"""Edge cases of the CUDA path: a mesh of one element of every type (the
smallest chunk, one CTA, every target private) for every form in float64
and float32, against the oracle; and a mesh with no elements, which returns
empty (or zero) results without launching a kernel."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu

ONE = {
    "triangle": ([[0.0, 0.0], [1.3, 0.1], [0.2, 0.9]], [[0, 1, 2]]),
    "triangle6": ([[0.0, 0.0], [1.3, 0.1], [0.2, 0.9], [0.75, 0.5], [0.1, 0.45], [0.65, 0.05]], [[0, 1, 2, 3, 4, 5]]),
    "tetra": ([[0.0, 0.0, 0.0], [1.1, 0.1, 0.0], [0.1, 0.9, 0.1], [0.2, 0.1, 1.2]], [[0, 1, 2, 3]]),
    "quad": ([[0.0, 0.0], [1.2, 0.1], [0.1, 0.9], [1.1, 1.05]], [[0, 1, 2, 3]]),
}


def _tet10():
    v = np.array(ONE["tetra"][0])
    edges = [[2, 3], [1, 3], [1, 2], [0, 3], [0, 2], [0, 1]]
    pts = np.concatenate([v, [(v[a] + v[b]) / 2 + 0.02 * (k + 1) for k, (a, b) in enumerate(edges)]])
    return pts.tolist(), [list(range(10))]


def _quad9():
    v = np.array(ONE["quad"][0])
    edges = [[0, 1], [0, 2], [1, 3], [2, 3]]
    mids = [(v[a] + v[b]) / 2 + 0.03 * (k + 1) for k, (a, b) in enumerate(edges)]
    return np.concatenate([v, mids, [v.mean(0)]]).tolist(), [list(range(9))]


ONE["tetra10"] = _tet10()
ONE["quad9"] = _quad9()


@pytest.mark.parametrize("etype", sorted(ONE))
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_single_element(etype, dtype, cuda):
    pts_l, conn_l = ONE[etype]
    pts = torch.tensor(pts_l, dtype=torch.float64)
    conn = torch.tensor(conn_l)
    tol = 1e-12 if dtype == torch.float64 else 2e-5
    mesh = tg.Mesh(pts.to(dtype), {etype: conn}).to(cuda)
    kappa = torch.tensor([1.7], dtype=dtype, device=cuda)
    K_asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    K = K_asm(mesh.points, element_data={"kappa": kappa})
    M = tg.MassElementAssembler.from_assembler(K_asm)(mesh.points)
    El = tg.LinearElasticityElementAssembler.from_assembler(K_asm, E=2.0, nu=0.3)(mesh.points)
    b = tg.const_node_assembler(1.5).from_mesh(mesh)(mesh.points)
    N = pts.shape[0]
    _, _, Ko = O.assemble_matrix(pts, conn, N, lambda p, c: O.element_locals_diffusion(p, c, etype, torch.tensor([1.7], dtype=torch.float64), 2))
    _, _, Mo = O.assemble_matrix(pts, conn, N, lambda p, c: O.element_locals_mass(p, c, etype, 2))
    _, _, Eo = O.assemble_matrix(pts, conn, N, lambda p, c: O.element_locals_elasticity(p, c, etype, 2.0, 0.3, 2))
    bo = O.assemble_load(pts, conn, etype, N, const=1.5)
    assert K.values.dtype == dtype
    assert rel_fro(K.values.double(), Ko) <= tol
    assert rel_fro(M.values.double(), Mo) <= tol
    assert rel_fro(El.values.double(), Eo) <= tol
    assert rel_fro(b.double(), bo) <= tol


def test_empty_mesh(cuda):
    pts = torch.tensor([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]], dtype=torch.float64)
    mesh = tg.Mesh(pts, {"triangle": torch.zeros((0, 3), dtype=torch.int64)}).to(cuda)
    K_asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    K = K_asm(mesh.points)
    assert K.values.numel() == 0 and K.shape == (3, 3)
    b = tg.const_node_assembler(1.0).from_mesh(mesh)(mesh.points)
    assert b.shape == (3,) and float(b.abs().sum()) == 0.0


@pytest.mark.parametrize("etype,make,qorder", [
    ("tetra10", lambda: tg.gen_unit_cube(3, order=2, jitter=0.1, seed=141), 4),
    ("triangle6", lambda: tg.gen_unit_square(6, order=2, jitter=0.1, seed=142), 4),
    ("quad9", lambda: tg.gen_unit_square(6, order=2, jitter=0.1, seed=143, cell="quad"), 7),
    ("quad", lambda: tg.gen_unit_square(8, jitter=0.2, seed=144, cell="quad"), 7),
])
def test_highest_quadrature_orders(etype, make, qorder, cuda):
    """The largest tabulated rules (tet and triangle order 4, quadrilateral
    order 7: 49 points) shrink the chunks until their shared memory fits;
    every form still matches the oracle."""
    from tensormesh_gb300.plan import chunk_elems, CHUNK_ELEMS
    base = make()
    mesh = base.to(cuda)
    E = base.n_elements
    kappa = torch.from_numpy(np.random.default_rng(145).lognormal(0.0, 1.0, E))
    Ey = torch.from_numpy(np.random.default_rng(146).uniform(0.5, 2.0, E))
    K_asm = tg.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=qorder)
    K, M = tg.assemble_forms([K_asm, tg.MassElementAssembler.from_assembler(K_asm)], mesh.points,
                             {"kappa": kappa.to(cuda)})
    El = tg.LinearElasticityElementAssembler.from_assembler(K_asm, nu=0.3)(mesh.points, element_data={"E": Ey.to(cuda)})
    pts, conn = base.points, base.elements()
    _, _, Ko = O.assemble_matrix(pts, conn, base.n_points,
                                 lambda p, c, kappa: O.element_locals_diffusion(p, c, etype, kappa, qorder), kappa=kappa)
    _, _, Mo = O.assemble_matrix(pts, conn, base.n_points, lambda p, c: O.element_locals_mass(p, c, etype, qorder))
    _, _, Eo = O.assemble_matrix(pts, conn, base.n_points,
                                 lambda p, c, E: O.element_locals_elasticity(p, c, etype, E, 0.3, qorder), E=Ey)
    assert rel_fro(K, Ko) <= 1e-12 and rel_fro(M, Mo) <= 1e-12
    assert rel_fro(El.values, Eo) <= 1e-12
    if etype == "quad9":
        assert chunk_elems(etype, True, qorder) < CHUNK_ELEMS[(etype, True)]
