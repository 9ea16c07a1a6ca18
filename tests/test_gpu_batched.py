"""Batched uneven-mesh Poisson: one assembly launch, one load launch and
one batched Jacobi-PCG launch for all meshes, against per-mesh solves
(the oracle's assembly and a direct SciPy solve).  Tolerances: solutions
within 1e-8 relative (systems solved to 1e-10 relative residual); float32
within 1e-3 of float64."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from tensormesh_gb300.batched import BatchedDiffusion
from conftest import rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


def _batch(sizes, seed=51):
    rng = np.random.default_rng(seed)
    meshes, kappas, fs = [], [], []
    for i, n in enumerate(sizes):
        m = tg.gen_unit_square(int(n), jitter=0.2, seed=seed * 100 + i)
        meshes.append(m)
        kappas.append(torch.from_numpy(rng.lognormal(0.0, 1.0, m.n_elements)))
        fs.append(torch.from_numpy(rng.uniform(-1.0, 1.0, m.n_points)))
    return meshes, kappas, fs


def _oracle_solution(m, kappa, f):
    et = m.default_element_type
    edges, _, K = O.assemble_matrix(m.points, m.elements(), m.n_points,
                                    lambda p, c, kappa: O.element_locals_diffusion(p, c, et, kappa, 2),
                                    kappa=kappa)
    b = O.assemble_load(m.points, m.elements(), et, m.n_points, f_nodes=f)
    return O.solve_dirichlet(K, edges[0], edges[1], m.n_points, m.boundary_mask, b)


def test_batched_solve_matches_per_mesh(cuda):
    sizes = [1, 3, 7, 16, 5, 24, 11]          # n = 1: every node on the boundary
    meshes, kappas, fs = _batch(sizes)
    batch = BatchedDiffusion([m.to(cuda) for m in meshes])
    u, st = batch.solve(torch.cat(kappas), torch.cat(fs), rtol=1e-12)
    assert st.all_converged, st.flag
    assert float(st.relative_residual.max()) <= 1e-12
    for m, k, f, ui in zip(meshes, kappas, fs, batch.split(u)):
        ref = _oracle_solution(m, k, f)
        if float(ref.norm()) == 0.0:
            assert float(ui.abs().max()) == 0.0
        else:
            assert rel_fro(ui, ref) <= 1e-9
    u2, _ = batch.solve(torch.cat(kappas), torch.cat(fs), rtol=1e-12)
    assert torch.equal(u, u2), "batched solve must be bitwise reproducible"


def test_graph_replay_and_float32(cuda):
    meshes, kappas, fs = _batch([6, 13, 9, 20], seed=52)
    batch = BatchedDiffusion([m.to(cuda) for m in meshes]).capture(rtol=1e-10)
    u_eager, _ = BatchedDiffusion([m.to(cuda) for m in meshes]).solve(torch.cat(kappas), torch.cat(fs), rtol=1e-10)
    u, st = batch.replay(torch.cat(kappas), torch.cat(fs))
    torch.cuda.synchronize()
    assert st.all_converged
    assert torch.equal(u, u_eager)
    k2 = [k * 2.0 for k in kappas]                  # new coefficients through the same graph
    u2, st2 = batch.replay(torch.cat(k2), torch.cat(fs))
    torch.cuda.synchronize()
    assert st2.all_converged
    assert rel_fro(u2, u_eager / 2.0) <= 1e-8
    b32 = BatchedDiffusion([m.to(cuda) for m in meshes], dtype=torch.float32)
    u32, st32 = b32.solve(torch.cat(kappas), torch.cat(fs), rtol=1e-6)
    assert u32.dtype == torch.float32 and st32.all_converged
    assert rel_fro(u32, u_eager) <= 1e-3


@pytest.mark.parametrize("order,cell", [(2, "triangle"), (1, "quad"), (2, "quad")])
def test_batched_other_element_types(order, cell, cuda):
    """Batches of P2 triangles, Q1 and Q2 quadrilaterals: the same launches
    (general assembly path, block-diagonal PCG) against per-mesh solves."""
    rng = np.random.default_rng(55)
    meshes, kappas, fs = [], [], []
    for i, n in enumerate([3, 6, 4]):
        m = tg.gen_unit_square(n, order=order, jitter=0.1, seed=560 + i, cell=cell)
        meshes.append(m)
        kappas.append(torch.from_numpy(rng.lognormal(0.0, 1.0, m.n_elements)))
        fs.append(torch.from_numpy(rng.uniform(-1.0, 1.0, m.n_points)))
    batch = BatchedDiffusion([m.to(cuda) for m in meshes])
    u, st = batch.solve(torch.cat(kappas), torch.cat(fs), rtol=1e-12)
    assert st.all_converged
    for m, k, f, ui in zip(meshes, kappas, fs, batch.split(u)):
        assert rel_fro(ui, _oracle_solution(m, k, f)) <= 1e-9


def test_mixed_precision_refinement_matches_per_mesh(cuda):
    """precision="mixed": float32 inner Jacobi-PCG solves inside float64
    refinement reach the same test on the true float64 residual; solutions
    against the oracle's direct solves, bitwise reproducible, and the graph
    replay equal to the eager call."""
    sizes = [1, 3, 7, 16, 5, 24, 11, 40]
    meshes, kappas, fs = _batch(sizes, seed=57)
    batch = BatchedDiffusion([m.to(cuda) for m in meshes])
    kap, f = torch.cat(kappas), torch.cat(fs)
    u, st = batch.solve(kap, f, rtol=1e-12, precision="mixed")
    assert st.all_converged, st.flag
    assert float(st.relative_residual.max()) <= 1e-12
    for m, k, fi, ui in zip(meshes, kappas, fs, batch.split(u)):
        ref = _oracle_solution(m, k, fi)
        if float(ref.norm()) == 0.0:
            assert float(ui.abs().max()) == 0.0
        else:
            assert rel_fro(ui, ref) <= 1e-9
    u2, _ = batch.solve(kap, f, rtol=1e-12, precision="mixed")
    assert torch.equal(u, u2)
    u64, st64 = batch.solve(kap, f, rtol=1e-12)
    assert rel_fro(u, u64) <= 1e-9
    g = BatchedDiffusion([m.to(cuda) for m in meshes]).capture(rtol=1e-12, precision="mixed")
    ug, stg = g.replay(kap, f)
    torch.cuda.synchronize()
    assert stg.all_converged and torch.equal(ug, u)


def test_mixed_precision_limits(cuda):
    """An inner tolerance outside (0, 1) and a float32 batch are refused;
    max_outer = 0 stops before any correction (flag max_iter)."""
    meshes, kappas, fs = _batch([6, 9], seed=58)
    batch = BatchedDiffusion([m.to(cuda) for m in meshes])
    kap, f = torch.cat(kappas), torch.cat(fs)
    with pytest.raises(RuntimeError):
        batch.solve(kap, f, precision="mixed", inner_rtol=1.5)
    _, st = batch.solve(kap, f, precision="mixed", max_outer=0)
    assert bool((st.flag == 2).all())
    b32 = BatchedDiffusion([m.to(cuda) for m in meshes], dtype=torch.float32)
    with pytest.raises(ValueError):
        b32.solve(kap, f, precision="mixed")
