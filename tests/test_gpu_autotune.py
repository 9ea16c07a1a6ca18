"""Chunk-size autotuner on the GPU: the tuned size becomes the plan of the
assembly calls; values differ from those of the static chunk size only at the
rounding level (1e-13 relative Frobenius; the reduction's grouping changes)
and not at all between two calls with one size; a batch tuned this way
solves like an untuned one (1e-10 relative)."""
import json

import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from tensormesh_gb300 import autotune
from tensormesh_gb300.batched import BatchedDiffusion
from conftest import rel_fro

pytestmark = pytest.mark.gpu


@pytest.fixture
def tuner(monkeypatch, tmp_path):
    path = tmp_path / "autotune.json"
    monkeypatch.setenv("TM_AUTOTUNE_CACHE", str(path))
    autotune.clear()
    yield path
    autotune.clear()


def test_tune_matrix_pair_and_vector(cuda, tuner):
    m = tg.gen_unit_cube(10, jitter=0.2, seed=3).to(cuda)
    kappa = torch.rand(m.n_elements, dtype=torch.float64, device=cuda) + 0.5
    K = tg.LaplaceElementAssembler.from_mesh(m)
    M = tg.MassElementAssembler.from_assembler(K)
    ref_k, ref_m = tg.assemble_forms([K, M], m.points, {"kappa": kappa})
    topo = K._topo(True)
    static = topo.chunk_for("scalar", cuda, torch.float64)
    best, times = autotune.tune_matrix([K, M], m.points, {"kappa": kappa}, sizes=(32, 128, 512), repeats=3,
                                       save=True)
    assert set(times) == {32, 128, 512, static}
    assert best == min(times, key=lambda c: (times[c], c))
    assert topo.chunk_for("scalar", cuda, torch.float64) == best
    assert topo.matrix_plan(cuda, dtype=torch.float64).chunk_elems == best
    assert topo.chunk_for("scalar", cuda, torch.float32) == static        # other dtypes keep the default
    k1, m1 = tg.assemble_forms([K, M], m.points, {"kappa": kappa})
    k2, m2 = tg.assemble_forms([K, M], m.points, {"kappa": kappa})
    assert torch.equal(k1, k2) and torch.equal(m1, m2)
    assert rel_fro(k1, ref_k) <= 1e-13 and rel_fro(m1, ref_m) <= 1e-13
    key = autotune.make_key(autotune.device_tag(cuda), "tetra", "scalar", 2, torch.float64)
    assert json.loads(tuner.read_text())[key] == best
    # losing candidates' device plans are released
    assert {k[1] for k in topo._plans if k[0] == "matrix"} <= {best, topo.chunk_for("block", cuda, torch.float64)}

    b_asm = tg.LoadNodeAssembler.from_mesh(m)
    f = torch.rand(m.n_points, dtype=torch.float64, device=cuda)
    ref_b = b_asm(m.points, point_data={"f": f})
    best_n, times_n = autotune.tune_vector(b_asm, m.points, {"f": f}, sizes=(32, 512), repeats=3)
    assert best_n in times_n and len(times_n) >= 2
    assert b_asm._topo(False).node_plan(cuda, dtype=torch.float64).chunk_elems == best_n
    assert rel_fro(b_asm(m.points, point_data={"f": f}), ref_b) <= 1e-13


def test_tune_elasticity_p2(cuda, tuner):
    m = tg.gen_unit_cube(3, order=2, jitter=0.1, seed=4).to(cuda)
    E = torch.rand(m.n_elements, dtype=torch.float64, device=cuda) + 0.5
    asm = tg.LinearElasticityElementAssembler.from_mesh(m)
    (ref,) = tg.assemble_forms([asm], m.points, {"E": E})
    static = asm._topo(True).chunk_for("block", cuda, torch.float64)
    best, times = autotune.tune_matrix([asm], m.points, {"E": E}, repeats=2)
    assert static in times
    assert set(times) <= set(autotune.candidates("tetra10", "block", 2, autotune.CANDIDATES + (static,)))
    assert asm._topo(True).matrix_plan(cuda, block=True, dtype=torch.float64).chunk_elems == best
    (val,) = tg.assemble_forms([asm], m.points, {"E": E})
    assert rel_fro(val, ref) <= 1e-13


def test_batched_autotune_solves_like_untuned(cuda, tuner):
    rng = np.random.default_rng(7)
    meshes, kappas, fs = [], [], []
    for i, n in enumerate([4, 9, 17, 6, 12]):
        mm = tg.gen_unit_square(n, jitter=0.2, seed=700 + i)
        meshes.append(mm.to(cuda))
        kappas.append(torch.from_numpy(rng.lognormal(0.0, 1.0, mm.n_elements)))
        fs.append(torch.from_numpy(rng.uniform(-1.0, 1.0, mm.n_points)))
    kappa, f = torch.cat(kappas).to(cuda), torch.cat(fs).to(cuda)
    u0, st0 = BatchedDiffusion(meshes).solve(kappa, f, rtol=1e-12)
    tuned = BatchedDiffusion(meshes, autotune=True)
    assert set(tuned.chunks) == {"matrix", "node"}
    u1, st1 = tuned.capture(rtol=1e-12).replay(kappa, f)
    assert st0.all_converged and st1.all_converged
    assert rel_fro(u1, u0) <= 1e-10
