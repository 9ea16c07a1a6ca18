"""The oracle (CPU restatement of the reference's assembly) against the
golden fixtures produced by the reference itself (tests/golden/make_golden.py)."""
import json
import math
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN, load_golden, rel_fro
from oracle import fem_oracle as O

CASES = ["tri3", "tri6", "tet4", "tet10", "quad", "quad9"]
ETYPE = {"tri3": "triangle", "tri6": "triangle6", "tet4": "tetra", "tet10": "tetra10", "quad": "quad",
         "quad9": "quad9"}


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference(case):
    g = load_golden(case)
    et = ETYPE[case]
    pts = torch.from_numpy(g["points"])
    conn = torch.from_numpy(g["conn"])
    N = pts.shape[0]
    kappa, E, f = (torch.from_numpy(g[k]) for k in ("kappa", "E", "f"))
    for qo in g["qorders"]:
        edges, slot = O.element_pattern(conn, N)
        assert np.array_equal(edges.numpy(), g[f"q{qo}_edges"])
        assert np.array_equal(slot.numpy(), g[f"q{qo}_slot"])
        assert O.layout_hash(edges[0], edges[1]) == str(g[f"q{qo}_hash"])
        asm = lambda fn, **kw: O.assemble_matrix(pts, conn, N, fn, **kw)[2]
        K = asm(lambda p, c, kappa: O.element_locals_diffusion(p, c, et, kappa, qo), kappa=kappa)
        L = asm(lambda p, c: O.element_locals_diffusion(p, c, et, None, qo))
        M = asm(lambda p, c: O.element_locals_mass(p, c, et, qo))
        El = asm(lambda p, c, E: O.element_locals_elasticity(p, c, et, E, 0.3, qo), E=E)
        El1 = asm(lambda p, c: O.element_locals_elasticity(p, c, et, 1.7, 0.25, qo))
        for name, val in (("K", K), ("L", L), ("M", M), ("El", El), ("El1", El1)):
            assert rel_fro(val, g[f"q{qo}_{name}"]) < 1e-13, name
        r, c = O.block_coo_indices(edges[0], edges[1], pts.shape[1])
        assert np.array_equal(r.numpy(), g[f"q{qo}_El_row"]) and np.array_equal(c.numpy(), g[f"q{qo}_El_col"])
        assert O.layout_hash(r, c) == str(g[f"q{qo}_El_hash"])
        b = O.assemble_load(pts, conn, et, N, f_nodes=f, qorder=qo)
        bc = O.assemble_load(pts, conn, et, N, const=2.5, qorder=qo)
        bf = O.assemble_load(pts, conn, et, N, qorder=qo,
                             func=lambda x: torch.sin(math.pi * x[..., 0]) * (1 + x[..., 1]))
        assert rel_fro(b, g[f"q{qo}_b"]) < 1e-13
        assert rel_fro(bc, g[f"q{qo}_bconst"]) < 1e-13
        assert rel_fro(bf, g[f"q{qo}_bfunc"]) < 1e-13


def _oracle_adjoint_loss(pts, conn, kappa, u_t, mask):
    N = pts.shape[0]
    _, _, K = O.assemble_matrix(pts, conn, N, lambda p, c, kappa: O.element_locals_diffusion(p, c, "tetra", kappa, 2),
                                kappa=kappa)
    b = O.assemble_load(pts, conn, "tetra", N, const=1.0)
    edges, _ = O.element_pattern(conn, N)
    Kd = torch.zeros(N, N, dtype=torch.float64).index_put((edges[0].long(), edges[1].long()), K, accumulate=True)
    inner = ~mask
    u = torch.linalg.solve(Kd[inner][:, inner], b[inner])
    return ((u - u_t[inner]) ** 2).sum()


def test_oracle_adjoint_matches_reference_autograd():
    g = load_golden("adjoint")
    pts = torch.from_numpy(g["points"]).requires_grad_(True)
    kappa = torch.from_numpy(g["kappa"]).requires_grad_(True)
    loss = _oracle_adjoint_loss(pts, torch.from_numpy(g["conn"]), kappa, torch.from_numpy(g["u_target"]),
                                torch.from_numpy(g["boundary"]))
    loss.backward()
    assert abs(loss.item() - float(g["loss"])) <= 1e-12 * abs(float(g["loss"]))
    assert rel_fro(kappa.grad, g["grad_kappa"]) < 1e-10
    assert rel_fro(pts.grad, g["grad_points"]) < 1e-10


def test_oracle_projector_matches_reference():
    g = load_golden("projector")
    for key in [k[2:] for k in g if k.startswith("x_")]:
        dst, x, y = (torch.from_numpy(g[f"{p}_{key}"]) for p in ("dst", "x", "y"))
        assert torch.allclose(O.reduce_project(dst, x, y.shape[0]), y, rtol=1e-14, atol=1e-14)
    r, c = O.block_coo_indices(torch.from_numpy(g["block_row"]), torch.from_numpy(g["block_col"]), 3)
    dense = torch.zeros(12, 12, dtype=torch.float64).index_put((r, c), torch.from_numpy(g["block_values"]).reshape(-1),
                                                               accumulate=True)
    assert torch.allclose(dense, torch.from_numpy(g["block_dense"]))
    assert O.layout_hash(r, c) == str(g["block_hash"])


def _full():
    with open(os.path.join(GOLDEN, "full_checksums.json")) as fh:
        return json.load(fh)


def _close(ck, ref, tol=1e-12):
    assert ck["n"] == ref["n"]
    for key in ("fro", "w1", "w2"):
        assert abs(ck[key] - ref[key]) <= tol * ref["abs"], (key, ck[key], ref[key])


def test_sketch_signs_are_splitmix64():
    i = torch.tensor([0, 1, 7, 123456789, (1 << 40) + 3, (1 << 62) + 11], dtype=torch.int64)
    h = O.splitmix64(i).tolist()
    assert [x % (1 << 64) for x in h] == [O.splitmix64_py(int(x)) for x in i]


def test_sketch_estimates_the_relative_error():
    """64 sign sketches estimate ||a - b|| / ||b|| within a factor of two,
    whatever the sign pattern of the difference."""
    g = torch.Generator().manual_seed(3)
    b = torch.randn(200_000, generator=g, dtype=torch.float64)
    sb = O.sketch(b)
    for d in (torch.randn(200_000, generator=g, dtype=torch.float64) * 1e-12,
              torch.full((200_000,), 1e-14, dtype=torch.float64),
              torch.zeros(200_000, dtype=torch.float64).index_fill_(0, torch.tensor([17]), 1e-9)):
        true = float(d.norm() / b.norm())
        est = O.sketch_rel_error(O.sketch(b + d), sb, float(b.norm()))
        assert 0.5 * true <= est <= 2.0 * true, (est, true)


def test_oracle_full_poisson_tri_256():
    """Full-size C1 through the oracle: pattern and slot-map hashes, K and b
    against the reference's fingerprints and sign sketches (relative
    Frobenius estimate below 1e-13) and the L2 error of the condensed direct
    solve (3.7935e-05 for the reference)."""
    from tensormesh_gb300 import workloads as W
    ref = _full()["poisson_tri_256"]
    wl = W.poisson_tri(256)
    m = wl.mesh
    edges, slot, K = O.assemble_matrix(m.points, m.elements(), m.n_points,
                                       lambda p, c: O.element_locals_diffusion(p, c, "triangle", None, 2))
    b = O.assemble_load(m.points, m.elements(), "triangle", m.n_points, f_nodes=wl.data["f"])
    assert O.layout_hash(edges[0], edges[1]) == ref["hash"]
    assert O.slot_hash(slot) == ref["slot_sha256"]
    _close(O.checksum(K), ref["K"])
    _close(O.checksum(b), ref["b"])
    for v, r in ((K, ref["K"]), (b, ref["b"])):
        assert O.sketch_rel_error(O.sketch(v), r["sketch"], r["fro"]) <= 1e-13
    u = O.solve_dirichlet(K, edges[0], edges[1], m.n_points, m.boundary_mask, b)
    err = float((u - wl.data["exact"]).norm() / wl.data["exact"].norm())
    assert abs(err - ref["l2_rel_error"]) <= 1e-9 * ref["l2_rel_error"]
    assert abs(err - 3.793522e-05) < 1e-11


def test_reference_per_mesh_path_solves_the_system():
    """The restated per-mesh path (pattern, assembly, Condenser, cg_py)
    reaches the direct solution of the oracle's condensed system."""
    import warnings
    from tensormesh_gb300 import workloads as W
    warnings.filterwarnings("ignore", category=UserWarning)
    w = W.batched_poisson_tri(2)[0]
    m = w.mesh
    u, it = O.reference_per_mesh_solve(m.points, m.elements(), m.boundary_mask, w.data["kappa"], w.data["f"])
    edges, _, K = O.assemble_matrix(m.points, m.elements(), m.n_points,
                                    lambda p, c, kappa: O.element_locals_diffusion(p, c, "triangle", kappa, 2),
                                    kappa=w.data["kappa"])
    b = O.assemble_load(m.points, m.elements(), "triangle", m.n_points, f_nodes=w.data["f"])
    ud = O.solve_dirichlet(K, edges[0], edges[1], m.n_points, m.boundary_mask, b)
    assert it > 1 and float((u - ud).norm() / ud.norm()) < 1e-8
