"""Dirichlet condensation through tm_condense (one launch) against the
oracle's condensation (operator/condense.py:182-337 restated with SciPy):
K_ii and rhs_i - K_io u_o within 1e-13 relative, for a scalar P1 matrix and
a 3x3-block elasticity matrix, one- and two-column right-hand sides, nonzero
Dirichlet values, and condense_rhs after update_dirichlet; gradients against
the same condensation written with torch gathers."""
import numpy as np
import pytest
import scipy.sparse
import scipy.sparse.linalg
import torch

import tensormesh_gb300 as tg
from conftest import rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-13


def _to_scipy(K):
    return scipy.sparse.coo_matrix((K.values.detach().reshape(-1).cpu().numpy(),
                                    (K.row_indices.cpu().numpy(), K.col_indices.cpu().numpy())),
                                   shape=K.shape).tocsr()


def _rel_sparse(A, B):
    return scipy.sparse.linalg.norm(A - B) / scipy.sparse.linalg.norm(B)


def _check(K, mask, rhs, value):
    cond = tg.Condenser(mask, value)
    Kc, fc = cond(K, rhs)
    row, col = K.row_indices.cpu(), K.col_indices.cpu()
    vals = K.values.detach().reshape(-1).cpu()
    m = mask.cpu()
    uo = value.cpu()[m] if value.shape[0] == m.shape[0] else value.cpu()
    cols = rhs.reshape(rhs.shape[0], -1).cpu()
    for w in range(cols.shape[1]):
        Kii, ri, _ = O.condense(vals, row, col, K.shape[0], m, cols[:, w], uo)
        assert _rel_sparse(_to_scipy(Kc), Kii) <= TOL
        got = fc.reshape(fc.shape[0], -1)[:, w].cpu().numpy()
        assert np.linalg.norm(got - ri) <= TOL * np.linalg.norm(ri)
    return cond, Kc, fc


def test_scalar_condense_matches_oracle(cuda):
    mesh = tg.gen_unit_cube(6, jitter=0.2, seed=81).to(cuda)
    rng = np.random.default_rng(82)
    kappa = torch.from_numpy(rng.lognormal(0.0, 1.0, mesh.n_elements)).to(cuda)
    K = tg.LaplaceElementAssembler.from_mesh(mesh)(mesh.points, element_data={"kappa": kappa})
    mask = mesh.boundary_mask
    value = torch.from_numpy(rng.standard_normal(mesh.n_points)).to(cuda)
    rhs1 = torch.from_numpy(rng.standard_normal(mesh.n_points)).to(cuda)
    rhs2 = torch.from_numpy(rng.standard_normal((mesh.n_points, 2))).to(cuda)
    cond, _, _ = _check(K, mask, rhs1, value)
    _check(K, mask, rhs2, value)
    # condense_rhs with new Dirichlet values reuses the cached K_io block
    cond(K, rhs1)
    v2 = torch.from_numpy(rng.standard_normal(int(mask.sum()))).to(cuda)
    cond.update_dirichlet(v2)
    f = cond.condense_rhs(rhs2)
    vals, row, col = K.values.cpu(), K.row_indices.cpu(), K.col_indices.cpu()
    for w in range(2):
        _, ri, _ = O.condense(vals, row, col, K.shape[0], mask.cpu(), rhs2[:, w].cpu(), v2.cpu())
        assert np.linalg.norm(f[:, w].cpu().numpy() - ri) <= TOL * np.linalg.norm(ri)
    # a second call on new values reuses the templates
    K2 = tg.LaplaceElementAssembler.from_mesh(mesh)(mesh.points, element_data={"kappa": 2 * kappa})
    Kc2, _ = cond(K2, rhs1)
    Kc1, _ = tg.Condenser(mask, v2)(K2, rhs1)
    assert torch.equal(Kc2.values, Kc1.values)


def test_block_condense_matches_oracle(cuda):
    mesh = tg.gen_unit_cube(3, order=2, jitter=0.1, seed=83).to(cuda)
    rng = np.random.default_rng(84)
    E = torch.from_numpy(rng.uniform(0.5, 2.0, mesh.n_elements)).to(cuda)
    K = tg.LinearElasticityElementAssembler.from_mesh(mesh, nu=0.3)(mesh.points, element_data={"E": E})
    clamp = (mesh.points[:, 2] == 0.0).repeat_interleave(3)
    value = torch.from_numpy(rng.standard_normal(int(clamp.sum()))).to(cuda)
    rhs = torch.from_numpy(rng.standard_normal(3 * mesh.n_points)).to(cuda)
    cond, Kc, _ = _check(K, clamp, rhs, value)
    assert Kc._block == 3


def test_condense_gradients(cuda):
    mesh = tg.gen_unit_cube(3, jitter=0.2, seed=85).to(cuda)
    rng = np.random.default_rng(86)
    K = tg.LaplaceElementAssembler.from_mesh(mesh)(mesh.points)
    mask = mesh.boundary_mask
    n_out = int(mask.sum())
    base_v = torch.from_numpy(rng.standard_normal(K.values.numel())).to(cuda)
    base_r = torch.from_numpy(rng.standard_normal(mesh.n_points)).to(cuda)
    base_u = torch.from_numpy(rng.standard_normal(n_out)).to(cuda)
    wk = torch.from_numpy(rng.standard_normal(10 ** 6)).to(cuda)

    def loss(vals, rhs, uo, fused):
        if fused:
            cond = tg.Condenser(mask, uo)
            Kc, f = cond(K.with_values(vals), rhs)
            kv = Kc.values
        else:
            inner = ~mask
            row, col = K.row_indices, K.col_indices
            ie = inner[row] & inner[col]
            oe = inner[row] & mask[col]
            loc = torch.full((mesh.n_points,), -1, dtype=torch.long, device=cuda)
            loc[inner] = torch.arange(int(inner.sum()), device=cuda)
            loc[mask] = torch.arange(n_out, device=cuda)
            kv = vals[ie]
            t = torch.zeros(int(inner.sum()), dtype=vals.dtype, device=cuda).index_add(
                0, loc[row[oe]], vals[oe] * uo[loc[col[oe]]])
            f = rhs[inner] - t
        return (kv * wk[:kv.numel()]).sum() + (f * wk[-f.numel():]).sum() + (f ** 2).sum()

    grads = []
    for fused in (True, False):
        v = base_v.clone().requires_grad_(True)
        r = base_r.clone().requires_grad_(True)
        u = base_u.clone().requires_grad_(True)
        loss(v, r, u, fused).backward()
        grads.append((v.grad, r.grad, u.grad))
    for a, b in zip(*grads):
        assert rel_fro(a, b) <= 1e-12
