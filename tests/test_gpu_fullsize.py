"""Full-size benchmark workloads on the GPU against fingerprints of the
reference's own outputs (tests/golden/full_checksums.json): Frobenius norm
and two positively weighted sums of the value arrays, within 1e-12 of the
sum of absolute values; pattern hashes bit-exact; the Poisson L2 error."""
import json
import os

import pytest
import torch

import tensormesh_gb300 as tg
from conftest import GOLDEN
from oracle import fem_oracle as O
from tensormesh_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _full():
    with open(os.path.join(GOLDEN, "full_checksums.json")) as fh:
        return json.load(fh)


def _close(values, ref, tol=1e-12):
    ck = O.checksum(values.detach().cpu())
    assert ck["n"] == ref["n"]
    for key in ("fro", "w1", "w2"):
        assert abs(ck[key] - ref[key]) <= tol * ref["abs"], (key, ck[key], ref[key])


def test_diffusion_mass_tet_64(cuda):
    ref = _full()["diffusion_mass_tet_64"]
    wl = W.diffusion_mass_tet(64)
    mesh = wl.mesh.to(cuda)
    K_asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    M_asm = tg.MassElementAssembler.from_assembler(K_asm)
    kappa = wl.data["kappa"].to(cuda)
    K, M = tg.assemble_forms([K_asm, M_asm], mesh.points, {"kappa": kappa})
    assert K_asm.edges.shape[1] == ref["nnz"]
    _close(K, ref["K"])
    _close(M, ref["M"])
    Ks = K_asm(mesh.points, element_data={"kappa": kappa})
    assert torch.equal(Ks.values, K)
    assert Ks.layout_hash == ref["hash"]


def test_poisson_tri_256(cuda):
    ref = _full()["poisson_tri_256"]
    wl = W.poisson_tri(256)
    mesh = wl.mesh.to(cuda)
    K = tg.LaplaceElementAssembler.from_mesh(mesh)(mesh.points)
    b = tg.LoadNodeAssembler.from_mesh(mesh)(mesh.points, point_data={"f": wl.data["f"].to(cuda)})
    assert K.layout_hash == ref["hash"]
    _close(K.values, ref["K"])
    _close(b, ref["b"])
    cond = tg.Condenser(mesh.boundary_mask)
    Ki, bi = cond(K, b)
    ui, info = tg.pcg_solve(Ki, bi, rtol=1e-13, return_info=True)
    assert info.converged
    u = cond.recover(ui).cpu()
    err = float((u - wl.data["exact"]).norm() / wl.data["exact"].norm())
    assert abs(err - ref["l2_rel_error"]) <= 1e-8 * ref["l2_rel_error"], err


def test_inverse_diffusion_tet_48(cuda):
    ref = _full()["inverse_diffusion_tet_48"]
    wl = W.inverse_diffusion_tet(48)
    mesh = wl.mesh.to(cuda)
    K = tg.LaplaceElementAssembler.from_mesh(mesh)(mesh.points, element_data={"kappa": wl.data["kappa_true"].to(cuda)})
    b = tg.LoadNodeAssembler.from_mesh(mesh)(mesh.points, point_data={"f": wl.data["f"].to(cuda)})
    assert K.layout_hash == ref["hash"]
    _close(K.values, ref["K"])
    _close(b, ref["b"])


def test_elasticity_p2tet_32(cuda):
    ref = _full()["elasticity_p2tet_32"]
    wl = W.elasticity_p2tet(32)
    mesh = wl.mesh.to(cuda)
    asm = tg.LinearElasticityElementAssembler.from_mesh(mesh, nu=0.3)
    El = asm(mesh.points, element_data={"E": wl.data["E"].to(cuda)})
    assert asm.edges.shape[1] == ref["nnz_blocks"]
    assert El.nnz == ref["nnz"]
    _close(El.values, ref["K"])
