"""CSR pattern and slot map built on the GPU (tm_pattern_count / _fill)
against the reference's from_mesh outputs: the small golden fixtures of every
element type bit for bit, the full-size workloads through the reference's
pattern hash and slot-map SHA-256, and random meshes against the host
builder.  Bad node indices are rejected."""
import json
import os

import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import GOLDEN, load_golden
from oracle import fem_oracle as O
from tensormesh_gb300 import _lib, workloads as W
from tensormesh_gb300.plan import HostPlan, device_pattern

pytestmark = pytest.mark.gpu

CASES = ["tri3", "tri6", "tet4", "tet10", "quad", "quad9"]


@pytest.mark.parametrize("case", CASES)
def test_device_pattern_matches_reference_fixtures(case, cuda):
    g = load_golden(case)
    conn = torch.from_numpy(g["conn"]).to(cuda)
    N = g["points"].shape[0]
    edges, slot, row_ptr = device_pattern(conn, N)
    qo = int(g["qorders"][0])
    assert np.array_equal(edges.cpu().numpy(), g[f"q{qo}_edges"])
    assert np.array_equal(slot.cpu().numpy(), g[f"q{qo}_slot"])
    rp = np.zeros(N + 1, dtype=np.int64)
    np.cumsum(np.bincount(g[f"q{qo}_edges"][0], minlength=N), out=rp[1:])
    assert np.array_equal(row_ptr.cpu().numpy(), rp)


@pytest.mark.parametrize("name,make,etype", [
    ("diffusion_mass_tet_64", lambda: W.diffusion_mass_tet(64).mesh, "tetra"),
    ("elasticity_p2tet_32", lambda: W.elasticity_p2tet(32).mesh, "tetra10"),
    ("inverse_diffusion_tet_48", lambda: W.inverse_diffusion_tet(48).mesh, "tetra"),
    ("poisson_tri_256", lambda: W.poisson_tri(256).mesh, "triangle"),
])
def test_device_pattern_full_size(name, make, etype, cuda):
    with open(os.path.join(GOLDEN, "full_checksums.json")) as fh:
        ref = json.load(fh)[name]
    m = make()
    edges, slot, _ = device_pattern(m.elements().to(cuda), m.n_points)
    assert O.slot_hash(slot) == ref["slot_sha256"]
    assert O.layout_hash(edges[0].cpu(), edges[1].cpu()) == ref.get("hash", ref.get("hash_blocks"))
    # an assembler built from the mesh on the GPU holds the same arrays
    asm = tg.LaplaceElementAssembler.from_mesh(m.to(cuda))
    assert torch.equal(asm.edges.cpu(), edges.cpu())
    assert torch.equal(asm.projector[etype].indices.cpu(), slot.cpu())


def test_device_pattern_matches_host_builder(cuda):
    rng = np.random.default_rng(5)
    for E, B, N in ((1, 3, 3), (500, 4, 300), (2000, 3, 5000), (300, 10, 900), (50, 9, 2000)):
        conn = np.stack([rng.choice(N, B, replace=False) for _ in range(E)]).astype(np.int64)
        host = HostPlan(conn, N, _lib.TM_PLAN_KIND_MATRIX, 64)
        edges, slot, _ = device_pattern(torch.from_numpy(conn).to(cuda), N)
        assert np.array_equal(edges[0].cpu().numpy(), host.arrays["edge_row"])
        assert np.array_equal(edges[1].cpu().numpy(), host.arrays["edge_col"])
        assert np.array_equal(slot.cpu().numpy(), host.arrays["slot"])


def test_device_pattern_high_degree_node(cuda):
    # a fan of 700 triangles around node 0: its row has 2100 candidates,
    # more than one warp's buffer (the CTA-wide pass takes it)
    n = 700
    conn = np.stack([np.zeros(n, np.int64), np.arange(1, n + 1), np.r_[np.arange(2, n + 1), 1]], 1)
    host = HostPlan(conn, n + 1, _lib.TM_PLAN_KIND_MATRIX, 64)
    edges, slot, _ = device_pattern(torch.from_numpy(conn).to(cuda), n + 1)
    assert np.array_equal(edges[1].cpu().numpy(), host.arrays["edge_col"])
    assert np.array_equal(slot.cpu().numpy(), host.arrays["slot"])


def test_device_pattern_rejects_bad_indices(cuda):
    conn = torch.tensor([[0, 1, 2], [1, 2, 7]], dtype=torch.int32, device=cuda)
    with pytest.raises(_lib.TmError):
        device_pattern(conn, 5)
