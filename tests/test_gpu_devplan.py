"""Processing order and chunk plans built on the GPU (tm_morton_order_device,
tm_chunk_plan_device) against the host builders (tm_morton_order,
tm_plan_build): the same arrays, bit for bit, for every element type, both
plan kinds and several chunk sizes; a mesh assembled through the GPU-built
plan gives bitwise the values of the host-built one."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from tensormesh_gb300 import _lib, workloads as W
from tensormesh_gb300.plan import (HostPlan, device_chunk_plan, device_morton_order, device_pattern,
                                   morton_order)

pytestmark = pytest.mark.gpu

MESHES = {
    "tetra": lambda: tg.gen_unit_cube(10, jitter=0.2, seed=51),
    "triangle": lambda: tg.gen_unit_square(40, jitter=0.2, seed=52),
    "tetra10": lambda: tg.gen_unit_cube(4, order=2, jitter=0.1, seed=53),
    "triangle6": lambda: tg.gen_unit_square(12, order=2, jitter=0.1, seed=54),
    "quad": lambda: tg.gen_unit_square(20, jitter=0.2, seed=55, cell="quad"),
    "quad9": lambda: tg.gen_unit_square(10, order=2, jitter=0.1, seed=56, cell="quad"),
}
PLAN_FIELDS = {"conn": "conn", "chunk_begin": "chunk_begin", "chunk_contrib": "chunk_contrib",
               "slot_ptr": "slot_ptr", "contrib": "contrib", "slot_target": "slot_target",
               "slot_mirror": "slot_mirror", "shared_ptr": "shared_ptr", "shared_target": "shared_target",
               "shared_mirror": "shared_mirror"}


def _same_plan(dp, hp):
    for name in PLAN_FIELDS:
        h = hp.arrays[name]
        d = getattr(dp, name).cpu().numpy()
        if name in ("slot_ptr", "contrib"):
            d = d[:h.shape[0]]                  # device copies carry 16 bytes of padding
        if name == "contrib":
            d = d.view(np.uint16)
        assert np.array_equal(d, h), name
    for k in ("n_shared", "n_partials", "max_chunk_slots", "max_chunk_contrib"):
        assert getattr(dp, k) == getattr(hp, k), k


@pytest.mark.parametrize("etype", list(MESHES))
def test_device_order_and_plans_match_host(etype, cuda):
    m = MESHES[etype]()
    conn = m.elements().long()
    conn_np = conn.numpy()
    perm_h = morton_order(m.points.numpy(), conn_np)
    perm_d = device_morton_order(m.points.to(cuda), conn.to(cuda))
    assert np.array_equal(perm_d.cpu().numpy(), perm_h)
    edges, slot, _ = device_pattern(conn.to(cuda), m.n_points)
    nnz = int(edges.shape[1])
    for ch in (16, 64, 256, 768):
        B = conn.shape[1]
        if ch * B * (B + 1) // 2 * 2 > 65536:
            continue
        if min(ch, conn.shape[0]) * B * (B + 1) // 2 > 8192:
            # beyond the device builder's per-chunk sort: it says so (the
            # topology then builds that plan on the host)
            with pytest.raises(_lib.TmError) as ei:
                device_chunk_plan(conn.to(cuda), perm_d, m.n_points, _lib.TM_PLAN_KIND_MATRIX, ch, slot, nnz)
            assert ei.value.status == _lib.TM_ERR_TOO_LARGE
        else:
            hp = HostPlan(conn_np, m.n_points, _lib.TM_PLAN_KIND_MATRIX, ch, perm_h, slot_map=slot.cpu().numpy())
            dp = device_chunk_plan(conn.to(cuda), perm_d, m.n_points, _lib.TM_PLAN_KIND_MATRIX, ch, slot, nnz)
            _same_plan(dp, hp)
        hn = HostPlan(conn_np, m.n_points, _lib.TM_PLAN_KIND_NODE, ch, perm_h)
        dn = device_chunk_plan(conn.to(cuda), perm_d, m.n_points, _lib.TM_PLAN_KIND_NODE, ch)
        _same_plan(dn, hn)


def test_grouped_order_matches_host(cuda):
    wls = W.batched_poisson_tri(24)
    meshes = [w.mesh for w in wls]
    off = np.zeros(len(meshes) + 1, dtype=np.int64)
    np.cumsum([mm.n_points for mm in meshes], out=off[1:])
    groups = np.zeros(len(meshes) + 1, dtype=np.int64)
    np.cumsum([mm.n_elements for mm in meshes], out=groups[1:])
    pts = torch.cat([mm.points for mm in meshes])
    conn = torch.cat([mm.elements().long() + int(off[i]) for i, mm in enumerate(meshes)])
    perm_h = morton_order(pts.numpy(), conn.numpy(), groups)
    perm_d = device_morton_order(pts.to(cuda), conn.to(cuda), groups)
    assert np.array_equal(perm_d.cpu().numpy(), perm_h)


def test_full_size_plan_matches_host(cuda):
    m = W.diffusion_mass_tet(64).mesh
    asm_h = tg.LaplaceElementAssembler.from_mesh(m)              # host mesh: host order, pattern, plan
    topo_h = asm_h._topology
    mg = m.to(cuda)
    asm_d = tg.LaplaceElementAssembler.from_mesh(mg)             # device mesh: all on the GPU
    topo_d = asm_d._topology
    assert np.array_equal(topo_d.perm, topo_h.perm)
    assert torch.equal(topo_d.edges, topo_h.edges) and torch.equal(topo_d.slot, topo_h.slot)
    ph, pd = topo_h.matrix_plan(cuda), topo_d.matrix_plan(cuda)
    for name in PLAN_FIELDS:
        assert torch.equal(getattr(ph, name), getattr(pd, name)), name
    kappa = W.diffusion_mass_tet(64).data["kappa"].to(cuda)
    Kh = asm_h.to(cuda)(mg.points, element_data={"kappa": kappa}).values
    Kd = asm_d(mg.points, element_data={"kappa": kappa}).values
    assert torch.equal(Kh, Kd)
