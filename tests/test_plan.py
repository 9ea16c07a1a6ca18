"""Native plan builder (tm_plan_build): CSR pattern and slot map bit-exact
with the oracle, and the chunk plan's fixed-order reduction (emulated here in
numpy on oracle element locals) equal to the oracle's index_add_ scatter."""
import numpy as np
import pytest
import torch

from tensormesh_gb300 import _lib
from tensormesh_gb300.mesh import gen_unit_cube, gen_unit_square
from tensormesh_gb300.plan import HostPlan, morton_order
from oracle import fem_oracle as O


def emulate_matrix(h, loc):
    """Phase 2 + finalisation of k_matrix on [E,B,B,H,H] locals (element order)."""
    a = h.arrays
    B = h.n_basis
    H = loc.shape[-1]
    iu = [(p, q) for p in range(B) for q in range(p, B)]
    L = np.stack([loc[a["perm"]][:, p, q] for p, q in iu], 1)
    out = np.full((h.nnz, H, H), np.nan)
    part = np.full((h.n_partials, H, H), np.nan)
    CH = h.chunk_elems
    for k in range(h.n_chunks):
        Lc = L[k * CH:(k + 1) * CH].reshape(-1, H, H)
        for s in range(a["chunk_begin"][k], a["chunk_begin"][k + 1]):
            acc = np.zeros((H, H))
            for p in range(a["slot_ptr"][s], a["slot_ptr"][s + 1]):
                code = int(a["contrib"][p])
                acc += Lc[code >> 1].T if code & 1 else Lc[code >> 1]
            t = a["slot_target"][s]
            if t >= 0:
                out[t] = acc
                if a["slot_mirror"][s] != t:
                    out[a["slot_mirror"][s]] = acc.T
            else:
                part[-t - 1] = acc
    for sh in range(h.n_shared):
        acc = part[a["shared_ptr"][sh]:a["shared_ptr"][sh + 1]].sum(0)
        t, m = a["shared_target"][sh], a["shared_mirror"][sh]
        out[t] = acc
        if m != t:
            out[m] = acc.T
    return out


def emulate_vector(h, loc, n_points):
    a = h.arrays
    L = loc[a["perm"]]
    out = np.zeros((n_points,) + loc.shape[2:])
    part = np.full((h.n_partials,) + loc.shape[2:], np.nan)
    CH = h.chunk_elems
    for k in range(h.n_chunks):
        Lc = L[k * CH:(k + 1) * CH].reshape(-1, *loc.shape[2:])
        for s in range(a["chunk_begin"][k], a["chunk_begin"][k + 1]):
            acc = sum(Lc[int(a["contrib"][p]) >> 1] for p in range(a["slot_ptr"][s], a["slot_ptr"][s + 1]))
            t = a["slot_target"][s]
            if t >= 0:
                out[t] = acc
            else:
                part[-t - 1] = acc
    for sh in range(h.n_shared):
        out[a["shared_target"][sh]] = part[a["shared_ptr"][sh]:a["shared_ptr"][sh + 1]].sum(0)
    return out


MESHES = [
    ("tetra", lambda: gen_unit_cube(3, jitter=0.2, seed=1)),
    ("triangle", lambda: gen_unit_square(5, jitter=0.2, seed=2)),
    ("tetra10", lambda: gen_unit_cube(2, order=2, jitter=0.1, seed=3)),
    ("triangle6", lambda: gen_unit_square(3, order=2, jitter=0.1, seed=4)),
]


@pytest.mark.parametrize("et,make", MESHES)
@pytest.mark.parametrize("chunk", [1, 5, 16, 500])
def test_pattern_and_reduction(et, make, chunk):
    m = make()
    conn = m.elements().numpy()
    perm = morton_order(m.points.numpy(), conn)
    h = HostPlan(conn, m.n_points, _lib.TM_PLAN_KIND_MATRIX, chunk, perm)
    edges, slot = O.element_pattern(m.elements(), m.n_points)
    assert np.array_equal(h.arrays["edge_row"], edges[0].numpy())
    assert np.array_equal(h.arrays["edge_col"], edges[1].numpy())
    assert np.array_equal(h.arrays["slot"], slot.numpy())
    E = torch.rand(conn.shape[0], dtype=torch.float64, generator=torch.Generator().manual_seed(0)) + 0.5
    loc = O.element_locals_elasticity(m.points, m.elements(), et, E, 0.3, 2).numpy()
    out = emulate_matrix(h, loc)
    _, _, ref = O.assemble_matrix(m.points, m.elements(), m.n_points,
                                  lambda p, c, E: O.element_locals_elasticity(p, c, et, E, 0.3, 2), E=E)
    assert not np.isnan(out).any()
    np.testing.assert_allclose(out, ref.numpy(), rtol=0, atol=1e-13 * np.abs(ref.numpy()).max())
    # node plan: load vector
    hn = HostPlan(conn, m.n_points, _lib.TM_PLAN_KIND_NODE, chunk, perm)
    locv = np.random.default_rng(0).standard_normal((conn.shape[0], conn.shape[1], 2))
    outv = emulate_vector(hn, locv, m.n_points)
    refv = O.reduce_project(torch.from_numpy(conn.reshape(-1)), torch.from_numpy(locv.reshape(-1, 2)), m.n_points)
    np.testing.assert_allclose(outv, refv.numpy(), atol=1e-13)


def test_slot_map_reuse_and_identity_perm():
    m = gen_unit_cube(2, jitter=0.1, seed=9)
    conn = m.elements().numpy()
    h1 = HostPlan(conn, m.n_points, _lib.TM_PLAN_KIND_MATRIX, 7)
    h2 = HostPlan(conn, m.n_points, _lib.TM_PLAN_KIND_MATRIX, 3, slot_map=h1.arrays["slot"])
    assert h2.nnz == h1.nnz
    assert np.array_equal(h1.arrays["perm"], np.arange(conn.shape[0]))
    loc = O.element_locals_diffusion(m.points, m.elements(), "tetra", None, 2).numpy()[..., None, None]
    np.testing.assert_allclose(emulate_matrix(h2, loc)[:, 0, 0], emulate_matrix(h1, loc)[:, 0, 0], atol=1e-14)


def test_degenerate_repeated_node():
    """An element listing a node twice maps two local pairs onto one diagonal
    slot (both the pair and its transpose are added)."""
    pts = torch.tensor([[0., 0.], [1., 0.], [0., 1.], [1., 1.]], dtype=torch.float64)
    conn = np.array([[0, 1, 2], [1, 3, 2], [1, 1, 2]])
    h = HostPlan(conn, 4, _lib.TM_PLAN_KIND_MATRIX, 2)
    rng = np.random.default_rng(1)
    loc = rng.standard_normal((3, 3, 3, 2, 2))
    loc = loc + loc.transpose(0, 2, 1, 4, 3)                 # symmetric element matrices
    edges, slot = O.element_pattern(torch.from_numpy(conn), 4)
    ref = O.reduce_project(slot, torch.from_numpy(loc.reshape(-1, 2, 2)), edges.shape[1]).numpy()
    np.testing.assert_allclose(emulate_matrix(h, loc), ref, atol=1e-13)


def _fan(n):
    """n triangles around node 0 (one node in every element: its targets
    are shared by every chunk), ring nodes in shuffled numbering."""
    ang = np.linspace(0.0, 2 * np.pi, n, endpoint=False)
    pts = np.concatenate([[[0.0, 0.0]], np.stack([np.cos(ang), np.sin(ang)], 1)])
    ring = 1 + np.random.default_rng(3).permutation(n)
    conn = np.stack([np.zeros(n, np.int64), ring, np.roll(ring, -1)], 1)
    return torch.from_numpy(pts), torch.from_numpy(conn)


@pytest.mark.parametrize("chunk", [3, 16, 128])
def test_fan_mesh_high_partial_counts(chunk):
    """A node in all of 600 elements: its shared targets have a partial from
    every chunk, and both reductions still match the oracle."""
    pts, conn_t = _fan(600)
    conn = conn_t.numpy()
    perm = morton_order(pts.numpy(), conn)
    h = HostPlan(conn, pts.shape[0], _lib.TM_PLAN_KIND_MATRIX, chunk, perm)
    assert np.diff(h.arrays["shared_ptr"]).max() == h.n_chunks
    E = torch.rand(conn.shape[0], dtype=torch.float64, generator=torch.Generator().manual_seed(2)) + 0.5
    loc = O.element_locals_elasticity(pts, conn_t, "triangle", E, 0.3, 2).numpy()
    _, _, ref = O.assemble_matrix(pts, conn_t, pts.shape[0],
                                  lambda p, c, E: O.element_locals_elasticity(p, c, "triangle", E, 0.3, 2), E=E)
    np.testing.assert_allclose(emulate_matrix(h, loc), ref.numpy(), rtol=0, atol=1e-13 * np.abs(ref.numpy()).max())
    hn = HostPlan(conn, pts.shape[0], _lib.TM_PLAN_KIND_NODE, chunk, perm)
    locv = np.random.default_rng(4).standard_normal((conn.shape[0], 3, 1))
    refv = O.reduce_project(conn_t.reshape(-1), torch.from_numpy(locv.reshape(-1, 1)), pts.shape[0])
    np.testing.assert_allclose(emulate_vector(hn, locv, pts.shape[0]), refv.numpy(), atol=1e-12)


def test_empty_mesh():
    h = HostPlan(np.zeros((0, 4), dtype=np.int64), 5, _lib.TM_PLAN_KIND_MATRIX, 16)
    assert h.nnz == 0 and h.n_chunks == 0 and h.n_partials == 0


def test_rejects_bad_input():
    with pytest.raises(_lib.TmError):
        HostPlan(np.array([[0, 1, 7]]), 3, _lib.TM_PLAN_KIND_MATRIX, 4)          # index out of range
    with pytest.raises(_lib.TmError):
        HostPlan(np.array([[0, 1, 2], [0, 2, 1]]), 3, _lib.TM_PLAN_KIND_MATRIX, 4, perm=np.array([1, 1]))
    with pytest.raises(_lib.TmError):
        HostPlan(np.zeros((10, 10), dtype=np.int64), 10, _lib.TM_PLAN_KIND_MATRIX, 1000)  # u16 overflow
    with pytest.raises(_lib.TmError):
        HostPlan(np.array([[0, 1, 2]]), 3, _lib.TM_PLAN_KIND_MATRIX, 4, slot_map=np.array([0, 1, 2, -1, 3, 4, 5, 6, 7]))


@pytest.mark.parametrize("kind", [_lib.TM_PLAN_KIND_MATRIX, _lib.TM_PLAN_KIND_NODE])
def test_plan_orderings(kind):
    """Slots of a chunk by decreasing contribution count, each target's
    contributions in (element, entry) order; shared targets by decreasing
    partial count, then target; partials of a target in chunk order."""
    m = gen_unit_cube(4, jitter=0.2, seed=5)
    conn = m.elements().numpy()
    h = HostPlan(conn, m.n_points, kind, 32, morton_order(m.points.numpy(), conn))
    a = h.arrays
    cnt = np.diff(a["slot_ptr"])
    for k in range(h.n_chunks):
        c = cnt[a["chunk_begin"][k]:a["chunk_begin"][k + 1]]
        assert (np.diff(c) <= 0).all()
        for s in range(a["chunk_begin"][k], a["chunk_begin"][k + 1]):
            codes = a["contrib"][a["slot_ptr"][s]:a["slot_ptr"][s + 1]] >> 1
            assert (np.diff(codes.astype(np.int64)) > 0).all()
    pc = np.diff(a["shared_ptr"])
    assert (pc >= 2).all() and (np.diff(pc) <= 0).all()
    key = -pc.astype(np.int64) * (1 << 32) + a["shared_target"]
    assert (np.diff(key) > 0).all()
    chunk_of_slot = np.repeat(np.arange(h.n_chunks), np.diff(a["chunk_begin"]))
    part_chunk = np.full(h.n_partials, -1)
    shared = a["slot_target"] < 0
    part_chunk[-a["slot_target"][shared] - 1] = chunk_of_slot[shared]
    for sh in range(h.n_shared):
        assert (np.diff(part_chunk[a["shared_ptr"][sh]:a["shared_ptr"][sh + 1]]) > 0).all()


@pytest.mark.parametrize("kind", [_lib.TM_PLAN_KIND_MATRIX, _lib.TM_PLAN_KIND_NODE])
def test_plan_independent_of_host_threads(kind, monkeypatch):
    """The plan is built on host threads (TM_HOST_THREADS, default all
    cores); every array is the same whatever their number."""
    m = gen_unit_cube(6, jitter=0.2, seed=7)
    fan_pts, fan_conn = _fan(900)
    for pts, conn, n_points in ((m.points.numpy(), m.elements().numpy(), m.n_points),
                                (fan_pts.numpy(), fan_conn.numpy(), fan_pts.shape[0])):
        perm = morton_order(pts, conn)
        built = []
        for threads in ("1", "3", "8"):
            monkeypatch.setenv("TM_HOST_THREADS", threads)
            built.append(HostPlan(conn, n_points, kind, 64, perm))
        for h in built[1:]:
            for name, arr in built[0].arrays.items():
                assert np.array_equal(arr, h.arrays[name]), name


def _spread(x, dims):
    x = x.astype(np.uint64)
    if dims == 2:
        x &= np.uint64(0xFFFFFFFF)
        for sh, mk in ((16, 0x0000FFFF0000FFFF), (8, 0x00FF00FF00FF00FF), (4, 0x0F0F0F0F0F0F0F0F),
                       (2, 0x3333333333333333), (1, 0x5555555555555555)):
            x = (x | (x << np.uint64(sh))) & np.uint64(mk)
        return x
    x &= np.uint64(0x1FFFFF)
    for sh, mk in ((32, 0x1F00000000FFFF), (16, 0x1F0000FF0000FF), (8, 0x100F00F00F00F00F),
                   (4, 0x10C30C30C30C30C3), (2, 0x1249249249249249)):
        x = (x | (x << np.uint64(sh))) & np.uint64(mk)
    return x


def _morton_numpy(points, conn):
    """The ordering restated in numpy: stable argsort of the interleaved
    quantised centroid coordinates."""
    D = points.shape[1]
    cent = points[conn[:, :D + 1]].mean(axis=1)
    lo, hi = cent.min(0), cent.max(0)
    span = np.where(hi > lo, hi - lo, 1.0)
    bits = 31 if D == 2 else 21
    q = np.floor((cent - lo) / span * ((1 << bits) - 1)).astype(np.uint64)
    key = np.zeros(conn.shape[0], dtype=np.uint64)
    for d in range(D):
        key |= _spread(q[:, d], D) << np.uint64(d)
    return np.argsort(key, kind="stable").astype(np.int32)


@pytest.mark.parametrize("make", [lambda: gen_unit_cube(7, jitter=0.25, seed=11),
                                  lambda: gen_unit_square(40, jitter=0.25, seed=12),
                                  lambda: gen_unit_cube(3, order=2, jitter=0.1, seed=13)])
def test_morton_order_matches_numpy(make, monkeypatch):
    m = make()
    pts, conn = m.points.numpy(), m.elements().numpy()
    ref = _morton_numpy(pts, conn)
    for threads in ("1", "5"):
        monkeypatch.setenv("TM_HOST_THREADS", threads)
        assert np.array_equal(morton_order(pts, conn), ref)
    with pytest.raises(_lib.TmError):
        morton_order(pts, np.full_like(conn, pts.shape[0]))


def test_grouped_morton_order_and_batch_topology():
    """Element groups (several meshes concatenated, overlapping in space):
    every group is ordered on its own and the groups follow one another; the
    CSR pattern and slot map do not depend on the order, and the chunk plan
    of a grouped batch shares far fewer targets between chunks."""
    from tensormesh_gb300.mesh import Mesh
    from tensormesh_gb300.plan import Topology
    meshes = [gen_unit_square(n, jitter=0.2, seed=40 + n) for n in (6, 9, 4, 12, 7)]
    noff = np.cumsum([0] + [m.n_points for m in meshes])
    eoff = np.cumsum([0] + [m.n_elements for m in meshes])
    pts = torch.cat([m.points for m in meshes])
    conn = torch.cat([m.elements() + int(noff[i]) for i, m in enumerate(meshes)])
    perm = morton_order(pts.numpy(), conn.numpy(), eoff)
    for i, m in enumerate(meshes):
        part = perm[eoff[i]:eoff[i + 1]]
        assert np.array_equal(part - eoff[i], morton_order(m.points.numpy(), m.elements().numpy()))
    with pytest.raises(ValueError):
        morton_order(pts.numpy(), conn.numpy(), eoff[:-1])
    batch = Mesh(pts, {"triangle": conn}, element_groups=eoff).to("cpu")
    assert np.array_equal(batch.element_groups, eoff)
    grouped = Topology(batch.points, batch.elements(), "triangle", 2, element_groups=batch.element_groups)
    mixed = Topology(pts, conn, "triangle", 2)
    assert np.array_equal(grouped.perm, perm)
    assert torch.equal(grouped.edges, mixed.edges) and torch.equal(grouped.slot, mixed.slot)
    ch = 16
    hg = HostPlan(conn.numpy(), pts.shape[0], _lib.TM_PLAN_KIND_MATRIX, ch, grouped.perm)
    hm = HostPlan(conn.numpy(), pts.shape[0], _lib.TM_PLAN_KIND_MATRIX, ch, mixed.perm)
    assert hg.n_partials < hm.n_partials
    E = torch.rand(conn.shape[0], dtype=torch.float64, generator=torch.Generator().manual_seed(6)) + 0.5
    loc = O.element_locals_elasticity(pts, conn, "triangle", E, 0.3, 2).numpy()
    _, _, ref = O.assemble_matrix(pts, conn, pts.shape[0],
                                  lambda p, c, E: O.element_locals_elasticity(p, c, "triangle", E, 0.3, 2), E=E)
    np.testing.assert_allclose(emulate_matrix(hg, loc), ref.numpy(), rtol=0, atol=1e-13 * np.abs(ref.numpy()).max())


def test_from_mesh_takes_the_mesh_element_groups():
    """ElementAssembler.from_mesh and NodeAssembler.from_mesh order the
    elements of a mesh with element groups group by group (as a batch does)."""
    import tensormesh_gb300 as tg
    from tensormesh_gb300.mesh import Mesh
    parts = [gen_unit_square(n, jitter=0.1, seed=60 + n) for n in (5, 3, 8)]
    noff = np.cumsum([0] + [m.n_points for m in parts])
    eoff = np.cumsum([0] + [m.n_elements for m in parts])
    pts = torch.cat([m.points for m in parts])
    conn = torch.cat([m.elements() + int(noff[i]) for i, m in enumerate(parts)])
    mesh = Mesh(pts, {"triangle": conn}, element_groups=eoff)
    expect = morton_order(pts.numpy(), conn.numpy(), eoff)
    K = tg.LaplaceElementAssembler.from_mesh(mesh)
    b = tg.LoadNodeAssembler.from_mesh(mesh)
    assert np.array_equal(K._topo(True).perm, expect)
    assert np.array_equal(b._topo(False).perm, expect)
    plain = tg.LaplaceElementAssembler.from_mesh(Mesh(pts, {"triangle": conn}))
    assert np.array_equal(plain._topo(True).perm, morton_order(pts.numpy(), conn.numpy()))
