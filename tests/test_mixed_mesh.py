"""Meshes with several element types (host side): the union pattern, the
per-type slot maps into it, and the combine segments."""
import numpy as np
import torch

import tensormesh_gb300 as tg
from oracle import fem_oracle as O


def test_union_pattern_and_slot_maps():
    m = tg.gen_unit_square_mixed(7, jitter=0.2, seed=3)
    assert set(m.cells) == {"quad", "triangle"}
    asm = tg.LaplaceElementAssembler.from_mesh(m)
    fns = {et: (lambda p, c, et=et: O.element_locals_diffusion(p, c, et, None, 2)) for et in m.cells}
    edges, _ = O.assemble_mixed(m.points, m.cells, m.n_points, fns)
    assert torch.equal(asm.edges, edges) and asm.edges.dtype == torch.int32
    key = edges[0].long() * m.n_points + edges[1].long()
    for et, conn in m.cells.items():
        B = conn.shape[1]
        pair = (conn[:, :, None].expand(-1, B, B) * m.n_points + conn[:, None, :].expand(-1, B, B)).reshape(-1)
        assert torch.equal(key[asm.projector[et].indices], pair)
    topo = asm._topology
    seg, src = topo.segments(torch.device("cpu"), "matrix")
    assert int(seg[-1]) == sum(t.nnz for t in topo.topos.values())
    # sources of each union position in type order
    offs = np.cumsum([0] + [topo.topos[et].nnz for et in topo.types])
    s = src.numpy()
    for u in range(0, topo.nnz, 37):
        ks = s[seg[u]:seg[u + 1]]
        assert (np.diff(ks) > 0).all()
        for k in ks:
            t = int(np.searchsorted(offs, k, side="right") - 1)
            assert topo.maps[topo.types[t]][k - offs[t]] == u


def test_single_type_mesh_unchanged():
    m = tg.gen_unit_square(4, jitter=0.1, seed=1)
    asm = tg.LaplaceElementAssembler.from_mesh(m)
    assert type(asm._topology).__name__ == "Topology"
