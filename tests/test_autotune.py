"""Chunk-size autotuner, host side: candidate filtering, cache keys, the JSON
cache round trip and the lookup that Topology makes before its static
default (a fake device tag stands in for a GPU)."""
import json

import pytest
import torch

from tensormesh_gb300 import autotune
from tensormesh_gb300.mesh import gen_unit_cube
from tensormesh_gb300.plan import CHUNK_ELEMS, NODE_CHUNK_ELEMS, Topology, chunk_elems, chunk_fits

FAKE_TAG = "Fake GPU|152sm|cc103"


@pytest.fixture
def fake_gpu(monkeypatch, tmp_path):
    monkeypatch.setenv("TM_AUTOTUNE_CACHE", str(tmp_path / "autotune.json"))
    monkeypatch.setattr(autotune, "device_tag", lambda device: FAKE_TAG)
    autotune.clear()
    yield tmp_path / "autotune.json"
    autotune.clear()


def test_candidates_fit_codes_and_shared_memory():
    # 16-bit contribution codes: ch * n_local * 2 <= 65536 (tetra10: n_local 55)
    assert max(autotune.candidates("tetra10", "scalar", 2, range(1, 2000))) <= 65536 // 110
    for et, blk in CHUNK_ELEMS:
        kind = "block" if blk else "scalar"
        for q in (1, 2, 3):
            c = autotune.candidates(et, kind, q)
            assert all(chunk_fits(et, blk, q, ch) for ch in c)
            assert chunk_fits(et, blk, q, chunk_elems(et, blk, q))
    # the default list reaches the high quadrature orders of quad9 (16 fits)
    assert autotune.candidates("quad9", "scalar", 7) == [16]
    assert autotune.candidates("triangle", "node", 2) == list(autotune.CANDIDATES)


def test_key_names_every_field():
    k = autotune.make_key(FAKE_TAG, "tetra", "scalar", 2, torch.float64)
    assert k == "Fake GPU|152sm|cc103|tetra|scalar|q2|float64"
    assert autotune.make_key(FAKE_TAG, "tetra", "node", 3, torch.float32).endswith("|node|q3|float32")
    with pytest.raises(ValueError):
        autotune.make_key(FAKE_TAG, "tetra", "matrix", 2, torch.float64)


def test_lookup_only_for_cuda_devices_and_a_dtype(fake_gpu):
    autotune.record(torch.device("cuda", 0), "tetra", "scalar", 2, torch.float64, 128)
    assert autotune.lookup(torch.device("cuda", 0), "tetra", "scalar", 2, torch.float64) == 128
    assert autotune.lookup(torch.device("cpu"), "tetra", "scalar", 2, torch.float64) is None
    assert autotune.lookup(torch.device("cuda", 0), "tetra", "scalar", 2, None) is None
    assert autotune.lookup(torch.device("cuda", 0), "tetra", "scalar", 2, torch.float32) is None
    assert autotune.lookup(torch.device("cuda", 0), "tetra", "block", 2, torch.float64) is None


def test_cache_round_trip_merges(fake_gpu):
    path = fake_gpu
    path.write_text(json.dumps({"Other GPU|1sm|cc90|triangle|node|q2|float64": 64}))
    autotune.record("cuda", "tetra", "scalar", 2, torch.float64, 256)
    autotune.save()
    data = json.loads(path.read_text())
    assert data["Other GPU|1sm|cc90|triangle|node|q2|float64"] == 64
    assert data[f"{FAKE_TAG}|tetra|scalar|q2|float64"] == 256
    autotune.clear()                                     # a new process reads the file on first lookup
    assert autotune.lookup("cuda", "tetra", "scalar", 2, torch.float64) == 256
    path.write_text("not json")                          # an unreadable cache is ignored
    autotune.clear()
    assert autotune.lookup("cuda", "tetra", "scalar", 2, torch.float64) is None


def test_clear_forgets_memoised_keys(fake_gpu, monkeypatch):
    cuda = torch.device("cuda", 0)
    autotune.record(cuda, "tetra", "scalar", 2, torch.float64, 64)
    assert autotune.lookup(cuda, "tetra", "scalar", 2, torch.float64) == 64
    autotune.clear()
    monkeypatch.setattr(autotune, "device_tag", lambda device: "Another GPU|8sm|cc90")
    autotune.record(cuda, "tetra", "scalar", 2, torch.float64, 128)
    assert autotune.lookup(cuda, "tetra", "scalar", 2, torch.float64) == 128


def test_topology_uses_the_tuned_size(fake_gpu):
    m = gen_unit_cube(2)
    topo = Topology(m.points, m.elements(), "tetra", 2)
    cuda = torch.device("cuda", 0)
    assert topo.chunk_for("scalar", cuda, torch.float64) == chunk_elems("tetra", False, 2)
    assert topo.chunk_for("node", cuda, torch.float64) == NODE_CHUNK_ELEMS["tetra"]
    autotune.record(cuda, "tetra", "scalar", 2, torch.float64, 96)
    autotune.record(cuda, "tetra", "node", 2, torch.float64, 48)
    assert topo.chunk_for("scalar", cuda, torch.float64) == 96
    assert topo.chunk_for("node", cuda, torch.float64) == 48
    assert topo.chunk_for("block", cuda, torch.float64) == chunk_elems("tetra", True, 2)
    assert topo.chunk_for("scalar", cuda, torch.float32) == chunk_elems("tetra", False, 2)
    assert topo.chunk_for("scalar", torch.device("cpu"), torch.float64) == chunk_elems("tetra", False, 2)
