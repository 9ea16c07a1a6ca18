"""Elements-per-chunk autotuning for the assembly kernels.

A matrix or vector assembly launches one CTA per chunk of consecutive
(Morton-ordered) elements.  The chunk size sets a CTA's work and its shared
memory: element locals, the staged reduction plan and, for elements whose
Jacobian varies (P2, quadrilaterals), the per-quadrature-point geometry of
every element of the chunk (chunk x Q: the quadrature tile).  It also sets
how many targets two chunks share, which the finalize pass sums.
``tune_matrix`` and ``tune_vector`` time the real assembly call for every
candidate chunk size that fits (CUDA events on the current stream, median of
``repeats`` calls after a warm-up) and keep the fastest.

Results are keyed by (GPU name, SM count, compute capability, element type,
kind ("scalar" | "block" | "node"), quadrature order, dtype).  They are held
for the process and, with ``save=True``, merged into a JSON file
(``TM_AUTOTUNE_CACHE``, default ``~/.cache/tensormesh_gb300/autotune.json``)
that later processes read on their first lookup.  ``Topology`` asks
``lookup`` before it falls back to the static table of ``plan.py``.

The chunk size changes only the grouping of the fixed-order reduction:
values move at the rounding level from one chunk size to another and stay
bitwise reproducible for a given one.
"""
import json
import os
import statistics
import tempfile
from pathlib import Path
from typing import Dict, Iterable, List, Optional

import torch

from . import _lib
from .element import element_info

# chunk sizes tried (those that fit the element type and kind), besides the
# static default
CANDIDATES = (16, 32, 64, 128, 256, 384, 512, 768, 1024)

_table: Dict[str, int] = {}
_loaded = False
_tags: Dict[torch.device, str] = {}
_keys: Dict[tuple, str] = {}


def cache_path() -> Path:
    env = os.environ.get("TM_AUTOTUNE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "tensormesh_gb300" / "autotune.json"


def device_tag(device: torch.device) -> str:
    """GPU model, SM count and compute capability of a CUDA device."""
    if device not in _tags:
        p = torch.cuda.get_device_properties(device)
        _tags[device] = f"{p.name}|{p.multi_processor_count}sm|cc{p.major}{p.minor}"
    return _tags[device]


def make_key(tag: str, etype: str, kind: str, qorder: int, dtype: torch.dtype) -> str:
    if kind not in ("scalar", "block", "node"):
        raise ValueError(f"kind must be 'scalar', 'block' or 'node', got {kind!r}")
    return f"{tag}|{etype}|{kind}|q{int(qorder)}|{str(dtype).replace('torch.', '')}"


def _load():
    global _loaded
    if _loaded:
        return
    _loaded = True
    path = cache_path()
    try:
        with open(path) as fh:
            data = json.load(fh)
    except (OSError, ValueError):
        return
    for k, v in data.items():
        if isinstance(v, int) and v > 0 and _cached_size_fits(k, v):
            _table.setdefault(k, v)


def _cached_size_fits(key: str, chunk: int) -> bool:
    """A cached chunk size is used only if it still fits its element type,
    kind and quadrature order (16-bit contribution codes, shared memory): a
    stale or hand-edited entry is dropped, and the static default applies."""
    parts = key.split("|")
    if len(parts) < 5:
        return False
    etype, kind, q = parts[-4], parts[-3], parts[-2]
    try:
        qorder = int(q[1:]) if q.startswith("q") else None
        return qorder is not None and bool(candidates(etype, kind, qorder, [chunk]))
    except (KeyError, ValueError):
        return False


def save(path: Optional[Path] = None):
    """Merge the process's results into the JSON cache (atomic replace)."""
    path = Path(path) if path is not None else cache_path()
    data = {}
    try:
        with open(path) as fh:
            data = json.load(fh)
    except (OSError, ValueError):
        pass
    data.update(_table)
    path.parent.mkdir(parents=True, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=str(path.parent), prefix=".autotune.")
    with os.fdopen(fd, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def clear():
    """Forget every result of this process, and the device tags and keys
    built so far (the cache file is kept and is read again on the next
    lookup)."""
    global _loaded
    _table.clear()
    _tags.clear()
    _keys.clear()
    _loaded = False


def lookup(device, etype: str, kind: str, qorder: int, dtype: Optional[torch.dtype]) -> Optional[int]:
    """The tuned chunk size for a CUDA device, or None (every assembly call
    asks: the key of each argument tuple is built once)."""
    if dtype is None or device is None:
        return None
    args = (device, etype, kind, qorder, dtype)
    key = _keys.get(args)
    if key is None:
        dev = torch.device(device)
        if dev.type != "cuda":
            return None
        key = _keys[args] = make_key(device_tag(dev), etype, kind, qorder, dtype)
    if not _loaded:
        _load()
    return _table.get(key)


def record(device, etype: str, kind: str, qorder: int, dtype: torch.dtype, chunk: int):
    _load()
    _table[make_key(device_tag(torch.device(device)), etype, kind, qorder, dtype)] = int(chunk)


def candidates(etype: str, kind: str, qorder: int, sizes: Iterable[int] = CANDIDATES) -> List[int]:
    """Chunk sizes that fit: 16-bit contribution codes and the shared-memory
    estimate of the matrix kernel (``plan.chunk_fits``); a vector chunk holds
    its tables and chunk x B x 3 values."""
    from .plan import _CHUNK_SMEM_BUDGET, chunk_fits
    info = element_info(etype)
    out = []
    for ch in sorted(set(int(c) for c in sizes)):
        if kind == "node":
            ok = 1 <= ch and ch * info.n_basis * 2 <= 65536 and 8 * ch * info.n_basis * 3 <= _CHUNK_SMEM_BUDGET // 2
        else:
            ok = chunk_fits(etype, kind == "block", qorder, ch)
        if ok:
            out.append(ch)
    return out


def _time(fn, repeats: int) -> float:
    """Median milliseconds of ``fn`` over ``repeats`` calls after one warm-up,
    CUDA events on the current stream."""
    fn()
    stream = torch.cuda.current_stream()
    ts = []
    for _ in range(repeats):
        b, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b.record(stream)
        fn()
        e.record(stream)
        e.synchronize()
        ts.append(b.elapsed_time(e))
    return statistics.median(ts)


def _sweep(topo, key_args, plan_kind, run, sizes, repeats, save_result):
    dev, etype, kind, qorder, dtype = key_args
    tag_key = make_key(device_tag(dev), etype, kind, qorder, dtype)
    _load()
    previous = _table.pop(tag_key, None)
    default = topo.chunk_for(kind, dev, dtype)
    times: Dict[int, float] = {}
    try:
        for ch in candidates(etype, kind, qorder, list(sizes) + [default]):
            _table[tag_key] = ch
            try:
                times[ch] = _time(run, repeats)
            except _lib.TmError:
                continue                   # the launch refused the chunk (shared memory)
    finally:
        if previous is None:
            _table.pop(tag_key, None)
        else:
            _table[tag_key] = previous
    if not times:
        raise RuntimeError(f"no candidate chunk size ran for {tag_key}")
    best = min(times, key=lambda c: (times[c], c))
    _table[tag_key] = best
    # drop the device plans of candidates that lost and that no kind uses
    used = {topo.chunk_for(k, dev, dtype) for k in ("scalar", "block", "node")}
    for k in [k for k in topo._plans if k[0] == plan_kind and k[2] == dev and k[1] in times and k[1] not in used]:
        del topo._plans[k]
    if save_result:
        save()
    return best, times


def tune_matrix(assemblers, points: Optional[torch.Tensor] = None, element_data=None, scalar_data=None,
                sizes: Iterable[int] = CANDIDATES, repeats: int = 5, save: bool = False):
    """Time ``assemble_forms(assemblers, points, element_data, scalar_data)``
    for every candidate chunk size of its element type and kind, record the
    fastest for this GPU and dtype and return (chunk, {chunk: ms})."""
    from .assemble import assemble_forms
    first = assemblers[0]
    et = first.element_types[0]
    trans = first.transformation[et]
    pts = trans.points if points is None else points
    _lib.require_cuda(pts, "points")
    topo = first._topo(True)
    kind = "block" if any(a._tm_kind() == "elasticity" for a in assemblers) else "scalar"
    run = lambda: assemble_forms(assemblers, pts, element_data, scalar_data)
    return _sweep(topo, (pts.device, et, kind, topo.quadrature_order, pts.dtype), "matrix", run, sizes, repeats,
                  save)


def tune_vector(assembler, points: Optional[torch.Tensor] = None, point_data=None,
                sizes: Iterable[int] = CANDIDATES, repeats: int = 5, save: bool = False):
    """Time ``assembler(points, point_data=point_data)`` (a built-in
    NodeAssembler) for every candidate node chunk size, record the fastest
    and return (chunk, {chunk: ms})."""
    et = assembler.element_types[0]
    trans = assembler.transformation[et]
    pts = trans.points if points is None else points
    _lib.require_cuda(pts, "points")
    topo = assembler._topo(False)
    run = lambda: assembler(pts, point_data=point_data)
    return _sweep(topo, (pts.device, et, "node", topo.quadrature_order, pts.dtype), "node", run, sizes, repeats,
                  save)
