"""Mesh topology: CSR pattern, element->CSR slot map and the element-chunk
reduction plans, built once per mesh by the native plan builder
(``tm_plan_build``) and kept on the device.

``ElementAssembler.from_mesh`` (assemble/element_assembler.py:769-878)
computes the pattern and slot map on the host with SciPy on every mesh; here
the same arrays come from ``tm_plan_build`` together with the chunk plan the
fused kernels reduce with.  Elements are processed in Morton (Z-curve) order
of their centroids so that a chunk of consecutive elements is spatially
compact and most CSR targets are reduced inside one chunk.
"""
import ctypes as C
import os
from concurrent.futures import ThreadPoolExecutor
from typing import Dict, Optional

import numpy as np
import torch

from . import _lib, autotune
from .element import element_info, element_tables, packed_tables


def _host_threads() -> int:
    """TM_HOST_THREADS if set, else all hardware threads (at most 64), as
    the native plan builder counts them."""
    try:
        n = int(os.environ.get("TM_HOST_THREADS", "0"))
    except ValueError:
        n = 0
    if n <= 0:
        n = os.cpu_count() or 1
    return max(1, min(n, 64))


def morton_order(points: np.ndarray, conn: np.ndarray, groups: Optional[np.ndarray] = None) -> np.ndarray:
    """Processing order of the elements: increasing Morton code of the
    centroid of their vertices, ties in element order (``tm_morton_order``,
    on host threads).  With ``groups`` (``[G+1]`` element offsets from 0 to
    E) each group is ordered on its own (within its own bounding box) and
    the groups follow one another."""
    E = conn.shape[0]
    perm = np.zeros(E, dtype=np.int32)
    if groups is not None:
        g = np.asarray(groups, dtype=np.int64)
        if g.ndim != 1 or g.size < 1 or g[0] != 0 or g[-1] != E or (np.diff(g) < 0).any():
            raise ValueError("element groups must be non-decreasing offsets from 0 to the element count")
        pts = np.ascontiguousarray(points, dtype=np.float64)
        c64 = np.ascontiguousarray(conn, dtype=np.int64)

        def one(be):
            b, e = be
            perm[b:e] = morton_order(pts, c64[b:e]) + np.int32(b)

        spans = [(int(b), int(e)) for b, e in zip(g[:-1], g[1:]) if e > b]
        # groups on host threads (the native call releases the interpreter lock)
        workers = min(len(spans), _host_threads())
        if workers > 1 and E >= 1 << 16:
            with ThreadPoolExecutor(max_workers=workers) as pool:
                list(pool.map(one, spans))
        else:
            for be in spans:
                one(be)
        return perm
    if E == 0:
        return perm
    pts = np.ascontiguousarray(points, dtype=np.float64)
    c64 = np.ascontiguousarray(conn, dtype=np.int64)
    _lib.check(_lib.load().tm_morton_order(pts.ctypes.data, pts.shape[0], pts.shape[1], c64.ctypes.data, E,
                                           c64.shape[1], perm.ctypes.data), "tm_morton_order")
    return perm


def device_pattern(conn: torch.Tensor, n_points: int):
    """CSR pattern and slot map of a connectivity on the GPU
    (``tm_pattern_count`` / ``tm_pattern_fill``): (edges int32 [2, nnz],
    slot int64 [E*B*B], row_ptr int64 [N+1]), all on conn's device, equal to
    the reference's ``from_mesh`` arrays."""
    _lib.require_cuda(conn, "conn")
    lib = _lib.load()
    dev = conn.device
    c = conn.to(torch.int32).contiguous()
    E, B = int(c.shape[0]), int(c.shape[1])
    ws = torch.empty(max(1, lib.tm_pattern_workspace_bytes(E, B, n_points)), dtype=torch.uint8, device=dev)
    row_ptr = torch.empty(n_points + 1, dtype=torch.int64, device=dev)
    nnz = C.c_int64(0)
    st = _lib.stream_handle(dev)
    _lib.check(lib.tm_pattern_count(_lib.ptr(c), E, B, n_points, _lib.ptr(ws), _lib.ptr(row_ptr), C.byref(nnz), st),
               "tm_pattern_count")
    edges = torch.empty(2, nnz.value, dtype=torch.int32, device=dev)
    slot = torch.empty(E * B * B, dtype=torch.int64, device=dev)
    _lib.check(lib.tm_pattern_fill(_lib.ptr(c), E, B, n_points, _lib.ptr(ws), _lib.ptr(row_ptr), _lib.ptr(edges[0]),
                                   _lib.ptr(edges[1]), _lib.ptr(slot), st), "tm_pattern_fill")
    return edges, slot, row_ptr


def device_morton_order(points: torch.Tensor, conn: torch.Tensor, groups: Optional[np.ndarray] = None) -> torch.Tensor:
    """``morton_order`` on the GPU (``tm_morton_order_device``): the same
    permutation, as a device int32 tensor."""
    lib = _lib.load()
    dev = conn.device
    c = conn.to(torch.int32).contiguous()
    E, B = int(c.shape[0]), int(c.shape[1])
    pts = points.detach().to(device=dev, dtype=torch.float64).contiguous()
    D = int(pts.shape[1])
    perm = torch.empty(E, dtype=torch.int32, device=dev)
    if E == 0:
        return perm
    g = None if groups is None else torch.as_tensor(np.asarray(groups, dtype=np.int64)).to(dev)
    G = 1 if g is None else int(g.shape[0]) - 1
    if g is not None and (G < 1 or int(groups[0]) != 0 or int(groups[-1]) != E or (np.diff(groups) < 0).any()):
        raise ValueError("element groups must be non-decreasing offsets from 0 to the element count")
    ws = torch.empty(max(1, lib.tm_morton_workspace_bytes(E, D, G)), dtype=torch.uint8, device=dev)
    _lib.check(lib.tm_morton_order_device(_lib.ptr(pts), int(pts.shape[0]), D, _lib.ptr(c), E, B, _lib.ptr(g), G,
                                          _lib.ptr(ws), _lib.ptr(perm), _lib.stream_handle(dev)),
               "tm_morton_order_device")
    return perm


def device_chunk_plan(conn: torch.Tensor, perm: torch.Tensor, n_points: int, kind: int, chunk_elems: int,
                      slot: Optional[torch.Tensor] = None, nnz: int = 0) -> "DevicePlan":
    """``tm_plan_build``'s chunk plan built on the GPU (``tm_chunk_plan_device``)
    from device conn (element order), perm and, for matrix plans, the device
    slot map: the same arrays, kept on the device."""
    lib = _lib.load()
    dev = conn.device
    c = conn.to(torch.int32).contiguous()
    E, B = int(c.shape[0]), int(c.shape[1])
    matrix = kind == _lib.TM_PLAN_KIND_MATRIX
    NL = B * (B + 1) // 2 if matrix else B
    n_targets = nnz if matrix else n_points
    n_chunks = (E + chunk_elems - 1) // chunk_elems
    cap_slots, cap_contrib, cap_shared = E * NL, (2 * E * NL if matrix else E * NL), max(1, n_targets)
    i32 = lambda n: torch.empty(max(1, n), dtype=torch.int32, device=dev)
    arrays = {"conn": i32(E * B), "chunk_begin": i32(n_chunks + 1), "chunk_contrib": i32(n_chunks + 1),
              "slot_ptr": i32(cap_slots + 1), "contrib": torch.empty(max(1, cap_contrib), dtype=torch.int16, device=dev),
              "slot_target": i32(cap_slots), "slot_mirror": i32(cap_slots), "shared_ptr": i32(cap_shared + 1),
              "shared_target": i32(cap_shared), "shared_mirror": i32(cap_shared)}
    out = _lib.DeviceChunkPlan()
    for k, v in arrays.items():
        setattr(out, k, _lib.ptr(v))
    out.cap_slots, out.cap_contrib, out.cap_shared = cap_slots, cap_contrib, cap_shared
    ws = torch.empty(max(1, lib.tm_chunk_plan_device_workspace_bytes(E, B, n_targets, kind, chunk_elems)),
                     dtype=torch.uint8, device=dev)
    _lib.check(lib.tm_chunk_plan_device(_lib.ptr(c), E, B, n_points, kind, chunk_elems, _lib.ptr(perm), _lib.ptr(slot),
                                        nnz, _lib.ptr(ws), C.byref(out), _lib.stream_handle(dev)),
               "tm_chunk_plan_device")
    del ws
    ns, nc, nsh = int(out.n_slots), int(out.n_contrib), int(out.n_shared)
    # exact sizes; the arrays staged by bulk copies keep 16 zero bytes past their end
    pad = lambda x, n: torch.cat([x[:n], torch.zeros(16 // x.element_size(), dtype=x.dtype, device=dev)])
    sizes = {"n_elements": E, "n_basis": B, "n_local": NL, "chunk_elems": chunk_elems, "n_chunks": int(out.n_chunks),
             "n_targets": n_targets, "n_shared": nsh, "n_partials": int(out.n_partials), "n_chunk_slots": ns,
             "n_contrib": nc, "max_chunk_slots": int(out.max_chunk_slots),
             "max_chunk_contrib": int(out.max_chunk_contrib)}
    dev_arrays = {"elem_perm": perm.to(torch.int32).contiguous(), "conn": arrays["conn"][:E * B],
                  "chunk_begin": arrays["chunk_begin"][:n_chunks + 1],
                  "chunk_contrib": arrays["chunk_contrib"][:n_chunks + 1],
                  "slot_ptr": pad(arrays["slot_ptr"], ns + 1), "contrib": pad(arrays["contrib"], nc),
                  "slot_target": arrays["slot_target"][:ns].clone(), "slot_mirror": arrays["slot_mirror"][:ns].clone(),
                  "shared_ptr": arrays["shared_ptr"][:nsh + 1].clone(),
                  "shared_target": arrays["shared_target"][:nsh].clone(),
                  "shared_mirror": arrays["shared_mirror"][:nsh].clone()}
    return DevicePlan.from_device(dev_arrays, sizes, dev)


class HostPlan:
    """Arrays of one ``tm_plan_build`` call, as numpy arrays."""

    _DTYPES = {
        _lib.PLAN_EDGE_ROW: np.int32, _lib.PLAN_EDGE_COL: np.int32, _lib.PLAN_SLOT: np.int64,
        _lib.PLAN_CHUNK_BEGIN: np.int32, _lib.PLAN_SLOT_PTR: np.int32, _lib.PLAN_CONTRIB: np.uint16,
        _lib.PLAN_SLOT_TARGET: np.int32, _lib.PLAN_SLOT_MIRROR: np.int32,
        _lib.PLAN_SHARED_PTR: np.int32, _lib.PLAN_SHARED_TARGET: np.int32,
        _lib.PLAN_SHARED_MIRROR: np.int32, _lib.PLAN_CONN: np.int32, _lib.PLAN_PERM: np.int32,
        _lib.PLAN_CHUNK_CONTRIB: np.int32,
    }
    _NAMES = {
        _lib.PLAN_EDGE_ROW: "edge_row", _lib.PLAN_EDGE_COL: "edge_col", _lib.PLAN_SLOT: "slot",
        _lib.PLAN_CHUNK_BEGIN: "chunk_begin", _lib.PLAN_SLOT_PTR: "slot_ptr",
        _lib.PLAN_CONTRIB: "contrib", _lib.PLAN_SLOT_TARGET: "slot_target",
        _lib.PLAN_SLOT_MIRROR: "slot_mirror", _lib.PLAN_SHARED_PTR: "shared_ptr",
        _lib.PLAN_SHARED_TARGET: "shared_target", _lib.PLAN_SHARED_MIRROR: "shared_mirror",
        _lib.PLAN_CONN: "conn", _lib.PLAN_PERM: "perm", _lib.PLAN_CHUNK_CONTRIB: "chunk_contrib",
    }

    def __init__(self, conn: np.ndarray, n_points: int, kind: int, chunk_elems: int,
                 perm: Optional[np.ndarray] = None, slot_map: Optional[np.ndarray] = None):
        lib = _lib.load()
        conn = np.ascontiguousarray(conn, dtype=np.int64)
        E, B = conn.shape
        perm_c = None if perm is None else np.ascontiguousarray(perm, dtype=np.int32)
        slot_c = None if slot_map is None else np.ascontiguousarray(slot_map, dtype=np.int64)
        handle = C.c_void_p()
        st = lib.tm_plan_build(conn.ctypes.data if E else None, E, B, n_points, kind, chunk_elems,
                               None if perm_c is None else perm_c.ctypes.data,
                               None if slot_c is None else slot_c.ctypes.data, C.byref(handle))
        _lib.check(st, "tm_plan_build")
        try:
            self.arrays: Dict[str, np.ndarray] = {}
            for aid, dt in self._DTYPES.items():
                n = lib.tm_plan_array_size(handle, aid)
                arr = np.empty(n, dtype=dt)
                if n:
                    _lib.check(lib.tm_plan_copy_array(handle, aid, arr.ctypes.data), "tm_plan_copy_array")
                self.arrays[self._NAMES[aid]] = arr
            self.nnz = lib.tm_plan_scalar(handle, 0)
            self.n_chunks = lib.tm_plan_scalar(handle, 1)
            self.n_chunk_slots = lib.tm_plan_scalar(handle, 2)
            self.n_contrib = lib.tm_plan_scalar(handle, 3)
            self.n_shared = lib.tm_plan_scalar(handle, 4)
            self.n_partials = lib.tm_plan_scalar(handle, 5)
            self.n_local = lib.tm_plan_scalar(handle, 6)
            self.max_chunk_slots = lib.tm_plan_scalar(handle, 7)
            self.max_chunk_contrib = lib.tm_plan_scalar(handle, 8)
        finally:
            lib.tm_plan_free(handle)
        self.kind, self.n_elements, self.n_basis, self.n_points = kind, E, B, n_points
        self.chunk_elems = chunk_elems


class DevicePlan:
    """A chunk plan on the device plus its ``tm_chunk_plan`` view."""

    _ARRAYS = ("elem_perm", "conn", "chunk_begin", "slot_ptr", "contrib", "slot_target", "slot_mirror",
               "shared_ptr", "shared_target", "shared_mirror", "chunk_contrib")

    def __init__(self, host: HostPlan, device: torch.device):
        a = host.arrays
        t = lambda x: torch.from_numpy(x).to(device)
        # arrays the assembly kernel stages with bulk copies: 16 bytes of
        # zeros past the end keep every 16-byte window readable
        tp = lambda x: torch.from_numpy(np.concatenate([x, np.zeros(16 // x.itemsize, x.dtype)])).to(device)
        self.elem_perm = t(a["perm"])
        self.conn = t(a["conn"])
        self.chunk_begin = t(a["chunk_begin"])
        self.chunk_contrib = t(a["chunk_contrib"])
        self.slot_ptr = tp(a["slot_ptr"])
        self.contrib = tp(a["contrib"].view(np.int16))   # uint16 bits
        self.slot_target = t(a["slot_target"])
        self.slot_mirror = t(a["slot_mirror"])
        self.shared_ptr = t(a["shared_ptr"])
        self.shared_target = t(a["shared_target"])
        self.shared_mirror = t(a["shared_mirror"])
        self.n_elements, self.n_basis, self.n_local = host.n_elements, host.n_basis, host.n_local
        self.chunk_elems, self.n_chunks = host.chunk_elems, host.n_chunks
        self.n_targets = host.nnz if host.kind == _lib.TM_PLAN_KIND_MATRIX else host.n_points
        self.n_shared, self.n_partials = host.n_shared, host.n_partials
        self.n_chunk_slots, self.n_contrib = host.n_chunk_slots, host.n_contrib
        self.max_chunk_slots, self.max_chunk_contrib = host.max_chunk_slots, host.max_chunk_contrib
        self.device = device

    @classmethod
    def from_device(cls, arrays: Dict[str, torch.Tensor], sizes: Dict[str, int], device: torch.device) -> "DevicePlan":
        """A plan whose arrays were built on the device (``device_chunk_plan``)."""
        p = cls.__new__(cls)
        for k, v in arrays.items():
            setattr(p, k, v)
        for k, v in sizes.items():
            setattr(p, k, v)
        p.device = device
        return p

    def struct(self) -> _lib.ChunkPlan:
        if getattr(self, "_struct", None) is not None:
            return self._struct
        p = _lib.ChunkPlan()
        p.n_elements, p.n_basis, p.n_local = self.n_elements, self.n_basis, self.n_local
        p.chunk_elems, p.n_chunks, p.n_targets = self.chunk_elems, self.n_chunks, self.n_targets
        p.n_shared, p.n_partials = self.n_shared, self.n_partials
        p.max_chunk_slots, p.max_chunk_contrib = self.max_chunk_slots, self.max_chunk_contrib
        for name in self._ARRAYS:
            setattr(p, name, _lib.ptr(getattr(self, name)))
        self._struct = p
        return p

    def nbytes(self) -> int:
        return sum(getattr(self, n).numel() * getattr(self, n).element_size() for n in self._ARRAYS)


# chunk sizes (elements per CTA) by element type and whether the form is a
# DxD block form; chosen so that the locals of a chunk fit in shared memory
CHUNK_ELEMS = {
    ("triangle", False): 768, ("triangle", True): 256,
    ("tetra", False): 768, ("tetra", True): 128,
    ("triangle6", False): 64, ("triangle6", True): 64,
    ("tetra10", False): 32, ("tetra10", True): 32,
    ("quad", False): 128, ("quad", True): 128,
    ("quad9", False): 64, ("quad9", True): 64,
}
NODE_CHUNK_ELEMS = {"triangle": 256, "tetra": 256, "triangle6": 128, "tetra10": 128, "quad": 256, "quad9": 128}

# shared memory a k_matrix chunk may fill (of the 227 KB a CTA can have)
_CHUNK_SMEM_BUDGET = 200 * 1024


def chunk_fits(etype: str, block: bool, qorder: int, ch: int) -> bool:
    """Whether a k_matrix chunk of ``ch`` elements fits: contribution codes
    are 16-bit (ch * n_local * 2 <= 65536), and for elements whose Jacobian
    varies (P2, quadrilaterals), which keep the shape gradients of every
    quadrature point in shared memory, the estimate of the kernel's layout
    (tables, coordinates, gradients and weights per point, locals, staged
    plan) stays within the budget.  P1 chunks hold their locals and |det|
    rho as 8-byte values and their share of the staged plan (about two
    slots and NL 2-byte contributions per element)."""
    info = element_info(etype)
    B, D = info.n_basis, info.dim
    NL = B * (B + 1) // 2
    if ch < 1 or ch * NL * 2 > 65536:
        return False
    if etype in ("triangle", "tetra"):
        return 64 + ch * (8 * NL + 8 + 4 * 3 + 2 * NL) <= _CHUNK_SMEM_BUDGET
    Q = len(element_tables(etype, qorder)["w"])
    # tables, mass template and their double-float copies
    fixed = 8 * (Q + Q * B + Q * D * B + B * B + B + 1) + 16 * NL + 8 * Q * (D * B + 1 + B) + 64
    # per element: coordinates, gradients and weights per quadrature point,
    # 16 bytes of scale exponents, then two moduli (elasticity, whose blocks
    # are formed during the reduction) or one value per local pair and form
    per = 8 * (B * D + Q * B * D + Q) + 16 + (16 if block else 16 * NL) + 6 * B * B
    return fixed + ch * per <= _CHUNK_SMEM_BUDGET


def chunk_elems(etype: str, block: bool, qorder: int) -> int:
    """Elements per k_matrix chunk: the default of ``CHUNK_ELEMS``, halved
    while the chunk does not fit (``chunk_fits``): high quadrature orders of
    P2 and quadrilateral elements need smaller chunks."""
    ch = CHUNK_ELEMS[(etype, block)]
    while ch > 8 and not chunk_fits(etype, block, qorder, ch):
        ch //= 2
    return ch


class Topology:
    """Everything about one mesh (one element type) that does not change
    between calls: connectivity, pattern, slot map, tables, chunk plans."""

    def __init__(self, points: torch.Tensor, conn: torch.Tensor, etype: str, quadrature_order: int,
                 matrix: bool = True, element_groups: Optional[np.ndarray] = None):
        info = element_info(etype)
        self.etype, self.info, self.quadrature_order = etype, info, quadrature_order
        self.n_points = int(points.shape[0])
        self.n_elements = int(conn.shape[0])
        # int64 connectivity as numpy, always a private copy: plans for other
        # chunk sizes and kinds are built from it later, and must match the
        # pattern and slot map even if the caller edits its cells in place
        conn_np = np.array(conn.detach().to("cpu", torch.int64).contiguous().numpy(), copy=True)
        # a mesh on the GPU is ordered, patterned and planned on the GPU
        self._dev = conn.device if (conn.is_cuda and self.n_elements > 0) else None
        if self._dev is not None:
            self._conn_dev = conn.detach().to(torch.int32).contiguous().clone()
            self._perm_dev = device_morton_order(points, self._conn_dev, element_groups)
            self.perm = self._perm_dev.cpu().numpy()   # host copy, for plans the host builds
        else:
            pts_np = points.detach().cpu().to(torch.float64).numpy()
            self.perm = morton_order(pts_np, conn_np, element_groups)
        self._conn_np = conn_np
        self._plans: Dict[tuple, DevicePlan] = {}
        self._host_node: Optional[HostPlan] = None
        self._tables: Dict[torch.device, torch.Tensor] = {}
        self._conn32: Dict[torch.device, torch.Tensor] = {}
        self.edges = None
        self.slot = None
        self._layout_hash = None
        self._row_ptr: Dict[torch.device, torch.Tensor] = {}
        if matrix:
            ch = chunk_elems(etype, False, quadrature_order)
            if self._dev is not None:
                # pattern and slot map on the GPU (tm_pattern_*); chunk
                # plans follow on the GPU from that slot map, per chunk size
                edges, slot, row_ptr = device_pattern(self._conn_dev, self.n_points)
                self._row_ptr[conn.device] = row_ptr
                self._slot_dev = slot
                self.edges, self.slot = edges.cpu(), slot.cpu()
                self.nnz = int(self.edges.shape[1])
                self._pending = {}
            else:
                host = HostPlan(conn_np, self.n_points, _lib.TM_PLAN_KIND_MATRIX, ch, self.perm)
                self.edges = torch.from_numpy(np.stack([host.arrays["edge_row"], host.arrays["edge_col"]]))
                self.slot = torch.from_numpy(host.arrays["slot"])
                self.nnz = int(host.nnz)
                self._pending = {("matrix", ch): host}
        else:
            self.nnz = 0
            self._pending = {}

    # -- device objects -------------------------------------------------------
    def tables(self, device: torch.device) -> torch.Tensor:
        if device not in self._tables:
            self._tables[device] = torch.from_numpy(packed_tables(self.etype, self.quadrature_order)).to(device)
        return self._tables[device]

    def table_struct(self, device: torch.device) -> _lib.ElementTables:
        cache = self.__dict__.setdefault("_table_structs", {})
        if device not in cache:
            t = _lib.ElementTables()
            t.element_type = self.info.code
            t.n_quad = len(element_tables(self.etype, self.quadrature_order)["w"])
            t.packed = _lib.ptr(self.tables(device))
            cache[device] = t
        return cache[device]

    def conn32(self, device: torch.device) -> torch.Tensor:
        if device not in self._conn32:
            self._conn32[device] = torch.from_numpy(self._conn_np.astype(np.int32)).to(device)
        return self._conn32[device]

    def chunk_for(self, kind: str, device: torch.device, dtype: Optional[torch.dtype] = None) -> int:
        """Elements per chunk for kind "scalar", "block" (matrix forms) or
        "node": the autotuned size for this GPU and dtype when one is
        recorded, else the static default."""
        tuned = autotune.lookup(device, self.etype, kind, self.quadrature_order, dtype)
        if tuned is not None:
            return tuned
        static = self.__dict__.setdefault("_static_chunk", {})
        if kind not in static:
            static[kind] = (NODE_CHUNK_ELEMS[self.etype] if kind == "node"
                            else chunk_elems(self.etype, kind == "block", self.quadrature_order))
        return static[kind]

    def matrix_plan(self, device: torch.device, block: bool = False,
                    dtype: Optional[torch.dtype] = None) -> DevicePlan:
        ch = self.chunk_for("block" if block else "scalar", device, dtype)
        key = ("matrix", ch, device)
        if key not in self._plans:
            plan = self._device_plan(device, _lib.TM_PLAN_KIND_MATRIX, ch)
            if plan is None:
                host = self._pending.pop(("matrix", ch), None)
                if host is None:
                    host = HostPlan(self._conn_np, self.n_points, _lib.TM_PLAN_KIND_MATRIX, ch, self.perm,
                                    slot_map=self.slot.numpy())
                plan = DevicePlan(host, device)
            self._plans[key] = plan
        return self._plans[key]

    def _device_plan(self, device: torch.device, kind: int, ch: int) -> Optional[DevicePlan]:
        """The chunk plan built on the GPU, for a mesh that lives on this
        device; None where the device builder does not apply (another device,
        chunks above 1024 elements or 8192 contributions), and the host
        builder takes over."""
        if self._dev is None or torch.device(device) != self._dev or ch > 1024:
            return None
        try:
            if kind == _lib.TM_PLAN_KIND_MATRIX:
                return device_chunk_plan(self._conn_dev, self._perm_dev, self.n_points, kind, ch, self._slot_dev,
                                         self.nnz)
            return device_chunk_plan(self._conn_dev, self._perm_dev, self.n_points, kind, ch)
        except _lib.TmError as err:
            if getattr(err, "status", None) == _lib.TM_ERR_TOO_LARGE:
                return None
            raise

    def node_plan(self, device: torch.device, dtype: Optional[torch.dtype] = None) -> DevicePlan:
        ch = self.chunk_for("node", device, dtype)
        key = ("node", ch, device)
        if key not in self._plans:
            plan = self._device_plan(device, _lib.TM_PLAN_KIND_NODE, ch)
            if plan is None:
                plan = DevicePlan(HostPlan(self._conn_np, self.n_points, _lib.TM_PLAN_KIND_NODE, ch, self.perm), device)
            self._plans[key] = plan
        return self._plans[key]

    def row_ptr(self, device: torch.device) -> torch.Tensor:
        """CSR row pointer of the (row-major sorted) pattern."""
        if device not in self._row_ptr:
            counts = np.bincount(self.edges[0].numpy(), minlength=self.n_points)
            rp = np.zeros(self.n_points + 1, dtype=np.int64)
            np.cumsum(counts, out=rp[1:])
            self._row_ptr[device] = torch.from_numpy(rp).to(device)
        return self._row_ptr[device]

    @property
    def layout_hash(self) -> str:
        """SHA-256 of the int32 row bytes followed by the int32 column bytes,
        the value ``SparseMatrix.__init__`` computes (sparse/matrix.py:82-86)."""
        if self._layout_hash is None:
            import hashlib
            self._layout_hash = hashlib.sha256(self.edges[0].numpy().tobytes()
                                               + self.edges[1].numpy().tobytes()).hexdigest()
        return self._layout_hash

    def block_layout_hash(self, H: int) -> str:
        """layout_hash of the (N*H, N*H) block matrix on this pattern (its
        expanded int64 scalar rows and columns), computed once per H."""
        cache = self.__dict__.setdefault("_block_hashes", {})
        if H not in cache:
            from .sparse import block_layout_hash
            cache[H] = block_layout_hash(self.edges[0], self.edges[1], H)
        return cache[H]


class MixedTopology:
    """A mesh with several element types: one ``Topology`` per type (its own
    pattern, plans and kernels) and the union pattern the assembled matrix
    lives on.

    The union pattern is the set of distinct (row, col) pairs over all types,
    sorted row-major (int32 ``edges``), as ``ElementAssembler.from_mesh``
    builds it from every type's local pairs (element_assembler.py:811-830).
    ``maps[t]`` sends type t's own CSR positions into the union, so that the
    union slot map of type t is ``maps[t][slot_t]``.  A matrix assembled per
    type is combined by one deterministic gather-sum (``tm_project_reduce``)
    whose segments list, for every union position, the contributing
    positions of the types in type order: the sum over types runs in the
    order of the mesh's element types, as the reference sums its projectors."""

    def __init__(self, points: torch.Tensor, elements: Dict[str, torch.Tensor], quadrature_order: int,
                 matrix: bool = True):
        self.n_points = int(points.shape[0])
        self.quadrature_order = quadrature_order
        self.types = list(elements.keys())
        self.topos: Dict[str, Topology] = {
            et: Topology(points, conn, et, quadrature_order, matrix=matrix) for et, conn in elements.items()}
        self.n_elements = {et: t.n_elements for et, t in self.topos.items()}
        self._row_ptr: Dict[torch.device, torch.Tensor] = {}
        self._seg: Dict[tuple, tuple] = {}
        self._layout_hash = None
        self.edges = None
        if not matrix:
            self.nnz = 0
            return
        N = np.int64(self.n_points)
        keys = {et: t.edges[0].numpy().astype(np.int64) * N + t.edges[1].numpy().astype(np.int64)
                for et, t in self.topos.items()}
        union = np.unique(np.concatenate(list(keys.values())))
        self.nnz = int(union.shape[0])
        self.edges = torch.from_numpy(np.stack([(union // N).astype(np.int32), (union % N).astype(np.int32)]))
        self.maps = {et: np.searchsorted(union, k).astype(np.int64) for et, k in keys.items()}
        self.slot = {et: torch.from_numpy(self.maps[et][t.slot.numpy()]) for et, t in self.topos.items()}

    def segments(self, device: torch.device, kind: str) -> tuple:
        """(seg_ptr, src) of the combine: "matrix" over the union pattern
        (sources: the types' CSR values, concatenated in type order),
        "node" over the nodes (sources: the types' nodal vectors)."""
        key = (kind, device)
        if key not in self._seg:
            if kind == "matrix":
                tgt = np.concatenate([self.maps[et] for et in self.types])
                n_to = self.nnz
            else:
                tgt = np.tile(np.arange(self.n_points, dtype=np.int64), len(self.types))
                n_to = self.n_points
            src = np.argsort(tgt, kind="stable").astype(np.int64)     # type order within a target
            seg = np.zeros(n_to + 1, dtype=np.int64)
            np.cumsum(np.bincount(tgt, minlength=n_to), out=seg[1:])
            self._seg[key] = (torch.from_numpy(seg).to(device), torch.from_numpy(src).to(device))
        return self._seg[key]

    def map_tensor(self, et: str, device: torch.device) -> torch.Tensor:
        """``maps[et]`` (type et's CSR positions -> union positions) on a device."""
        key = ("map", et, device)
        if key not in self._seg:
            self._seg[key] = torch.from_numpy(self.maps[et]).to(device)
        return self._seg[key]

    def row_ptr(self, device: torch.device) -> torch.Tensor:
        """CSR row pointer of the union pattern."""
        if device not in self._row_ptr:
            counts = np.bincount(self.edges[0].numpy(), minlength=self.n_points)
            rp = np.zeros(self.n_points + 1, dtype=np.int64)
            np.cumsum(counts, out=rp[1:])
            self._row_ptr[device] = torch.from_numpy(rp).to(device)
        return self._row_ptr[device]

    @property
    def layout_hash(self) -> str:
        """SHA-256 of the union pattern's int32 rows then columns
        (sparse/matrix.py:82-86)."""
        if self._layout_hash is None:
            import hashlib
            self._layout_hash = hashlib.sha256(self.edges[0].numpy().tobytes()
                                               + self.edges[1].numpy().tobytes()).hexdigest()
        return self._layout_hash

    def block_layout_hash(self, H: int) -> str:
        cache = self.__dict__.setdefault("_block_hashes", {})
        if H not in cache:
            from .sparse import block_layout_hash
            cache[H] = block_layout_hash(self.edges[0], self.edges[1], H)
        return cache[H]
