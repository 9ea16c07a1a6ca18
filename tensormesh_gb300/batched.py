"""Batched assembly and solve of many diffusion problems on meshes of
uneven size (one element type per batch: any type the assemblers take).

The reference handles a set of different meshes by looping: build the mesh,
``from_mesh``, assemble, condense, solve, one mesh after another
(docs/source/user_guide/batched_workflows.rst:247-249).  ``BatchedDiffusion``
concatenates the meshes with node and element offsets into one
block-diagonal problem: one chunk plan covers every mesh, so a single
``k_matrix`` launch assembles all stiffness matrices, a single ``k_vector``
launch all load vectors, and a single ``tm_batched_pcg`` launch solves every
system (Dirichlet nodes masked, no extraction of the condensed blocks).
``capture()`` records the three launches in one CUDA graph; ``replay()``
copies new coefficients and sources into its static buffers and runs it.
With ``autotune=True`` the elements per chunk of the stiffness and load
launches are timed over the candidate sizes on the batch itself
(``autotune.tune_matrix`` / ``tune_vector``) before anything is captured;
``chunks`` holds the sizes used.

``precision="mixed"`` (float64 batches) solves by mixed-precision iterative
refinement instead (``tm_batched_pcg_mixed``): float64 residuals and
corrections around float32 Jacobi-PCG inner solves, to the same test on the
true float64 residual, ||b - A x|| <= rtol ||b||.  GB300 runs float64 at
1/64 of the float32 rate, and the float64 PCG of a system is bound by it.
"""
import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from .mesh import Mesh


@dataclass
class BatchStatus:
    iterations: torch.Tensor          # [n_systems] int32
    flag: torch.Tensor                # [n_systems] int32 (1 converged, 2 max_iter, 3 breakdown)
    relative_residual: torch.Tensor   # [n_systems] float64

    @property
    def all_converged(self) -> bool:
        return bool((self.flag == _lib.TM_PCG_CONVERGED).all())


class BatchedDiffusion:
    """K_m(kappa_m) u_m = b_m(f_m) with zero Dirichlet data on each mesh's
    boundary, for a list of meshes of one element type."""

    def __init__(self, meshes: Sequence[Mesh], quadrature_order: int = 2,
                 device: Optional[torch.device] = None, dtype: torch.dtype = torch.float64,
                 autotune: bool = False):
        from .builtin import LaplaceElementAssembler, LoadNodeAssembler
        from .element import element_info
        types = {m.default_element_type for m in meshes}
        if len(types) != 1:
            raise NotImplementedError("a batch holds meshes of one element type")
        element_info(next(iter(types)))             # raises for a type the assemblers do not take
        etype = next(iter(types))
        dev = torch.device(device) if device is not None else meshes[0].device
        self.n_systems = len(meshes)
        self.node_offset = np.zeros(self.n_systems + 1, dtype=np.int64)
        self.elem_offset = np.zeros(self.n_systems + 1, dtype=np.int64)
        np.cumsum([m.n_points for m in meshes], out=self.node_offset[1:])
        np.cumsum([m.n_elements for m in meshes], out=self.elem_offset[1:])
        # concatenated where the meshes live (on the GPU the order, pattern
        # and plans are then built there too)
        src = meshes[0].device
        pts = torch.cat([m.points.detach().to(src, dtype) for m in meshes])
        conn = torch.cat([m.elements().to(src).long() + int(self.node_offset[i]) for i, m in enumerate(meshes)])
        bnd = torch.cat([m.boundary_mask.to(src).bool() for m in meshes])
        # one element group per mesh: the meshes overlap in space, and one
        # order over all of them would mix meshes in every chunk
        self.mesh = Mesh(pts, {etype: conn}, {"is_boundary": bnd}, element_groups=self.elem_offset).to(dev)
        self.K_asm = LaplaceElementAssembler.from_mesh(self.mesh, quadrature_order)
        self.b_asm = LoadNodeAssembler.from_mesh(self.mesh, quadrature_order)
        self.device, self.dtype = dev, dtype
        self.system_offset = torch.from_numpy(self.node_offset).to(dev)
        # the solver's queue takes the largest systems first
        sizes = np.diff(self.node_offset)
        self.order = torch.from_numpy(np.argsort(-sizes, kind="stable").astype(np.int32)).to(dev)
        self.dirichlet = bnd.to(dev).to(torch.uint8)
        self._graph = None
        self._values32 = None
        if autotune:
            from . import autotune as tuner
            pts = self.mesh.points.to(dtype)
            ones = torch.ones(self.n_elements, dtype=dtype, device=dev)
            zeros = torch.zeros(self.n_points, dtype=dtype, device=dev)
            tuner.tune_matrix([self.K_asm], pts, {"kappa": ones})
            tuner.tune_vector(self.b_asm, pts, {"f": zeros})
        topo = self.K_asm._topo(True)
        self.chunks = {"matrix": topo.chunk_for("scalar", dev, dtype),
                       "node": self.b_asm._topo(False).chunk_for("node", dev, dtype)}
        # the plans of those chunk sizes, built now (on the GPU for device meshes)
        topo.matrix_plan(dev, dtype=dtype)
        self.b_asm._topo(False).node_plan(dev, dtype=dtype)

    @property
    def n_points(self) -> int:
        return self.mesh.n_points

    @property
    def n_elements(self) -> int:
        return self.mesh.n_elements

    def split(self, x: torch.Tensor) -> List[torch.Tensor]:
        return [x[int(self.node_offset[i]):int(self.node_offset[i + 1])] for i in range(self.n_systems)]

    # ------------------------------------------------------------------
    def _solve_into(self, kappa: torch.Tensor, f: torch.Tensor, x: torch.Tensor, work: torch.Tensor,
                    queue: torch.Tensor, status: torch.Tensor, rtol: float, max_iter: int,
                    precision: str = "float64", inner_rtol: float = 1e-4, max_outer: int = 30):
        from .assemble import assemble_forms
        lib = _lib.load()
        (values,) = assemble_forms([self.K_asm], self.mesh.points, {"kappa": kappa})
        b = self.b_asm(self.mesh.points, point_data={"f": f})
        K = self.K_asm._build_output(values)
        rp, col, perm, H = K._csr_structure()
        op = _lib.LinearOperator()
        op.dtype = _lib.dtype_code(values.dtype)
        op.block = 1
        op.n_rows = self.n_points
        op.row_ptr, op.col, op.values = _lib.ptr(rp), _lib.ptr(col), _lib.ptr(values)
        a = _lib.BatchedPcgArgs()
        a.n_systems = self.n_systems
        a.max_iter = int(max_iter)
        a.rtol = float(rtol)
        a.system_offset = _lib.ptr(self.system_offset)
        a.A = op
        a.dirichlet = _lib.ptr(self.dirichlet)
        a.b, a.x, a.work = _lib.ptr(b), _lib.ptr(x), _lib.ptr(work)
        a.queue, a.status = _lib.ptr(queue), _lib.ptr(status)
        a.order = _lib.ptr(self.order)
        x.zero_()
        if precision == "mixed":
            if values.dtype != torch.float64:
                raise ValueError("precision='mixed' refines float64 batches")
            if self._values32 is None or self._values32.numel() != values.numel():
                self._values32 = torch.empty(values.numel(), dtype=torch.float32, device=self.device)
            m = _lib.BatchedMixedArgs()
            m.base = a
            m.values32 = _lib.ptr(self._values32)
            m.inner_rtol, m.max_outer = float(inner_rtol), int(max_outer)
            _lib.check(lib.tm_batched_pcg_mixed(C.byref(m), _lib.stream_handle(self.device)),
                       "tm_batched_pcg_mixed")
        elif precision == "float64":
            _lib.check(lib.tm_batched_pcg(C.byref(a), _lib.stream_handle(self.device)), "tm_batched_pcg")
        else:
            raise ValueError(f"precision must be 'float64' or 'mixed', not {precision!r}")
        return values, b

    def _buffers(self):
        dev, dt = self.device, self.dtype
        return (torch.empty(self.n_points, dtype=dt, device=dev),
                torch.empty(5 * self.n_points, dtype=dt, device=dev),
                torch.zeros(1, dtype=torch.int32, device=dev),
                torch.zeros(self.n_systems * 16, dtype=torch.uint8, device=dev))

    def _status(self, raw: torch.Tensor) -> BatchStatus:
        ints = raw.view(torch.int32).reshape(self.n_systems, 4)
        dbl = raw.view(torch.float64).reshape(self.n_systems, 2)
        return BatchStatus(ints[:, 0].clone(), ints[:, 1].clone(), dbl[:, 1].clone())

    def solve(self, kappa: torch.Tensor, f: torch.Tensor, rtol: float = 1e-10, max_iter: int = 100000,
              precision: str = "float64", inner_rtol: float = 1e-4, max_outer: int = 30):
        """Assemble every system and solve them all; returns (u [n_points]
        concatenated, BatchStatus).  ``precision="mixed"``: iterative
        refinement with float32 inner solves (``inner_rtol``: their residual
        reduction; at most ``max_outer`` corrections)."""
        if torch.is_grad_enabled() and (kappa.requires_grad or f.requires_grad):
            raise NotImplementedError("batched solves are not differentiable; use the per-mesh path "
                                      "(assembler, Condenser, SparseMatrix.solve) for gradients")
        kappa = kappa.to(device=self.device, dtype=self.dtype).contiguous()
        f = f.to(device=self.device, dtype=self.dtype).contiguous()
        x, work, queue, status = self._buffers()
        self._solve_into(kappa, f, x, work, queue, status, rtol, max_iter, precision, inner_rtol, max_outer)
        return x, self._status(status)

    # ------------------------------------------------------------------
    def capture(self, rtol: float = 1e-10, max_iter: int = 100000, precision: str = "float64",
                inner_rtol: float = 1e-4, max_outer: int = 30):
        """Record assembly + load + batched solve as one CUDA graph."""
        opts = (precision, inner_rtol, max_outer)
        dev = self.device
        self._kappa = torch.ones(self.n_elements, dtype=self.dtype, device=dev)
        self._f = torch.zeros(self.n_points, dtype=self.dtype, device=dev)
        self._x, self._work, self._queue, self._status_raw = self._buffers()
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):                    # warm-up: plans, tables, allocator pools
            self._solve_into(self._kappa, self._f, self._x, self._work, self._queue, self._status_raw, rtol, 1,
                             *opts)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        self._graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self._graph):
            self._solve_into(self._kappa, self._f, self._x, self._work, self._queue, self._status_raw,
                             rtol, max_iter, *opts)
        return self

    def replay(self, kappa: torch.Tensor, f: torch.Tensor):
        if self._graph is None:
            raise RuntimeError("call capture() first")
        if torch.is_grad_enabled() and (kappa.requires_grad or f.requires_grad):
            raise NotImplementedError("batched solves are not differentiable; use the per-mesh path "
                                      "(assembler, Condenser, SparseMatrix.solve) for gradients")
        self._kappa.copy_(kappa.to(self._kappa.dtype), non_blocking=True)
        self._f.copy_(f.to(self._f.dtype), non_blocking=True)
        self._graph.replay()
        return self._x, self._status(self._status_raw)
