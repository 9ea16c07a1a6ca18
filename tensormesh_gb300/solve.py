"""SpMV, Jacobi-preconditioned CG and Jacobi-preconditioned BiCGSTAB over
``SparseMatrix`` (GPU kernels of ``csrc/tm_solve.cu``).

``pcg_solve`` replaces ``SparseMatrix.solve`` for the symmetric positive
definite systems of the assembly path; ``bicgstab_solve`` the reference's
``bicgstab_py`` for general square systems.  The reference inherits ``solve``
from torch-sla (direct solvers, or CG for large systems,
docs/source/user_guide/batched_workflows.rst:124-131); its in-tree Krylov
templates are ``cg_py`` / ``bicgstab_py`` (sparse/solve/torch_solve.py:70-248).
"""
import ctypes as C
from dataclasses import dataclass
from typing import Optional

import torch

from . import _lib


def _register():
    return _lib.load()


LinearOperator = _lib.LinearOperator
PcgArgs = _lib.PcgArgs


def operator_of(A) -> tuple:
    """(LinearOperator struct, tensors to keep alive) for a SparseMatrix."""
    rp, col, perm, H = A._csr_structure()
    vals = A.values.detach()
    if perm is not None:
        vals = vals.reshape(-1, H * H)[perm].reshape(-1)
    vals = vals.contiguous()
    op = LinearOperator()
    op.dtype = _lib.dtype_code(vals.dtype)
    op.block = H
    op.n_rows = rp.numel() - 1
    op.row_ptr, op.col, op.values = _lib.ptr(rp), _lib.ptr(col), _lib.ptr(vals)
    order = A._row_order()
    op.row_order = _lib.ptr(order)
    return op, (rp, col, vals, order)


def spmv(A, x: torch.Tensor, out: Optional[torch.Tensor] = None, alpha: float = 1.0,
         beta: float = 0.0) -> torch.Tensor:
    lib = _register()
    _lib.require_cuda(A.values, "SparseMatrix values")
    x = x.to(device=A.values.device, dtype=A.values.dtype).contiguous()
    if out is None:
        out = torch.empty(A.shape[0], dtype=A.values.dtype, device=A.values.device)
        beta = 0.0
    op, keep = operator_of(A)
    _lib.check(lib.tm_spmv(C.byref(op), _lib.ptr(x), _lib.ptr(out), alpha, beta,
                           _lib.stream_handle(x.device)), "tm_spmv")
    return out


def _differentiable(A, b, return_info, **kw):
    """A solve whose values or right-hand side require grad: through
    ``SparseSolve`` (the adjoint solve with A^T in the backward)."""
    from .adjoint import SparseSolve
    out = []
    x = SparseSolve.apply(A.values, b, A, dict(kw, _info_out=out))
    return (x, out[0]) if return_info else x


@dataclass
class SolveInfo:
    iterations: int
    relative_residual: float
    converged: bool
    breakdown: bool


def pcg_solve(A, b: torch.Tensor, x0: Optional[torch.Tensor] = None, rtol: float = 1e-10,
              max_iter: Optional[int] = None, check_every: int = 25, return_info: bool = False):
    """Solve A x = b with Jacobi-preconditioned CG to ||b - A x|| <= rtol ||b||.

    Iterations run in one persistent cooperative kernel per batch
    (``tm_pcg_iterate_until``: grid barriers between phases, stop on the
    device at convergence); a batch is at most ``max(check_every, 2000)``
    iterations, and the host reads the scalars between batches."""
    if torch.is_grad_enabled() and (A.values.requires_grad or (torch.is_tensor(b) and b.requires_grad)):
        return _differentiable(A, b, return_info, method="cg", x0=x0, rtol=rtol, max_iter=max_iter,
                               check_every=check_every)
    lib = _register()
    _lib.require_cuda(A.values, "SparseMatrix values")
    dev, dt = A.values.device, A.values.dtype
    b = b.to(device=dev, dtype=dt).contiguous()
    n = A.shape[0]
    if max_iter is None:
        max_iter = max(1000, 10 * n)
    x = torch.zeros(n, dtype=dt, device=dev) if x0 is None else x0.to(device=dev, dtype=dt).clone()
    work = torch.empty(5, n, dtype=dt, device=dev)
    scal = torch.zeros(8, dtype=torch.float64, device=dev)
    partials = torch.empty(lib.tm_pcg_partials_bytes() // 8, dtype=torch.float64, device=dev)
    op, keep = operator_of(A)
    args = PcgArgs()
    args.A = op
    args.b, args.x = _lib.ptr(b), _lib.ptr(x)
    args.r, args.z, args.p, args.q, args.dinv = (_lib.ptr(work[i]) for i in range(5))
    args.scalars, args.partials = _lib.ptr(scal), _lib.ptr(partials)
    stream = _lib.stream_handle(dev)
    _lib.check(lib.tm_pcg_start(C.byref(args), stream), "tm_pcg_start")
    host = torch.empty(8, dtype=torch.float64, pin_memory=True)
    done = 0
    while True:
        host.copy_(scal, non_blocking=True)
        torch.cuda.current_stream(dev).synchronize()
        rr, bb, flag = float(host[3]), float(host[4]), float(host[6])
        rel = (rr / bb) ** 0.5 if bb > 0 else rr ** 0.5
        if rel <= rtol or flag != 0.0 or done >= max_iter or bb == 0.0:
            break
        k = min(max(check_every, 2000), max_iter - done)
        _lib.check(lib.tm_pcg_iterate_until(C.byref(args), k, rtol, stream), "tm_pcg_iterate_until")
        done += k
    _lib.check(lib.tm_device_fault(), "pcg_solve")
    info = SolveInfo(int(host[5]), rel, rel <= rtol, flag == 2.0 and rel > rtol)
    if return_info:
        return x, info
    return x


def bicgstab_solve(A, b: torch.Tensor, x0: Optional[torch.Tensor] = None, atol: float = 1e-5,
                   rtol: float = 0.0, max_iter: int = 10000, check_every: int = 50, return_info: bool = False):
    """Solve A x = b for a general square A with Jacobi-preconditioned
    BiCGSTAB (the reference's ``bicgstab_py``,
    sparse/solve/torch_solve.py:130-248: right preconditioning by
    1 / diag(A), its breakdown and omega safeguards) until
    ||b - A x|| <= max(atol, rtol ||b||).

    Iterations run on the device with every scalar there
    (``tm_bicgstab_iterate``); the host reads the residual between batches
    of ``check_every`` iterations.  Where the reference warns that it did
    not converge, this returns the iterate as well (``return_info`` tells)."""
    if torch.is_grad_enabled() and (A.values.requires_grad or (torch.is_tensor(b) and b.requires_grad)):
        return _differentiable(A, b, return_info, method="bicgstab", x0=x0, atol=atol, rtol=rtol,
                               max_iter=max_iter, check_every=check_every)
    lib = _register()
    _lib.require_cuda(A.values, "SparseMatrix values")
    dev, dt = A.values.device, A.values.dtype
    b = b.to(device=dev, dtype=dt).contiguous()
    n = A.shape[0]
    x = torch.zeros(n, dtype=dt, device=dev) if x0 is None else x0.to(device=dev, dtype=dt).reshape(-1).clone()
    work = torch.empty(8, n, dtype=dt, device=dev)
    scal = torch.zeros(16, dtype=torch.float64, device=dev)
    partials = torch.empty(lib.tm_pcg_partials_bytes() // 8, dtype=torch.float64, device=dev)
    op, keep = operator_of(A)
    args = _lib.BicgstabArgs()
    args.A = op
    args.b, args.x, args.work = _lib.ptr(b), _lib.ptr(x), _lib.ptr(work)
    args.scalars, args.partials = _lib.ptr(scal), _lib.ptr(partials)
    args.atol, args.rtol = float(atol), float(rtol)
    stream = _lib.stream_handle(dev)
    _lib.check(lib.tm_bicgstab_start(C.byref(args), stream), "tm_bicgstab_start")
    host = torch.empty(16, dtype=torch.float64, pin_memory=True)
    done = 0
    while True:
        host.copy_(scal, non_blocking=True)
        torch.cuda.current_stream(dev).synchronize()
        flag = float(host[_lib.TM_BICG_FLAG])
        if flag != 0.0 or done >= max_iter:
            break
        k = min(check_every, max_iter - done)
        _lib.check(lib.tm_bicgstab_iterate(C.byref(args), k, stream), "tm_bicgstab_iterate")
        done += k
    rr, bb = float(host[_lib.TM_BICG_RR]), float(host[_lib.TM_BICG_BB])
    rel = (rr / bb) ** 0.5 if bb > 0 else rr ** 0.5
    info = SolveInfo(int(host[_lib.TM_BICG_ITER]), rel, flag == 1.0, flag == 2.0)
    if return_info:
        return x, info
    return x
