"""Benchmark: P1-tet diffusion + mass assembly (FP64) on the Kuhn-split unit
cube, 64^3 cubes x 6 (1,572,864 elements, 274,625 nodes), per-element kappa
~ lognormal(0,1), jittered interior nodes -- the workload the headline metric
"P1-tet elements assembled/s" is quoted on.

One step = one assembly pass producing the CSR values of K(kappa) and M.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm prints ``value`` (elements/s, inputs resident in HBM, L2 flushed
between steps), ``e2e`` (the same through the public API with the inputs
copied from pinned host memory and both value arrays copied back, every
step), the roofline of the assembly pass, the CPU baseline (the oracle on
the host cores) and the SM clocks seen during the timed region.  The
reference arm times the reference's op sequence (a restatement in torch) on
the host cores.  With torchrun, every rank assembles its own copy of the
mesh ("replicas only": the path has no exchange step).

The other workloads of the path, each printing its own line
(``--workload``): ``poisson`` (131,072 P1 triangles: a whole solve through
the public API and its L2 error), ``elasticity`` (196,608 P2 tets: the
assembly pass, its e2e, condensation and Jacobi-PCG; ``--impl reference
--workload elasticity`` for the reference's op sequence), ``spmv`` (the
condensed elasticity operator's SpMV), ``inverse`` (663,552 P1 tets:
forward solve against the adjoint gradient) and ``batched`` (512 uneven
triangle meshes in one graph replay against per-mesh calls).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "P1-tet elements assembled/s vs ref torch-GPU (FP64, <=1e-12 rel); batched solves/s"
WORKLOAD = "diffusion_mass_tet_64: P1 tet K(kappa)+M, 64^3 cubes x 6 Kuhn, 1,572,864 elements, 274,625 nodes, FP64"


def _workload_name(n):
    if n == 64:
        return WORKLOAD
    return f"diffusion_mass_tet_{n}: P1 tet K(kappa)+M, {n}^3 cubes x 6 Kuhn, {6 * n ** 3} elements, FP64"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1 and not torch.distributed.is_initialized():
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        torch.distributed.init_process_group(backend)
    return ws, rank, local


def _barrier(ws):
    if ws > 1:
        torch.distributed.barrier()


def _max_over_ranks(x, ws, dev):
    if ws == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples (every 200 ms) of the SM clock and throttle reasons."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="tm_clocks_", suffix=".csv")
        os.close(fd)

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    smax.append(float(f[2]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic():
    """DRAM bytes per assembly pass from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "k_p1df_tet4_diffusion_mass.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh).get("dram_bytes_per_pass")
    return None


# float64 FMA rate of this GPU, measured with an FMA-chain probe (1:62 of
# FP32): the roof of any kernel that does its arithmetic in native float64
FP64_PEAK_GFLOPS = 1254.0


def algorithmic_bytes(N, E, nnz):
    """Inputs read once, outputs written once, int32 indices, slot map
    included: 24N (points) + 16E (connectivity) + 8E (kappa) + 64E (4x4 int32
    slot map) + 2 x 8 nnz (K and M values)."""
    return 24 * N + 16 * E + 8 * E + 64 * E + 16 * nnz


def cpu_baseline(wl, budget_s=12.0):
    from oracle import fem_oracle as O
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    pts = wl.mesh.points
    conn = wl.mesh.elements()
    edges, slot = O.element_pattern(conn, wl.mesh.n_points)
    kappa = wl.data["kappa"]
    O.reference_call_diffusion_mass(pts[:0], conn[:0], kappa[:0], slot[:0], edges[:, :0], with_hash=False)
    runs, t0 = 0, time.perf_counter()
    while True:
        O.reference_call_diffusion_mass(pts, conn, kappa, slot, edges)
        runs += 1
        el = time.perf_counter() - t0
        if el >= budget_s or runs >= 5:
            break
    E = conn.shape[0]
    return {"value": E * runs / el, "unit": "elements/s", "cores": threads, "kind": "port",
            "sample": f"{runs} full passes ({E} elements each, K+M incl. per-call SparseMatrix hashing) "
                      f"of the reference op sequence in torch on {threads} host threads, {el:.1f} s"}


def run_ours(args, ws, rank, local):
    import tensormesh_gb300 as tg
    from tensormesh_gb300 import _lib, workloads as W
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    wl = W.diffusion_mass_tet(args.cubes)
    mesh = wl.mesh.to(dev)
    kappa = wl.data["kappa"].to(dev)
    K_asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    M_asm = tg.MassElementAssembler.from_assembler(K_asm)
    N, E, nnz = mesh.n_points, mesh.n_elements, K_asm.edges.shape[1]
    ed = {"kappa": kappa}
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)      # > 129 MB of L2
    kb, ke = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for ev in (kb, ke):
        ev.record()
    for _ in range(args.warmup):
        tg.assemble_forms([K_asm, M_asm], mesh.points, ed)
    torch.cuda.synchronize()
    # set-up of a device mesh in a warm process: from_mesh (processing
    # order, pattern, slot map on the GPU) and the chunk plan of the first call
    t0 = time.perf_counter()
    K_new = tg.LaplaceElementAssembler.from_mesh(mesh)
    K_new._topology.matrix_plan(dev, dtype=torch.float64)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    del K_new
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    kbeg = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    kend = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    kdone = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for ev in kbeg + kend + kdone:
        ev.record()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    _barrier(ws)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        starts[k].record()
        tg.assemble_forms([K_asm, M_asm], mesh.points, ed, _events=(kbeg[k], None, kdone[k]))
        ends[k].record()
    torch.cuda.synchronize()
    _barrier(ws)
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    # device time of the pass: from the element-chunk kernel's launch to the
    # end of its finalisation, events recorded by the library on the
    # launching stream; the API step (host call included) beside it
    api_ms = statistics.mean(s.elapsed_time(e) for s, e in zip(starts, ends))
    pass_ms = [s.elapsed_time(e) for s, e in zip(kbeg, kdone)]
    ms = _max_over_ranks(statistics.mean(pass_ms), ws, dev)
    # the element-chunk kernel alone, after the timed region (an event
    # between the two kernels serialises their launches)
    for k in range(args.steps):
        flush.zero_()
        tg.assemble_forms([K_asm, M_asm], mesh.points, ed, _events=(kbeg[k], kend[k]))
    torch.cuda.synchronize()
    kms = statistics.mean(s.elapsed_time(e) for s, e in zip(kbeg, kend))

    # e2e: public API, host buffers, copies inside the timed region.  Steps
    # alternate between two streams so that one step's copies overlap the
    # other's kernels; the time per step is the total over K steps / K.
    pts_h = wl.mesh.points.clone().pin_memory()
    kap_h = wl.data["kappa"].clone().pin_memory()
    streams = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]
    bufs = []
    for _ in range(2):
        bufs.append((torch.empty_like(mesh.points), torch.empty_like(kappa),
                     torch.empty(nnz, dtype=torch.float64).pin_memory(),
                     torch.empty(nnz, dtype=torch.float64).pin_memory()))

    def e2e_step(k):
        st = streams[k % 2]
        pts_d, kap_d, K_h, M_h = bufs[k % 2]
        with torch.cuda.stream(st):
            pts_d.copy_(pts_h, non_blocking=True)
            kap_d.copy_(kap_h, non_blocking=True)
            K, M = tg.assemble_forms([K_asm, M_asm], pts_d, {"kappa": kap_d})
            K_h.copy_(K, non_blocking=True)
            M_h.copy_(M, non_blocking=True)
            K.record_stream(st)
            M.record_stream(st)

    for k in range(max(2, args.warmup)):
        e2e_step(k)
    torch.cuda.synchronize()
    e_s, e_e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    _barrier(ws)
    cur = torch.cuda.current_stream(dev)
    e_s.record(cur)
    for st in streams:
        st.wait_stream(cur)
    for k in range(args.steps):
        e2e_step(k)
    for st in streams:
        cur.wait_stream(st)
    e_e.record(cur)
    torch.cuda.synchronize()
    e2e_ms = _max_over_ranks(e_s.elapsed_time(e_e) / args.steps, ws, dev)
    h2d = pts_h.numel() * 8 + kap_h.numel() * 8
    d2h = 2 * nnz * 8

    # the host link's own rate for the same bytes: the two result copies
    # alone (device to pinned host), which bound e2e from below
    K0, M0 = tg.assemble_forms([K_asm, M_asm], mesh.points, ed)
    K_h0, M_h0 = bufs[0][2], bufs[0][3]
    for _ in range(3):
        K_h0.copy_(K0, non_blocking=True)
        M_h0.copy_(M0, non_blocking=True)
    torch.cuda.synchronize()
    l_s, l_e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l_s.record(cur)
    for _ in range(args.steps):
        K_h0.copy_(K0, non_blocking=True)
        M_h0.copy_(M0, non_blocking=True)
    l_e.record(cur)
    torch.cuda.synchronize()
    d2h_ms = l_s.elapsed_time(l_e) / args.steps
    del K0, M0

    peak, peak_kind = _peaks()
    abytes = algorithmic_bytes(N, E, nnz)
    achieved = abytes / (ms * 1e-3) / 1e9
    traffic = _traffic()
    line = {
        "metric": METRIC,
        "value": E * ws / (ms * 1e-3),
        "unit": "elements/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded jittered Kuhn-split cube, lognormal kappa)",
        "config": {"workload": _workload_name(args.cubes), "elements": E, "nodes": N, "nnz": nnz, "forms": ["diffusion", "mass"],
                   "quadrature_order": 2, "l2": "flushed between steps (512 MB write)",
                   "parallelism": f"replicas x{ws}"},
        "e2e": {"value": E * ws / (e2e_ms * 1e-3), "unit": "elements/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "d2h_copy_ms": d2h_ms, "d2h_link_gbs": d2h / (d2h_ms * 1e-3) / 1e9,
                "link_frac": d2h_ms / e2e_ms},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": "k_p1df + k_p1df_finalize (one assembly pass)",
                     "algorithmic_bytes": abytes, "k_matrix_ms": kms,
                     "fp64_gflops": 125.0 * E / (ms * 1e-3) / 1e9, "fp64_peak_gflops": FP64_PEAK_GFLOPS,
                     "fp64_frac": 125.0 * E / (ms * 1e-3) / 1e9 / FP64_PEAK_GFLOPS},
        "clocks": clocks,
        "gpu_launches": 2 * args.steps,
        "setup_s": setup_s,
        "wall_s_timed_region": wall,
        "api_ms_per_step": api_ms,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl)
    if rank == 0 and ws == 1 and not args.no_batched:
        # the metric's second half: batched solves/s (C5), with its own clocks
        line["batched"] = batched_summary(args, dev)
    if rank == 0 and ws == 1 and not args.no_secondary:
        line["secondary"] = secondary_summary(args, local)
    if rank == 0:
        print(json.dumps(line), flush=True)


def secondary_summary(args, local):
    """The other rows' figures, each with its own clock samples (a few
    steps each): C1 Poisson solve, C3 elasticity assembly pass and solve,
    C4 adjoint cost ratio."""
    import copy
    a = copy.copy(args)
    a.steps, a.warmup = 5, 2
    out = {}
    p = poisson_line(a, local)
    out["poisson_c1"] = {k: p[k] for k in ("value", "unit", "ms_per_step", "assembly_ms", "iterations",
                                           "l2_relative_error", "reference_l2_relative_error", "clocks")}
    e = elasticity_line(a, 1, local)
    out["elasticity_c3"] = {"pass_ms": e["ms_per_step"], "elements_per_s": e["value"],
                            "element_kernel_ms": e["roofline"]["k_matrix_ms"],
                            "fp64_frac": e["roofline"]["fp64_frac"], "e2e_ms": e["e2e"]["ms_per_step"],
                            "pcg_ms_per_iteration": e["solve"]["ms_per_iteration"],
                            "pcg_iterations": e["solve"]["iterations"], "clocks": e["clocks"]}
    i = inverse_line(a, local)
    out["inverse_c4"] = {k: i[k] for k in ("value", "unit", "forward_ms", "backward_ms", "adjoint_kernel_ms",
                                           "assembly_ms", "clocks")}
    return out


def run_reference(args, ws, rank, local):
    """The reference's op sequence (restated in torch, oracle/fem_oracle.py)
    on the host cores.  Each step assembles K and M over a bounded sample of
    the workload -- 1/8 of its elements, scattered into the full pattern --
    so that the run ends within minutes on the GPU machine's host cores."""
    if rank != 0:
        return
    from oracle import fem_oracle as O
    from tensormesh_gb300 import workloads as W
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    wl = W.diffusion_mass_tet(args.cubes)
    pts, conn, kappa = wl.mesh.points, wl.mesh.elements(), wl.data["kappa"]
    edges, slot = O.element_pattern(conn, wl.mesh.n_points)
    E = conn.shape[0]
    Es = max(1, E // 8)
    sample = (conn[:Es], kappa[:Es], slot[:Es * 16])
    for _ in range(args.warmup):
        O.reference_call_diffusion_mass(pts, *sample, edges, with_hash=False)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.reference_call_diffusion_mass(pts, *sample, edges)
        times.append(time.perf_counter() - t0)
    # a step assembles 1/8 of the elements but hashes the whole pattern
    # (twice, one SparseMatrix per form): the rate of a full pass is the
    # sample's assembly time scaled to all elements plus those two hashes
    hs = []
    for _ in range(3):
        t0 = time.perf_counter()
        for _ in range(2):
            O.layout_hash(edges[0], edges[1])
        hs.append(time.perf_counter() - t0)
    t_hash = statistics.median(hs)
    s_full = (statistics.mean(times) - t_hash) * (E / Es) + t_hash
    line = {"metric": METRIC, "impl": "reference", "value": E / s_full, "unit": "elements/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": s_full * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded jittered Kuhn-split cube, lognormal kappa)",
            "config": {"workload": _workload_name(args.cubes), "elements": E, "parallelism": "host cores"},
            "cpu_baseline": {"value": E / s_full, "unit": "elements/s", "cores": threads, "kind": "port",
                             "sample": f"{Es} of {E} elements per step (K+M into the full pattern), reference "
                                       f"op sequence restated in torch on {threads} host threads; the rate is "
                                       f"that of a full pass: the sample's assembly time scaled to all "
                                       f"elements plus the per-call SparseMatrix hashing of the full pattern "
                                       f"({t_hash:.3f} s)"},
            "e2e": {"value": E / s_full, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if torch.cuda.is_available() and not args.no_gpu_reference:
        dev = torch.device("cuda", local)
        pd, cd, kd, sd, ed = pts.to(dev), conn.to(dev), kappa.to(dev), slot.to(dev), edges.to(dev)
        for _ in range(max(3, args.warmup)):
            O.reference_call_diffusion_mass(pd, cd, kd, sd, ed)
        torch.cuda.synchronize()
        res = {}
        for with_hash in (True, False):
            ts = []
            for _ in range(max(3, min(args.steps, 10))):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                O.reference_call_diffusion_mass(pd, cd, kd, sd, ed, with_hash=with_hash)
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
            res["with_hash" if with_hash else "without_hash"] = E / statistics.median(ts)
        line["torch_gpu"] = {"value": res["with_hash"], "value_without_hash": res["without_hash"],
                             "unit": "elements/s",
                             "note": "the reference op sequence (torch einsum/inverse/det/index_add_) on the GPU"}
    print(json.dumps(line), flush=True)


def _time_ms(fn, dev):
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    s.record()
    out = fn()
    e.record()
    torch.cuda.synchronize(dev)
    return s.elapsed_time(e), out


def run_inverse(args, ws, rank, local):
    line = inverse_line(args, local)
    if rank == 0:
        print(json.dumps(line), flush=True)


def inverse_line(args, local):
    """C4: P1 tets 48^3 x 6, loss ||u(kappa) - u_target||^2, forward solve vs
    the adjoint backward (one adjoint PCG solve + the adjoint element pass)."""
    import tensormesh_gb300 as tg
    from tensormesh_gb300 import workloads as W
    from tensormesh_gb300.adjoint import _adjoint_call
    from tensormesh_gb300 import _lib
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    wl = W.inverse_diffusion_tet(48)
    mesh = wl.mesh.to(dev)
    asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    src = tg.const_node_assembler(1.0).from_mesh(mesh)
    cond = tg.Condenser(mesh.boundary_mask)
    with torch.no_grad():
        u_t = tg.solve_diffusion(asm, src, cond, mesh.points, wl.data["kappa_true"].to(dev), rtol=1e-10)
    fw, bw = [], []
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    for k in range(args.warmup + args.steps):
        pts = mesh.points.clone().requires_grad_(True)
        kappa = torch.ones(mesh.n_elements, dtype=torch.float64, device=dev, requires_grad=True)
        t_f, loss = _time_ms(lambda: ((tg.solve_diffusion(asm, src, cond, pts, kappa, rtol=1e-10) - u_t) ** 2).sum(), dev)
        t_b, _ = _time_ms(lambda: loss.backward(), dev)
        if k >= args.warmup:
            fw.append(t_f)
            bw.append(t_b)
    u = u_t
    lam = torch.randn_like(u)
    ka = torch.ones(mesh.n_elements, dtype=torch.float64, device=dev)
    t_adj = [_time_ms(lambda: _adjoint_call(asm._topology, mesh.points, ka, 1.0, _lib.TM_ADJ_K_OUTER, u=u, lam=lam,
                                             load_source=_lib.TM_ADJ_LOAD_CONST, load_const=1.0), dev)[0]
             for _ in range(max(3, args.steps))]
    t_asm = [_time_ms(lambda: asm(mesh.points, element_data={"kappa": ka}), dev)[0] for _ in range(max(3, args.steps))]
    clocks = sampler.stop()
    f, b = statistics.median(fw), statistics.median(bw)
    line = {"metric": "adjoint gradient cost / forward solve cost (P1 tet inverse diffusion, FP64)",
            "value": b / f, "unit": "ratio", "higher_is_better": False, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "dtype": "f64", "data": "synthetic (seeded lognormal kappa_true)",
            "config": {"workload": "inverse_diffusion_tet_48: 663,552 P1 tets, f = 1, zero Dirichlet, PCG rtol 1e-10"},
            "forward_ms": f, "backward_ms": b, "adjoint_kernel_ms": statistics.median(t_adj),
            "assembly_ms": statistics.median(t_asm), "clocks": clocks}
    return line


def run_poisson(args, ws, rank, local):
    line = poisson_line(args, local)
    if rank == 0:
        print(json.dumps(line), flush=True)


def poisson_line(args, local):
    """C1: P1 triangles on the unit square, 256 x 256 cells x 2 (131,072
    elements, 66,049 nodes), f = 2 pi^2 sin(pi x) sin(pi y), zero Dirichlet
    data.  One step = the whole solve through the public API: K and b
    assembled, the boundary condensed, Jacobi-PCG to 1e-12, the solution
    recovered; the L2 error against sin(pi x) sin(pi y) is reported (the
    reference's own pipeline gives 3.7935e-05 on this mesh).  A small,
    launch-bound workload: no roofline is claimed for it."""
    import tensormesh_gb300 as tg
    from tensormesh_gb300 import workloads as W
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    wl = W.poisson_tri(256)
    mesh = wl.mesh.to(dev)
    f = wl.data["f"].to(dev)
    exact = wl.data["exact"].to(dev)
    K_asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    b_asm = tg.LoadNodeAssembler.from_mesh(mesh)
    cond = tg.Condenser(mesh.boundary_mask)

    def step():
        K = K_asm(mesh.points)
        b = b_asm(mesh.points, point_data={"f": f})
        Ki, bi = cond(K, b)
        ui, info = tg.pcg_solve(Ki, bi, rtol=1e-12, return_info=True)
        return cond.recover(ui), info

    for _ in range(args.warmup):
        step()
    times, asm_times = [], []
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    for _ in range(args.steps):
        t, (u, info) = _time_ms(step, dev)
        times.append(t)
        ta, _ = _time_ms(lambda: (K_asm(mesh.points), b_asm(mesh.points, point_data={"f": f})), dev)
        asm_times.append(ta)
    clocks = sampler.stop()
    ms = statistics.median(times)
    err = float((u - exact).norm() / exact.norm())
    line = {"metric": "P1-triangle Poisson solves/s (assemble K and b, condense, Jacobi-PCG to 1e-12, FP64)",
            "value": 1e3 / ms, "unit": "solves/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (structured unit square, f = 2 pi^2 sin(pi x) sin(pi y))",
            "config": {"workload": "poisson_tri_256: 131,072 P1 triangles, 66,049 nodes, zero Dirichlet data"},
            "assembly_ms": statistics.median(asm_times), "iterations": info.iterations,
            "converged": info.converged, "l2_relative_error": err,
            "reference_l2_relative_error": 3.7935219e-05, "clocks": clocks}
    return line


def _elastic_name(n):
    return (f"elasticity_p2tet_{n}: P2 tet isotropic elasticity (10-node tets, E ~ U[0.5, 2] per element, "
            f"nu = 0.3), {n}^3 cubes x 6 Kuhn, {6 * n ** 3:,} elements, {(2 * n + 1) ** 3:,} nodes, 3x3 blocks, FP64")


def elasticity_bytes(N, E, nnz, B=10):
    """Inputs read once, outputs written once: 24N (points) + 4BE (int32
    connectivity) + 8E (Young's modulus) + 4B^2 E (int32 block slot map) +
    8 nnz (scalar values of the 3x3 blocks)."""
    return 24 * N + 4 * B * E + 8 * E + 4 * B * B * E + 8 * nnz


# FP64 flops per P2-tet elasticity element in the fewest-op formulation
# (4 quadrature points; Jacobian, cofactors and 10 gradients per point; the
# 55 unique 3x3 blocks of B_i^T C B_j per point), the figure the FP64 roof of
# this workload is quoted on
ELASTIC_FLOPS_PER_ELEMENT = 13000.0


def run_elasticity(args, ws, rank, local):
    line = elasticity_line(args, ws, local)
    if rank == 0:
        print(json.dumps(line), flush=True)


def elasticity_line(args, ws, local):
    """C3: one step = the 3x3 block values of K(E) for 196,608 P2 tets
    (FP64).  Also times the set-up (from_mesh), the end-to-end call with host
    buffers, and the solve that follows in the reference's examples:
    condensation of the clamped face z = 0 and Jacobi-PCG to 1e-10."""
    import tensormesh_gb300 as tg
    from tensormesh_gb300 import workloads as W
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    wl = W.elasticity_p2tet(args.elastic_n)
    mesh = wl.mesh.to(dev)
    Ey = wl.data["E"].to(dev)
    t0 = time.perf_counter()
    asm = tg.LinearElasticityElementAssembler.from_mesh(mesh, nu=0.3)
    setup_s = time.perf_counter() - t0
    N, E = mesh.n_points, mesh.n_elements
    nnz = asm.edges.shape[1] * 9
    ed = {"E": Ey}
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        tg.assemble_forms([asm], mesh.points, ed)
    torch.cuda.synchronize()
    kbeg = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    kdone = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for ev in kbeg + kdone:
        ev.record()                              # torch creates an event's handle on its first record
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    _barrier(ws)
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()
        tg.assemble_forms([asm], mesh.points, ed, _events=(kbeg[k], None, kdone[k]))
    torch.cuda.synchronize()
    _barrier(ws)
    clocks = sampler.stop()
    ms = _max_over_ranks(statistics.mean(s.elapsed_time(e) for s, e in zip(kbeg, kdone)), ws, dev)
    # the element-chunk kernel alone, after the timed region (an event
    # between the two kernels serialises their launches)
    kend = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for ev in kend:
        ev.record()
    for k in range(args.steps):
        flush.zero_()
        tg.assemble_forms([asm], mesh.points, ed, _events=(kbeg[k], kend[k]))
    torch.cuda.synchronize()
    kms = statistics.mean(s.elapsed_time(e) for s, e in zip(kbeg, kend))

    # e2e: points and E from pinned host memory, the block values back;
    # steps alternate between two streams (as the P1 line's) so that one
    # step's 553 MB copy overlaps the other's kernels
    pts_h = wl.mesh.points.clone().pin_memory()
    E_h = wl.data["E"].clone().pin_memory()
    streams = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]
    bufs = [(torch.empty_like(mesh.points), torch.empty_like(Ey), torch.empty(nnz, dtype=torch.float64).pin_memory())
            for _ in range(2)]

    def e2e_step(k):
        st = streams[k % 2]
        pts_d, E_d, vals_h = bufs[k % 2]
        with torch.cuda.stream(st):
            pts_d.copy_(pts_h, non_blocking=True)
            E_d.copy_(E_h, non_blocking=True)
            (K,) = tg.assemble_forms([asm], pts_d, {"E": E_d})
            vals_h.copy_(K.reshape(-1), non_blocking=True)
            K.record_stream(st)

    for k in range(max(2, args.warmup)):
        e2e_step(k)
    torch.cuda.synchronize()
    e_s, e_e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    cur = torch.cuda.current_stream(dev)
    e_s.record(cur)
    for st in streams:
        st.wait_stream(cur)
    for k in range(args.steps):
        e2e_step(k)
    for st in streams:
        cur.wait_stream(st)
    e_e.record(cur)
    torch.cuda.synchronize()
    e2e_ms = _max_over_ranks(e_s.elapsed_time(e_e) / args.steps, ws, dev)

    # the solve: condense the clamped face, Jacobi-PCG (3x3 block rows)
    K = asm(mesh.points, element_data=ed)
    b = tg.const_node_assembler(torch.tensor([0.0, 0.0, -1.0])).from_mesh(mesh)(mesh.points)
    clamp = (mesh.points[:, 2] == 0.0).repeat_interleave(3)
    cond = tg.Condenser(clamp)
    Kc, bc = cond(K, b)
    tg.pcg_solve(Kc, bc, rtol=1e-10, max_iter=50000, check_every=100)
    t_c, (Kc, bc) = _time_ms(lambda: cond(K, b), dev)
    t_s, (uc, info) = _time_ms(lambda: tg.pcg_solve(Kc, bc, rtol=1e-10, max_iter=50000, check_every=100,
                                                    return_info=True), dev)
    n_c, nnz_c = bc.numel(), Kc.values.numel()
    it_bytes = 8 * nnz_c + 4 * (nnz_c // 9) + 4 * (n_c // 3 + 1) + 7 * 8 * n_c
    it_ms = t_s / max(1, info.iterations)

    peak, peak_kind = _peaks()
    abytes = elasticity_bytes(N, E, nnz)
    achieved = abytes / (ms * 1e-3) / 1e9
    line = {"metric": "P2-tet elasticity elements assembled/s (FP64, <=1e-12 rel)",
            "value": E * ws / (ms * 1e-3), "unit": "elements/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Kuhn-split cube, uniform E)",
            "config": {"workload": _elastic_name(args.elastic_n), "elements": E, "nodes": N, "nnz": nnz,
                       "l2": "flushed between steps (512 MB write)", "parallelism": f"replicas x{ws}"},
            "e2e": {"value": E * ws / (e2e_ms * 1e-3), "unit": "elements/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": pts_h.numel() * 8 + E_h.numel() * 8, "d2h_bytes_per_step": nnz * 8},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_kind": peak_kind,
                         "kernel": "k_matrix + k_matrix_finalize (one assembly pass)", "algorithmic_bytes": abytes,
                         "k_matrix_ms": kms,
                         "fp64_gflops": ELASTIC_FLOPS_PER_ELEMENT * E / (ms * 1e-3) / 1e9,
                         "fp64_peak_gflops": FP64_PEAK_GFLOPS,
                         "fp64_frac": ELASTIC_FLOPS_PER_ELEMENT * E / (ms * 1e-3) / 1e9 / FP64_PEAK_GFLOPS},
            "setup_s": setup_s,
            "solve": {"condense_ms": t_c, "pcg_ms": t_s, "iterations": info.iterations,
                      "relative_residual": info.relative_residual, "converged": info.converged,
                      "ms_per_iteration": it_ms, "bytes_per_iteration": it_bytes,
                      "hbm_frac_per_iteration": it_bytes / (it_ms * 1e-3) / 1e9 / peak,
                      "unknowns": n_c, "nnz": nnz_c},
            "clocks": clocks, "gpu_launches": 2 * args.steps}
    return line


def _elastic_system(n, dev):
    """The condensed P2-tet elasticity system (clamped face z = 0, body force
    (0, 0, -1)) at n^3 cubes x 6."""
    import tensormesh_gb300 as tg
    from tensormesh_gb300 import workloads as W
    wl = W.elasticity_p2tet(n)
    mesh = wl.mesh.to(dev)
    K = tg.LinearElasticityElementAssembler.from_mesh(mesh, nu=0.3)(mesh.points, element_data={"E": wl.data["E"].to(dev)})
    b = tg.const_node_assembler(torch.tensor([0.0, 0.0, -1.0])).from_mesh(mesh)(mesh.points)
    clamp = (mesh.points[:, 2] == 0.0).repeat_interleave(3)
    return tg.Condenser(clamp)(K, b)


def run_spmv(args, ws, rank, local):
    """The solver's operator kernel: y = A x on the condensed P2-tet
    elasticity system (3x3 block rows, FP64), one step = one SpMV through
    tm_spmv.  Its roofline: the values, block columns, row pointers and
    row order once, x and y once (bytes), against 2 flops per stored value
    (float64 FMAs, which bind first on this GPU)."""
    from tensormesh_gb300 import solve as S
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    Kc, bc = _elastic_system(args.elastic_n, dev)
    x = torch.randn(bc.numel(), dtype=torch.float64, device=dev)
    y = torch.empty_like(x)
    for _ in range(args.warmup):
        S.spmv(Kc, x, y)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    for k in range(args.steps):
        starts[k].record()
        S.spmv(Kc, x, y)
        ends[k].record()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = statistics.mean(s.elapsed_time(e) for s, e in zip(starts, ends))
    n, nnz = bc.numel(), Kc.values.numel()
    nb = n // 3
    abytes = 8 * nnz + 4 * (nnz // 9) + 8 * (nb + 1) + 4 * nb + 16 * n
    peak, peak_kind = _peaks()
    line = {"metric": "condensed P2-tet elasticity SpMVs/s (3x3 block rows, FP64)", "value": 1e3 / ms,
            "unit": "SpMV/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Kuhn-split cube, uniform E; random x)",
            "config": {"workload": f"elasticity_p2tet_{args.elastic_n} condensed operator: {n} unknowns, "
                                   f"{nnz} values", "l2": "inputs larger than L2 (values alone)"},
            "roofline": {"bound": "hbm", "achieved": abytes / (ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": abytes / (ms * 1e-3) / 1e9 / peak, "traffic": None, "peak_kind": peak_kind,
                         "kernel": "k_spmv_op", "algorithmic_bytes": abytes,
                         "fp64_gflops": 2.0 * nnz / (ms * 1e-3) / 1e9, "fp64_peak_gflops": FP64_PEAK_GFLOPS,
                         "fp64_frac": 2.0 * nnz / (ms * 1e-3) / 1e9 / FP64_PEAK_GFLOPS},
            "clocks": clocks, "gpu_launches": args.steps}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_reference_elasticity(args, ws, rank, local):
    """The reference's per-call elasticity work (restated in torch,
    oracle/fem_oracle.py) on the host cores over a bounded sample (1/16 of
    the elements, scattered into the full pattern, with the full layout
    hash) and, whole, on the GPU."""
    if rank != 0:
        return
    from oracle import fem_oracle as O
    from tensormesh_gb300 import workloads as W
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    wl = W.elasticity_p2tet(args.elastic_n)
    pts, conn, Ey = wl.mesh.points, wl.mesh.elements(), wl.data["E"]
    edges, slot = O.element_pattern(conn, wl.mesh.n_points)
    E = conn.shape[0]
    Es = max(1, E // 16)
    sample = (conn[:Es], Ey[:Es], slot[:Es * 100])
    O.reference_call_elasticity(pts, *sample, edges, with_hash=False)
    times = []
    for _ in range(min(args.steps, 5)):
        t0 = time.perf_counter()
        O.reference_call_elasticity(pts, *sample, edges)
        times.append(time.perf_counter() - t0)
    s = statistics.mean(times)
    line = {"metric": "P2-tet elasticity elements assembled/s (FP64, <=1e-12 rel)", "impl": "reference",
            "value": Es / s, "unit": "elements/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": s * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded Kuhn-split cube, uniform E)",
            "config": {"workload": _elastic_name(args.elastic_n), "elements": E, "parallelism": "host cores"},
            "cpu_baseline": {"value": Es / s, "unit": "elements/s", "cores": threads, "kind": "port",
                             "sample": f"{Es} of {E} elements per step (block K into the full pattern, incl. "
                                       f"the per-call from_block_coo layout hash), reference op sequence restated "
                                       f"in torch on {threads} host threads"},
            "e2e": {"value": Es / s, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if torch.cuda.is_available() and not args.no_gpu_reference:
        dev = torch.device("cuda", local)
        pd, cd, Ed, sd, ed = pts.to(dev), conn.to(dev), Ey.to(dev), slot.to(dev), edges.to(dev)
        for _ in range(max(3, args.warmup)):
            O.reference_call_elasticity(pd, cd, Ed, sd, ed, with_hash=False)
        torch.cuda.synchronize()
        res = {}
        for with_hash in (True, False):
            ts = []
            for _ in range(max(3, min(args.steps, 5))):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                O.reference_call_elasticity(pd, cd, Ed, sd, ed, with_hash=with_hash)
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
            res[with_hash] = E / statistics.median(ts)
        line["torch_gpu"] = {"value": res[True], "value_without_hash": res[False], "unit": "elements/s",
                             "note": "the reference op sequence (torch einsum/inverse/det/index_add_) on the GPU"}
    print(json.dumps(line), flush=True)


def batched_summary(args, dev):
    """C5: 512 uneven P1 triangle meshes, one graph launch (assembly + load +
    batched Jacobi-PCG to 1e-10), clocked, against two per-mesh baselines on
    a sample of the meshes scaled by element count: per-mesh calls of this
    library, and the reference's per-mesh path (its op sequence restated in
    torch on the GPU: from_mesh pattern, assembly, Condenser, the in-tree
    conjugate gradient cg_py with atol = 1e-10 ||b||)."""
    import warnings
    import tensormesh_gb300 as tg
    from oracle import fem_oracle as O
    from tensormesh_gb300 import workloads as W
    from tensormesh_gb300.batched import BatchedDiffusion
    warnings.filterwarnings("ignore", category=UserWarning)
    wls = W.batched_poisson_tri(args.meshes)
    meshes = [w.mesh for w in wls]
    kappa = torch.cat([w.data["kappa"] for w in wls]).to(dev)
    f = torch.cat([w.data["f"] for w in wls]).to(dev)
    dmeshes = [m.to(dev) for m in meshes]
    torch.cuda.synchronize(dev)
    # set-up alone (device meshes: order, pattern and plans on the GPU), then
    # the batch used below, with its chunk sizes tuned on the batch
    BatchedDiffusion(dmeshes)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    BatchedDiffusion(dmeshes)
    torch.cuda.synchronize(dev)
    setup_plain_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    batch = BatchedDiffusion(dmeshes, autotune=True).capture(rtol=1e-10)
    setup_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        batch.replay(kappa, f)
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    time.sleep(0.3)
    times = []
    for _ in range(args.steps):
        t, (u, st) = _time_ms(lambda: batch.replay(kappa, f), dev)
        times.append(t)
    clocks = sampler.stop()
    ms = statistics.median(times)
    # the same batch by mixed-precision refinement (float32 inner solves,
    # the float64 residual test), its own graph and clocks
    mbatch = BatchedDiffusion(dmeshes, autotune=True).capture(rtol=1e-10, precision="mixed")
    for _ in range(args.warmup):
        mbatch.replay(kappa, f)
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    time.sleep(0.3)
    mtimes = []
    for _ in range(args.steps):
        t, (um, stm) = _time_ms(lambda: mbatch.replay(kappa, f), dev)
        mtimes.append(t)
    mclocks = sampler.stop()
    mms = statistics.median(mtimes)
    mixed = {"value": len(meshes) / (mms * 1e-3), "unit": "solves/s", "ms_per_step": mms,
             "all_converged": stm.all_converged, "max_inner_iterations": int(stm.iterations.max()),
             "max_relative_residual": float(stm.relative_residual.max()),
             "relative_difference_vs_float64_pcg": float((um - u).norm() / u.norm()),
             "clocks": mclocks,
             "note": "tm_batched_pcg_mixed: float64 residual and corrections around float32 Jacobi-PCG "
                     "inner solves (inner rtol 1e-4), stopped by the same ||b - A x|| <= 1e-10 ||b|| test "
                     "on the true float64 residual"}
    del mbatch
    b32 = BatchedDiffusion([m.to(dev) for m in meshes], dtype=torch.float32)
    u32, st32 = b32.solve(kappa, f, rtol=1e-6)
    err32 = float((u32.double() - u).norm() / u.norm())
    sample = list(range(0, len(meshes), max(1, len(meshes) // args.sample)))[:args.sample]
    frac = sum(wls[i].mesh.n_elements for i in sample) / sum(m.n_elements for m in meshes)

    def per_mesh(run):
        out = []
        for i in [sample[-1]] + sample:          # one untimed call first
            torch.cuda.synchronize(dev)
            t1 = time.perf_counter()
            run(wls[i])
            torch.cuda.synchronize(dev)
            out.append(time.perf_counter() - t1)
        return sum(out[1:]) / frac

    def ours(w):
        m = w.mesh.to(dev)
        K = tg.LaplaceElementAssembler.from_mesh(m)(m.points, element_data={"kappa": w.data["kappa"].to(dev)})
        bb = tg.LoadNodeAssembler.from_mesh(m)(m.points, point_data={"f": w.data["f"].to(dev)})
        Kc, bc = tg.Condenser(m.boundary_mask)(K, bb)
        tg.pcg_solve(Kc, bc, rtol=1e-10)

    ref_iters = []

    def reference(w):
        m = w.mesh
        _, it = O.reference_per_mesh_solve(m.points.to(dev), m.elements().to(dev), m.boundary_mask.to(dev),
                                           w.data["kappa"].to(dev), w.data["f"].to(dev))
        ref_iters.append(it)

    loop_s = per_mesh(ours)
    ref_s = per_mesh(reference)
    return {"metric": "batched solves/s (uneven P1 triangle Poisson, one graph launch)",
            "value": len(meshes) / (ms * 1e-3), "unit": "solves/s", "higher_is_better": True,
            "ms_per_step": ms, "steps": args.steps, "warmup": args.warmup, "dtype": "f64",
            "config": {"workload": f"batched_poisson_tri: {len(meshes)} meshes, n ~ U{{16..128}}, "
                                   f"{batch.n_elements} elements, {batch.n_points} nodes, rtol 1e-10",
                       "elements_per_chunk": batch.chunks, "chunks_chosen_by": "autotune (timed on the batch)"},
            "all_converged": st.all_converged, "max_iterations": int(st.iterations.max()),
            "max_relative_residual": float(st.relative_residual.max()), "clocks": clocks,
            "per_mesh_calls": {"solves_per_s": len(meshes) / loop_s, "sample_meshes": len(sample),
                               "note": "this library per mesh: from_mesh + assemble + load + Condenser + "
                                       "pcg_solve, scaled from the sample by element count"},
            "reference_per_mesh": {"solves_per_s": len(meshes) / ref_s, "sample_meshes": len(sample),
                                   "cg_iterations_median": statistics.median(ref_iters),
                                   "note": "the reference's per-mesh path restated in torch on the GPU: "
                                           "from_mesh pattern (host SciPy), assembly op sequence, Condenser, "
                                           "cg_py to ||r|| < 1e-10 ||b||; scaled from the sample by element "
                                           "count"},
            "speedup_vs_per_mesh_calls": loop_s / (ms * 1e-3),
            "speedup_vs_reference_per_mesh": ref_s / (ms * 1e-3),
            "batch_setup_s": setup_plain_s, "batch_setup_s_with_autotune": setup_s,
            "float32": {"relative_error_vs_float64": err32, "all_converged": st32.all_converged},
            "mixed_precision_refinement": mixed}


def run_batched(args, ws, rank, local):
    """C5 alone (its own line)."""
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    line = batched_summary(args, dev)
    line.update({"n_gpus": 1, "data": "synthetic (seeded meshes, lognormal kappa, uniform f)"})
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-gpu-reference", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="leave the batched solves out of the default line")
    ap.add_argument("--no-secondary", action="store_true",
                    help="leave the C1 / C3 / C4 summaries out of the default line")
    ap.add_argument("--cubes", type=int, default=64, help="cubes per side of the Kuhn-split cube (64: 1,572,864 elements)")
    ap.add_argument("--workload", default="diffusion_mass",
                    choices=["diffusion_mass", "poisson", "elasticity", "spmv", "inverse", "batched"])
    ap.add_argument("--elastic-n", type=int, default=32,
                    help="cubes per side of the P2-tet elasticity workload (32: 196,608 elements)")
    ap.add_argument("--meshes", type=int, default=512)
    ap.add_argument("--sample", type=int, default=32)
    args = ap.parse_args()
    ws, rank, local = _dist()
    if args.impl == "reference" and args.workload == "elasticity":
        run_reference_elasticity(args, ws, rank, local)
    elif args.impl == "reference":
        run_reference(args, ws, rank, local)
    elif args.workload == "poisson":
        run_poisson(args, ws, rank, local)
    elif args.workload == "elasticity":
        run_elasticity(args, ws, rank, local)
    elif args.workload == "spmv":
        run_spmv(args, ws, rank, local)
    elif args.workload == "inverse":
        run_inverse(args, ws, rank, local)
    elif args.workload == "batched":
        run_batched(args, ws, rank, local)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
