"""CUDA path against the reference's golden fixtures (small meshes, every
form and quadrature order) through the public API and the C ABI.

Tolerances: float64 results within 1e-12 relative Frobenius of the
reference (the bar for the assembly path); patterns, slot maps and layout
hashes bit-exact; float32 results within 2e-5."""
import math

import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import load_golden, rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu

CASES = ["tri3", "tri6", "tet4", "tet10", "quad", "quad9"]
ETYPE = {"tri3": "triangle", "tri6": "triangle6", "tet4": "tetra", "tet10": "tetra10", "quad": "quad",
         "quad9": "quad9"}
TOL = 1e-12


def _mesh(g, case, dev):
    pts = torch.from_numpy(g["points"])
    conn = torch.from_numpy(g["conn"])
    return tg.Mesh(pts, {ETYPE[case]: conn}, {"is_boundary": torch.from_numpy(g["boundary"])}).to(dev)


@pytest.mark.parametrize("case", CASES)
def test_bilinear_forms_match_reference(case, cuda):
    g = load_golden(case)
    mesh = _mesh(g, case, cuda)
    kappa, E = (torch.from_numpy(g[k]).to(cuda) for k in ("kappa", "E"))
    for qo in g["qorders"]:
        asm = tg.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=int(qo))
        assert np.array_equal(asm.edges.cpu().numpy(), g[f"q{qo}_edges"])
        assert asm.edges.dtype == torch.int32
        assert np.array_equal(asm.projector[ETYPE[case]].indices.cpu().numpy(), g[f"q{qo}_slot"])
        K = asm(mesh.points, element_data={"kappa": kappa})
        assert rel_fro(K.values, g[f"q{qo}_K"]) <= TOL
        assert K.layout_hash == str(g[f"q{qo}_hash"])
        assert torch.equal(K.row_indices.cpu(), torch.from_numpy(g[f"q{qo}_edges"][0]).long())
        L = asm(mesh.points)
        assert rel_fro(L.values, g[f"q{qo}_L"]) <= TOL
        M = tg.MassElementAssembler.from_assembler(asm)(mesh.points)
        assert rel_fro(M.values, g[f"q{qo}_M"]) <= TOL
        el = tg.LinearElasticityElementAssembler.from_assembler(asm)
        El = el(mesh.points, element_data={"E": E})
        assert El.shape == (mesh.n_points * mesh.dim,) * 2
        assert rel_fro(El.values, g[f"q{qo}_El"]) <= TOL
        assert np.array_equal(El.row_indices.cpu().numpy(), g[f"q{qo}_El_row"])
        assert np.array_equal(El.col_indices.cpu().numpy(), g[f"q{qo}_El_col"])
        assert El.layout_hash == str(g[f"q{qo}_El_hash"])
        El1 = tg.LinearElasticityElementAssembler.from_assembler(asm, E=1.7, nu=0.25)(mesh.points)
        assert rel_fro(El1.values, g[f"q{qo}_El1"]) <= TOL


@pytest.mark.parametrize("case", CASES)
def test_fused_and_deterministic(case, cuda):
    g = load_golden(case)
    mesh = _mesh(g, case, cuda)
    kappa = torch.from_numpy(g["kappa"]).to(cuda)
    asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    mass = tg.MassElementAssembler.from_assembler(asm)
    Kf, Mf = tg.assemble_forms([asm, mass], mesh.points, {"kappa": kappa})
    K1 = asm(mesh.points, element_data={"kappa": kappa}).values
    K2 = asm(mesh.points, element_data={"kappa": kappa}).values
    M1 = mass(mesh.points).values
    assert torch.equal(K1, K2), "assembly must be bitwise reproducible"
    assert torch.equal(Kf, K1) and torch.equal(Mf, M1)
    # symmetric forms: value at (r, c) equals value at (c, r)
    e = asm.edges.long().cpu()
    key = e[0] * mesh.n_points + e[1]
    tkey = e[1] * mesh.n_points + e[0]
    pos = torch.searchsorted(key, tkey)
    assert torch.equal(K1.cpu()[pos], K1.cpu())


@pytest.mark.parametrize("case", CASES)
def test_linear_forms_match_reference(case, cuda):
    g = load_golden(case)
    mesh = _mesh(g, case, cuda)
    f = torch.from_numpy(g["f"]).to(cuda)
    for qo in g["qorders"]:
        src = tg.LoadNodeAssembler.from_mesh(mesh, quadrature_order=int(qo))
        b = src(mesh.points, point_data={"f": f})
        assert b.shape == (mesh.n_points,)
        assert rel_fro(b, g[f"q{qo}_b"]) <= TOL
        bc = tg.const_node_assembler(2.5).from_assembler(src)(mesh.points)
        assert rel_fro(bc, g[f"q{qo}_bconst"]) <= TOL
        fn = tg.func_node_assembler(lambda x: torch.sin(math.pi * x[..., 0]) * (1 + x[..., 1]))
        bf = fn.from_assembler(src)(mesh.points)
        assert rel_fro(bf, g[f"q{qo}_bfunc"]) <= TOL

        class Source(tg.NodeAssembler):          # the reference's documented load form
            def forward(self, v, f):
                return f * v

        bs = Source.from_assembler(src)(mesh.points, point_data={"f": f})
        assert rel_fro(bs, g[f"q{qo}_b"]) <= TOL
        bv = tg.const_node_assembler(torch.tensor([0.0, 1.0, -2.0][:mesh.dim])).from_assembler(src)(mesh.points)
        ones = tg.const_node_assembler(1.0).from_assembler(src)(mesh.points)
        assert bv.shape == (mesh.n_points * mesh.dim,)
        ref = torch.stack([ones * c for c in [0.0, 1.0, -2.0][:mesh.dim]], 1).reshape(-1)
        assert rel_fro(bv, ref) <= 1e-14


@pytest.mark.parametrize("case", ["tri3", "tet4", "tet10", "quad9"])
def test_float32(case, cuda):
    g = load_golden(case)
    mesh = _mesh(g, case, cuda).to(dtype=torch.float32)
    kappa = torch.from_numpy(g["kappa"]).float().to(cuda)
    asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    K = asm(mesh.points, element_data={"kappa": kappa})
    assert K.values.dtype == torch.float32
    assert rel_fro(K.values, g["q2_K"]) <= 2e-5
    M = tg.MassElementAssembler.from_assembler(asm)(mesh.points)
    assert rel_fro(M.values, g["q2_M"]) <= 2e-5


def test_projectors_match_reference(cuda):
    g = load_golden("projector")
    for key in [k[2:] for k in g if k.startswith("x_")]:
        dst, x, y = (torch.from_numpy(g[f"{p}_{key}"]) for p in ("dst", "x", "y"))
        n_from, n_to, width = (int(v) for v in key.split("_"))
        p = tg.ReduceProjector(dst, from_shape=n_from, to_shape=n_to).to(cuda)
        out = p(x.to(cuda))
        assert out.shape == y.shape
        assert torch.allclose(out.cpu(), y, rtol=1e-13, atol=1e-13)
        sp = tg.SparseProjector(torch.arange(n_from), dst, from_shape=n_from, to_shape=n_to).to(cuda)
        assert torch.equal(sp(x.to(cuda)), out)
    S = tg.SparseMatrix.from_block_coo(torch.from_numpy(g["block_values"]).to(cuda), torch.from_numpy(g["block_row"]),
                                       torch.from_numpy(g["block_col"]), (4, 4))
    assert torch.allclose(S.to_dense().cpu(), torch.from_numpy(g["block_dense"]))
    assert S.layout_hash == str(g["block_hash"])
    x = torch.arange(12, dtype=torch.float64)
    assert torch.allclose((S @ x.to(cuda)).cpu(), torch.from_numpy(g["block_dense"]) @ x, rtol=1e-13)


def test_geometry_kernel_matches_oracle(cuda):
    g = load_golden("tet10")
    pts, conn = torch.from_numpy(g["points"]), torch.from_numpy(g["conn"])
    tr = tg.Transformation(pts.to(cuda), conn.to(cuda), "tetra10", 3)
    grad, jxw = tr.batch_shape_grad_jxw()
    og, oj = O.shape_grad_jxw(pts, conn, "tetra10", 3)
    assert rel_fro(grad, og) <= 1e-13 and rel_fro(jxw, oj) <= 1e-13


def test_spmv_and_pcg(cuda):
    g = load_golden("tet4")
    mesh = _mesh(g, "tet4", cuda)
    K = tg.LaplaceElementAssembler.from_mesh(mesh)(mesh.points, element_data={"kappa": torch.from_numpy(g["kappa"]).to(cuda)})
    x = torch.from_numpy(np.random.default_rng(0).standard_normal(mesh.n_points)).to(cuda)
    assert rel_fro(K @ x, K.to_dense() @ x) <= 1e-14
    cond = tg.Condenser(mesh.boundary_mask)
    b = tg.const_node_assembler(1.0).from_mesh(mesh)(mesh.points)
    Ki, bi = cond(K, b)
    ui, info = tg.pcg_solve(Ki, bi, rtol=1e-13, return_info=True)
    assert info.converged
    ref = torch.linalg.solve(Ki.to_dense(), bi)
    assert rel_fro(ui, ref) <= 1e-11


@pytest.mark.parametrize("block", [False, True])
def test_spmv_row_order(block, cuda):
    """tm_spmv through the C ABI: the longest-first row order changes which
    lanes sum a row, not its value (bitwise equal to the natural order, and
    within 1e-14 of a dense product); an order entry outside [0, n_rows)
    is skipped, leaving that row of y as it was."""
    import ctypes
    from tensormesh_gb300 import _lib, solve as S
    if block:
        mesh = tg.gen_unit_cube(3, order=2, jitter=0.1, seed=95).to(cuda)
        E = torch.from_numpy(np.random.default_rng(96).uniform(0.5, 2.0, mesh.n_elements)).to(cuda)
        K = tg.LinearElasticityElementAssembler.from_mesh(mesh, nu=0.3)(mesh.points, element_data={"E": E})
    else:
        mesh = tg.gen_unit_cube(6, jitter=0.2, seed=97).to(cuda)
        K = tg.LaplaceElementAssembler.from_mesh(mesh)(mesh.points)
    lib = _lib.load()
    st = _lib.stream_handle(torch.device(cuda))
    x = torch.from_numpy(np.random.default_rng(98).standard_normal(K.shape[0])).to(cuda)
    op, keep = S.operator_of(K)
    assert op.row_order

    def run(op):
        y = torch.full_like(x, float("nan"))
        _lib.check(lib.tm_spmv(ctypes.byref(op), _lib.ptr(x), _lib.ptr(y), 1.0, 0.0, st), "tm_spmv")
        torch.cuda.synchronize()
        return y

    y_ordered = run(op)
    natural = S.operator_of(K)[0]
    natural.row_order = None
    y_natural = run(natural)
    assert torch.equal(y_ordered, y_natural)
    assert rel_fro(y_ordered, K.to_dense() @ x) <= 1e-14
    order = K._row_order().clone()
    first = int(order[0])
    order[0] = op.n_rows                     # outside [0, n_rows): skipped
    op.row_order = _lib.ptr(order)
    y_skip = run(op)
    H = K._block
    rows = torch.arange(first * H, first * H + H, device=cuda)
    assert bool(torch.isnan(y_skip[rows]).all())
    keep_rows = torch.ones_like(x, dtype=torch.bool)
    keep_rows[rows] = False
    assert torch.equal(y_skip[keep_rows], y_ordered[keep_rows])


@pytest.mark.parametrize("etype", ["tetra", "triangle"])
def test_double_float_path_and_fp64_fallback(etype, cuda):
    """Float64 P1 diffusion/mass runs in double-float arithmetic; chunks whose
    data leave its range are recomputed in FP64.  Both must match the oracle
    to 1e-12, and the stats counter tells which path ran."""
    make = (lambda: tg.gen_unit_cube(6, jitter=0.2, seed=31)) if etype == "tetra" else \
        (lambda: tg.gen_unit_square(40, jitter=0.2, seed=32))
    base = make()
    E = base.n_elements
    rng = np.random.default_rng(33)
    cases = {
        "plain": (1.0, 0.0, rng.lognormal(0.0, 1.0, E), False),
        "translated": (1.0, 1.0e4, rng.lognormal(0.0, 1.0, E), False),
        "tiny": (1.0e-9, 0.0, rng.lognormal(0.0, 1.0, E), True),
        "huge_kappa": (1.0, 0.0, rng.lognormal(0.0, 1.0, E) * 1e12, True),
    }
    for name, (scale, shift, kap, expect_fallback) in cases.items():
        pts = base.points * scale + shift
        conn = base.elements()
        kappa = torch.from_numpy(kap)
        mesh = tg.Mesh(pts, {etype: conn}).to(cuda)
        K_asm = tg.LaplaceElementAssembler.from_mesh(mesh)
        M_asm = tg.MassElementAssembler.from_assembler(K_asm)
        stats = torch.zeros(1, dtype=torch.int32, device=cuda)
        K, M = tg.assemble_forms([K_asm, M_asm], mesh.points, {"kappa": kappa.to(cuda)}, _stats=stats)
        _, _, Ko = O.assemble_matrix(pts, conn, base.n_points,
                                     lambda p, c, kappa: O.element_locals_diffusion(p, c, etype, kappa, 2), kappa=kappa)
        _, _, Mo = O.assemble_matrix(pts, conn, base.n_points, lambda p, c: O.element_locals_mass(p, c, etype, 2))
        assert rel_fro(K, Ko) <= TOL, name
        assert rel_fro(M, Mo) <= TOL, name
        fell_back = int(stats.item())
        assert (fell_back > 0) == expect_fallback, (name, fell_back)


@pytest.mark.parametrize("etype,make", [
    ("tetra10", lambda: tg.gen_unit_cube(3, order=2, jitter=0.1, seed=34)),
    ("triangle6", lambda: tg.gen_unit_square(8, order=2, jitter=0.1, seed=35)),
    ("quad9", lambda: tg.gen_unit_square(8, order=2, jitter=0.1, seed=36, cell="quad")),
])
def test_elasticity_double_float_path_and_fp64_fallback(etype, make, cuda):
    """Float64 elasticity on non-affine elements forms its blocks in
    double-float arithmetic on per-element power-of-two scaled values;
    chunks whose scales leave the window keep FP64.  Both match the oracle
    to 1e-12, and the stats counter tells which path ran."""
    base = make()
    E = base.n_elements
    Ey = np.random.default_rng(37).uniform(0.5, 2.0, E)
    cases = {
        "plain": (1.0, 0.0, 1.0, False),
        "scaled": (1.0e-3, 0.0, 1.0e4, False),
        # (a larger shift makes the FP64 Jacobian of any summation order
        # lose ~shift/h ulps to cancellation, as the reference's does)
        "translated": (1.0, 10.0, 1.0, False),
        # in 3-D the blocks scale with h (S = -84 here: FP64); in 2-D they do
        # not depend on the size, and the scaled double-float path keeps them
        "tiny": (1.0e-25, 0.0, 1.0, base.points.shape[1] == 3),
        "huge_modulus": (1.0, 0.0, 1.0e35, True),
    }
    for name, (scale, shift, emul, expect_fallback) in cases.items():
        pts = base.points * scale + shift
        conn = base.elements()
        Et = torch.from_numpy(Ey * emul)
        mesh = tg.Mesh(pts, {etype: conn}).to(cuda)
        asm = tg.LinearElasticityElementAssembler.from_mesh(mesh, nu=0.3)
        stats = torch.zeros(1, dtype=torch.int32, device=cuda)
        (K,) = tg.assemble_forms([asm], mesh.points, {"E": Et.to(cuda)}, _stats=stats)
        _, _, Ko = O.assemble_matrix(pts, conn, base.n_points,
                                     lambda p, c, E: O.element_locals_elasticity(p, c, etype, E, 0.3, 2), E=Et)
        assert rel_fro(K, Ko) <= TOL, (name, rel_fro(K, Ko))
        fell_back = int(stats.item())
        assert (fell_back > 0) == expect_fallback, (name, fell_back)


@pytest.mark.parametrize("etype,make", [
    ("tetra10", lambda: tg.gen_unit_cube(3, order=2, jitter=0.1, seed=38)),
    ("triangle6", lambda: tg.gen_unit_square(8, order=2, jitter=0.1, seed=39)),
    ("quad9", lambda: tg.gen_unit_square(8, order=2, jitter=0.1, seed=40, cell="quad")),
])
def test_scalar_forms_double_float_path_and_fp64_fallback(etype, make, cuda):
    """Float64 diffusion and mass on non-affine elements integrate each local
    pair in double-float arithmetic on per-element power-of-two scaled
    values; chunks whose scales leave the window keep FP64.  Fused K + M and
    K alone match the oracle to 1e-12, and the stats counter tells which path
    ran (kappa = 0 on some elements stays on the double-float path)."""
    base = make()
    E = base.n_elements
    rng = np.random.default_rng(41)
    kap0 = rng.lognormal(0.0, 1.0, E)
    zeros = kap0.copy()
    zeros[::7] = 0.0
    cases = {
        "plain": (1.0, kap0, False),
        "scaled": (1.0e-3, kap0 * 1e4, False),
        "zero_kappa": (1.0, zeros, False),
        "tiny": (1.0e-25, kap0, True),
        "huge_kappa": (1.0, kap0 * 1e35, True),
    }
    for name, (scale, kap, expect_fallback) in cases.items():
        pts = base.points * scale
        conn = base.elements()
        kappa = torch.from_numpy(kap)
        mesh = tg.Mesh(pts, {etype: conn}).to(cuda)
        K_asm = tg.LaplaceElementAssembler.from_mesh(mesh)
        M_asm = tg.MassElementAssembler.from_assembler(K_asm)
        stats = torch.zeros(1, dtype=torch.int32, device=cuda)
        K, M = tg.assemble_forms([K_asm, M_asm], mesh.points, {"kappa": kappa.to(cuda)}, _stats=stats)
        (K1,) = tg.assemble_forms([K_asm], mesh.points, {"kappa": kappa.to(cuda)})
        _, _, Ko = O.assemble_matrix(pts, conn, base.n_points,
                                     lambda p, c, kappa: O.element_locals_diffusion(p, c, etype, kappa, 2), kappa=kappa)
        _, _, Mo = O.assemble_matrix(pts, conn, base.n_points, lambda p, c: O.element_locals_mass(p, c, etype, 2))
        assert rel_fro(K, Ko) <= TOL, (name, rel_fro(K, Ko))
        assert rel_fro(M, Mo) <= TOL, (name, rel_fro(M, Mo))
        assert rel_fro(K1, Ko) <= TOL, (name, rel_fro(K1, Ko))
        fell_back = int(stats.item())
        assert (fell_back > 0) == expect_fallback, (name, fell_back)


@pytest.mark.parametrize("etype,make", [
    ("tetra", lambda: tg.gen_unit_cube(12, jitter=0.2, seed=71)),
    ("tetra10", lambda: tg.gen_unit_cube(5, order=2, jitter=0.1, seed=72)),
    ("triangle6", lambda: tg.gen_unit_square(20, order=2, jitter=0.1, seed=73)),
])
def test_staged_plan_multichunk(etype, make, cuda):
    """Many chunks, each staging its slots and contributions into shared
    memory by bulk copy: values match the oracle, no wait ran out."""
    from tensormesh_gb300 import _lib
    base = make()
    m = base.to(cuda)
    kap = torch.from_numpy(np.random.default_rng(74).lognormal(0.0, 1.0, base.n_elements))
    K_asm = tg.LaplaceElementAssembler.from_mesh(m)
    assert K_asm._topo(True).matrix_plan(torch.device(cuda)).n_chunks > 4
    K = K_asm(m.points, element_data={"kappa": kap.to(cuda)})
    _, _, Ko = O.assemble_matrix(base.points, base.elements(), base.n_points,
                                 lambda p, c, kappa: O.element_locals_diffusion(p, c, etype, kappa, 2), kappa=kap)
    assert rel_fro(K.values, Ko) <= TOL
    assert _lib.load().tm_device_fault() == _lib.TM_OK


@pytest.mark.parametrize("block", [False, True])
def test_persistent_pcg_matches_launch_loop(block, cuda):
    """tm_pcg_iterate_until (one cooperative launch, stop on the device)
    reaches the same solution as tm_pcg_iterate (six launches per
    iteration), sets the converged flag, and repeats bit for bit."""
    import ctypes
    from tensormesh_gb300 import _lib, solve as S
    if block:
        mesh = tg.gen_unit_cube(4, order=2, jitter=0.1, seed=91).to(cuda)
        E = torch.from_numpy(np.random.default_rng(92).uniform(0.5, 2.0, mesh.n_elements)).to(cuda)
        K = tg.LinearElasticityElementAssembler.from_mesh(mesh, nu=0.3)(mesh.points, element_data={"E": E})
        mask = (mesh.points[:, 2] == 0.0).repeat_interleave(3)
    else:
        mesh = tg.gen_unit_cube(10, jitter=0.2, seed=93).to(cuda)
        K = tg.LaplaceElementAssembler.from_mesh(mesh)(mesh.points)
        mask = mesh.boundary_mask
    b = torch.from_numpy(np.random.default_rng(94).standard_normal(K.shape[0])).to(cuda)
    Kc, bc = tg.Condenser(mask)(K, b)
    lib = _lib.load()

    def solve(until):
        n = bc.numel()
        x = torch.zeros(n, dtype=torch.float64, device=cuda)
        work = torch.empty(5, n, dtype=torch.float64, device=cuda)
        scal = torch.zeros(8, dtype=torch.float64, device=cuda)
        part = torch.empty(lib.tm_pcg_partials_bytes() // 8, dtype=torch.float64, device=cuda)
        op, keep = S.operator_of(Kc)
        a = S.PcgArgs()
        a.A = op
        a.b, a.x = _lib.ptr(bc), _lib.ptr(x)
        a.r, a.z, a.p, a.q, a.dinv = (_lib.ptr(work[i]) for i in range(5))
        a.scalars, a.partials = _lib.ptr(scal), _lib.ptr(part)
        st = _lib.stream_handle(torch.device(cuda))
        _lib.check(lib.tm_pcg_start(ctypes.byref(a), st), "start")
        if until:
            _lib.check(lib.tm_pcg_iterate_until(ctypes.byref(a), 20000, 1e-12, st), "until")
        else:
            done = 0
            while done < 20000:
                _lib.check(lib.tm_pcg_iterate(ctypes.byref(a), 50, st), "iterate")
                done += 50
                s = scal.cpu()
                if s[3] <= 1e-24 * s[4]:
                    break
        torch.cuda.synchronize()
        return x.clone(), scal.cpu().clone()

    x1, s1 = solve(True)
    x2, s2 = solve(True)
    x0, s0 = solve(False)
    assert torch.equal(x1, x2) and torch.equal(s1, s2)
    assert s1[6] == 1.0 and s1[3] <= 1e-24 * s1[4]
    assert s1[5] <= s0[5]
    assert rel_fro(x1, x0) <= 1e-10
    assert lib.tm_device_fault() == 0
