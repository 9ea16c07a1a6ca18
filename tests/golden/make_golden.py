"""Generate the golden fixtures by running the reference itself (TensorMesh,
imported from its source tree with the two stand-ins of ``refshim.py``) on
CPU in float64.

Usage (from the repository root, with the reference source tree available)::

    python tests/golden/make_golden.py /path/to/TensorMesh [--only=facet|--only=quad|--only=full|--only=krylov]

Writes

* ``tests/golden/small_<case>.npz``: small meshes with every input and the
  reference's outputs (pattern, slot map, values, load vectors, layout
  hash, adjoint gradients).
* ``tests/golden/small_facet.npz``: the reference's FacetAssembler on the
  small meshes (``--only=facet`` writes this file alone).
* ``tests/golden/small_quad.npz``, ``small_quad9.npz`` and
  ``small_facet_quad.npz``: the same cases on quadrilateral meshes
  (``--only=quad`` writes these three alone).
* ``tests/golden/full_checksums.json``: the reference's outputs on the
  full-size workloads of ``tensormesh_gb300/workloads.py``: pattern and
  slot-map hashes, fingerprints (``checksum()`` of ``oracle/fem_oracle.py``)
  and 64 sign sketches (``sketch()``) of every value array
  (``--only=full`` writes this file alone).
* ``tests/golden/small_krylov.npz``: the reference's Jacobi-BiCGSTAB and its
  autograd wrapper on a small non-symmetric system (``--only=krylov``
  writes this file alone).

The reference's user-level forms are written exactly as its documentation
and examples write them (a ``forward(gradu, gradv, kappa)`` diffusion form,
a ``forward(gradu, gradv, E)`` elasticity form with ``voigt_stiffness``, a
``forward(v, f)`` load form).
"""
import json
import math
import os
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)


def facet_golden(tm, to_ref, quads=False):
    """small_facet.npz: the reference's FacetAssembler (integrand forms as its
    docstring writes them: ``forward(v)``, ``forward(v, f)``, a function of
    ``x`` and a constant traction vector) on the small meshes
    (small_facet_quad.npz: on the quadrilateral meshes)."""
    from tensormesh_gb300.mesh import gen_unit_square, gen_unit_cube

    class Unit(tm.FacetAssembler):
        def forward(self, v):
            return v

    class Nodal(tm.FacetAssembler):
        def forward(self, v, f):
            return f * v

    class Func(tm.FacetAssembler):
        def forward(self, v, x):
            return torch.sin(math.pi * x[0]) * (1 + x[1]) * v

    out = {}
    cases = {
        "tri3": (gen_unit_square(5, jitter=0.2, seed=111), [1, 2, 3]),
        "tri6": (gen_unit_square(3, order=2, jitter=0.1, seed=112), [2, 3]),
        "tet4": (gen_unit_cube(3, jitter=0.2, seed=113), [1, 2, 3]),
        "tet10": (gen_unit_cube(2, order=2, jitter=0.1, seed=114), [2, 3]),
    }
    if quads:
        cases = {
            "quad": (gen_unit_square(4, jitter=0.2, seed=115, cell="quad"), [1, 2, 3]),
            "quad9": (gen_unit_square(3, order=2, jitter=0.1, seed=116, cell="quad"), [2, 3]),
        }
    for name, (m, qorders) in cases.items():
        rm = to_ref(m)
        D = m.points.shape[1]
        traction = torch.tensor([0.5, -1.0] if D == 2 else [0.5, -1.0, 0.25])

        class Traction(tm.FacetAssembler):
            def forward(self, v):
                return v[:, None] * traction

        f = torch.from_numpy(np.random.default_rng(12).uniform(-1.0, 1.0, m.n_points))
        out[f"{name}_points"] = m.points.numpy()
        out[f"{name}_conn"] = m.elements().numpy()
        out[f"{name}_boundary"] = m.boundary_mask.numpy()
        out[f"{name}_f"] = f.numpy()
        out[f"{name}_traction"] = traction.numpy()
        out[f"{name}_qorders"] = np.array(qorders)
        for qo in qorders:
            out[f"{name}_q{qo}_unit"] = Unit.from_mesh(rm, quadrature_order=qo)(rm.points).numpy()
            out[f"{name}_q{qo}_nodal"] = Nodal.from_mesh(rm, quadrature_order=qo)(rm.points, point_data={"f": f}).numpy()
            out[f"{name}_q{qo}_func"] = Func.from_mesh(rm, quadrature_order=qo)(rm.points).numpy()
            out[f"{name}_q{qo}_traction"] = Traction.from_mesh(rm, quadrature_order=qo)(rm.points).numpy()
    name = "small_facet_quad.npz" if quads else "small_facet.npz"
    np.savez_compressed(os.path.join(HERE, name), **out)
    print("wrote", name)


def krylov_golden():
    """The reference's Jacobi-BiCGSTAB (sparse/solve/torch_solve.py:130-248)
    and its autograd wrapper SparseSolveTorch (:252-270) on a small
    non-symmetric system: a 5-point convection-diffusion operator on a
    15 x 15 grid (upwind convection, so A != A^T), seeded right-hand side and
    loss weights.  Writes small_krylov.npz."""
    from tensormesh.sparse.solve.torch_solve import SparseSolveTorch, bicgstab_py
    g, c = 15, 0.7
    n = g * g
    rows, cols, vals = [], [], []
    for iy in range(g):
        for ix in range(g):
            i = iy * g + ix
            ent = {i: 4.0 + 2.0 * c}
            if ix > 0:
                ent[i - 1] = -1.0 - 2.0 * c        # upwind: flow in +x and +y
            if ix < g - 1:
                ent[i + 1] = -1.0
            if iy > 0:
                ent[i - g] = -1.0 - 0.5 * c
            if iy < g - 1:
                ent[i + g] = -1.0 + 0.5 * c
            for j in sorted(ent):
                rows.append(i)
                cols.append(j)
                vals.append(ent[j])
    row = torch.tensor(rows, dtype=torch.int64)
    col = torch.tensor(cols, dtype=torch.int64)
    values = torch.tensor(vals, dtype=torch.float64)
    # right-hand side and loss weights of size 1e6: the reference's absolute
    # safeguards (|r0^ . v| and t . t against 1e-12) then leave atol = 1e-6,
    # a relative residual near 1e-12, as the criterion that ends the solve
    rng = np.random.default_rng(71)
    b = torch.from_numpy(rng.uniform(-1.0, 1.0, n) * 1e6)
    w = torch.from_numpy(rng.uniform(-1.0, 1.0, n) * 1e6)
    x = bicgstab_py(torch.stack([row, col], 0), values, n, n, b, atol=1e-6, max_iter=2000)
    # (SparseSolveTorch's backward passes the transposed indices, no longer
    # row-major, to a COO tensor declared coalesced; its gradients on this
    # system are not finite, so the fixture keeps the forward solve and the
    # weights, and the tests check gradients against direct solves)
    u = SparseSolveTorch.apply(values, row, col, (n, n), b, None, 1e-6, 2000)
    np.savez_compressed(os.path.join(HERE, "small_krylov.npz"), row=row.numpy(), col=col.numpy(),
                        values=values.numpy(), b=b.numpy(), w=w.numpy(), x=x.detach().numpy(),
                        x_autograd_forward=u.detach().numpy())
    print("wrote small_krylov.npz")


def main(reference_root, only=None):
    import refshim
    refshim.install(reference_root)
    torch.set_default_dtype(torch.float64)   # the reference builds C at the default dtype
    import meshio
    import tensormesh as tm
    from tensormesh.functional.elasticity import voigt_shape_grad, voigt_stiffness
    from tensormesh.assemble.projector import ReduceProjector
    from tensormesh.sparse import SparseMatrix
    from tensormesh_gb300.mesh import gen_unit_square, gen_unit_cube
    from tensormesh_gb300 import workloads as W
    from oracle.fem_oracle import checksum

    class KappaDiffusion(tm.ElementAssembler):
        def forward(self, gradu, gradv, kappa):
            return kappa * (gradu @ gradv)

    class ElasticityE(tm.ElementAssembler):
        def __post_init__(self, nu=0.3):
            self.nu = nu

        def forward(self, gradu, gradv, E):
            Ba = voigt_shape_grad(gradu)
            Bb = voigt_shape_grad(gradv)
            C = voigt_stiffness(E, self.nu, gradu.shape[0])
            return Ba.T @ C @ Bb

    class Source(tm.NodeAssembler):
        def forward(self, v, f):
            return f * v

    def to_ref(m):
        et = m.default_element_type
        mm = meshio.Mesh(m.points.numpy(), [meshio.CellBlock(et, m.elements().numpy())],
                         point_data={"is_boundary": m.point_data["is_boundary"].numpy()})
        return tm.Mesh(mm)

    if only == "facet":
        facet_golden(tm, to_ref)
        return
    if only == "krylov":
        krylov_golden()
        return
    if only == "full":
        full_golden(tm, to_ref, KappaDiffusion, ElasticityE, Source)
        return

    # ------------------------------------------------------------------ small
    cases = {
        "tri3": (gen_unit_square(5, jitter=0.2, seed=101), [1, 2, 3, 4]),
        "tri6": (gen_unit_square(3, order=2, jitter=0.1, seed=102), [2, 4]),
        "tet4": (gen_unit_cube(3, jitter=0.2, seed=103), [1, 2, 3]),
        "tet10": (gen_unit_cube(2, order=2, jitter=0.1, seed=104), [2, 3]),
    }
    if only == "quad":
        # quadrilaterals (written by --only=quad, with their facet file)
        cases = {
            "quad": (gen_unit_square(5, jitter=0.2, seed=107, cell="quad"), [1, 2, 3]),
            "quad9": (gen_unit_square(3, order=2, jitter=0.1, seed=108, cell="quad"), [2, 3, 4]),
        }
    for name, (m, qorders) in cases.items():
        rm = to_ref(m)
        et = m.default_element_type
        E_el = m.n_elements
        rng = np.random.default_rng(7)
        kappa = torch.from_numpy(rng.lognormal(0.0, 1.0, E_el))
        Ey = torch.from_numpy(rng.uniform(0.5, 2.0, E_el))
        f = torch.from_numpy(rng.uniform(-1.0, 1.0, m.n_points))
        out = {"points": m.points.numpy(), "conn": m.elements().numpy(), "kappa": kappa.numpy(),
               "E": Ey.numpy(), "f": f.numpy(), "boundary": m.boundary_mask.numpy(),
               "qorders": np.array(qorders)}
        for qo in qorders:
            asm = KappaDiffusion.from_mesh(rm, quadrature_order=qo)
            K = asm(rm.points, element_data={"kappa": kappa})
            L = tm.LaplaceElementAssembler.from_assembler(asm)(rm.points)
            M = tm.MassElementAssembler.from_assembler(asm)(rm.points)
            El = ElasticityE.from_assembler(asm)(rm.points, element_data={"E": Ey})
            El1 = tm.LinearElasticityElementAssembler.from_assembler(asm, E=1.7, nu=0.25)(rm.points)
            src = Source.from_mesh(rm, quadrature_order=qo)
            b = src(rm.points, point_data={"f": f})
            bc = tm.const_node_assembler(2.5).from_assembler(src)(rm.points)
            bf = tm.func_node_assembler(lambda x: torch.sin(math.pi * x[..., 0]) * (1 + x[..., 1]))
            bfun = bf.from_assembler(src)(rm.points)
            out[f"q{qo}_edges"] = asm.edges.numpy()
            out[f"q{qo}_slot"] = asm.projector[et].indices.numpy()
            out[f"q{qo}_K"] = K.values.numpy()
            out[f"q{qo}_L"] = L.values.numpy()
            out[f"q{qo}_M"] = M.values.numpy()
            out[f"q{qo}_El"] = El.values.numpy()
            out[f"q{qo}_El_row"] = El.row_indices.numpy()
            out[f"q{qo}_El_col"] = El.col_indices.numpy()
            out[f"q{qo}_El1"] = El1.values.numpy()
            out[f"q{qo}_b"] = b.numpy()
            out[f"q{qo}_bconst"] = bc.numpy()
            out[f"q{qo}_bfunc"] = bfun.numpy()
            out[f"q{qo}_hash"] = np.array(K.layout_hash)
            out[f"q{qo}_El_hash"] = np.array(El.layout_hash)
        np.savez_compressed(os.path.join(HERE, f"small_{name}.npz"), **out)
        print("wrote", name)
    if only == "quad":
        facet_golden(tm, to_ref, quads=True)
        return

    # -------------------------------------------------------- small adjoint
    m = gen_unit_cube(3, jitter=0.2, seed=105)
    rm = to_ref(m)
    rng = np.random.default_rng(8)
    kappa = torch.from_numpy(rng.lognormal(0.0, 0.5, m.n_elements)).requires_grad_(True)
    u_t = torch.from_numpy(rng.uniform(0.0, 0.1, m.n_points))
    pts = rm.points.clone().requires_grad_(True)
    asm = KappaDiffusion.from_mesh(rm)
    src = Source.from_mesh(rm)
    K = asm(pts, element_data={"kappa": kappa})
    b = src(pts, point_data={"f": torch.ones(m.n_points)})
    mask = m.boundary_mask
    Kc, bc = tm.Condenser(mask)(K, b)
    u_i = torch.linalg.solve(Kc.to_dense(), bc)
    loss = ((u_i - u_t[~mask]) ** 2).sum()
    loss.backward()
    np.savez_compressed(os.path.join(HERE, "small_adjoint.npz"),
                        points=m.points.numpy(), conn=m.elements().numpy(),
                        kappa=kappa.detach().numpy(), u_target=u_t.numpy(),
                        boundary=mask.numpy(), loss=np.array(loss.item()),
                        grad_kappa=kappa.grad.numpy(), grad_points=pts.grad.numpy())
    print("wrote adjoint")

    # ------------------------------------------------------ small projector
    g = torch.Generator().manual_seed(9)
    proj = {}
    for n_from, n_to, width in [(10, 7, 1), (1000, 100, 8), (1000, 1000, 1), (100, 10, 128)]:
        dst = torch.randint(0, n_to, (n_from,), generator=g)
        x = torch.randn(n_from, width, generator=g, dtype=torch.float64)
        y = ReduceProjector(dst, from_shape=n_from, to_shape=n_to)(x)
        key = f"{n_from}_{n_to}_{width}"
        proj[f"dst_{key}"] = dst.numpy()
        proj[f"x_{key}"] = x.numpy()
        proj[f"y_{key}"] = y.numpy()
    blocks = torch.randn(6, 3, 3, generator=g, dtype=torch.float64)
    brow = torch.tensor([0, 1, 1, 2, 3, 3])
    bcol = torch.tensor([0, 0, 1, 2, 1, 3])
    S = SparseMatrix.from_block_coo(blocks, brow, bcol, (4, 4))
    proj.update(block_values=blocks.numpy(), block_row=brow.numpy(), block_col=bcol.numpy(),
                block_dense=S.to_dense().numpy(), block_hash=np.array(S.layout_hash))
    np.savez_compressed(os.path.join(HERE, "small_projector.npz"), **proj)
    print("wrote projector")

    full_golden(tm, to_ref, KappaDiffusion, ElasticityE, Source)


def _values(v):
    """Fingerprints and sign sketches of one of the reference's value arrays."""
    from oracle.fem_oracle import checksum, sketch
    out = checksum(v)
    out["sketch"] = sketch(v)
    return out


def full_golden(tm, to_ref, KappaDiffusion, ElasticityE, Source):
    """full_checksums.json: for each full-size workload of
    ``tensormesh_gb300/workloads.py``, the reference's pattern hash, the
    SHA-256 of its slot map (int32 bytes, element-major), and for each value
    array its fingerprints and 64 sign sketches (``oracle.fem_oracle.sketch``:
    a relative-Frobenius estimate of any other array against it)."""
    from oracle.fem_oracle import slot_hash
    from tensormesh_gb300 import workloads as W

    full = {}
    t0 = time.time()
    wl = W.poisson_tri(256)
    rm = to_ref(wl.mesh)
    asm = tm.LaplaceElementAssembler.from_mesh(rm)
    K = asm(rm.points)
    b = Source.from_mesh(rm)(rm.points, point_data={"f": wl.data["f"]})
    mask = wl.mesh.boundary_mask
    Kc, bc = tm.Condenser(mask)(K, b)
    u_i = Kc.solve(bc)
    u = torch.zeros(wl.mesh.n_points)
    u[~mask] = u_i
    err = float((u - wl.data["exact"]).norm() / wl.data["exact"].norm())
    full[wl.name] = {"nnz": int(K.nnz), "hash": K.layout_hash, "slot_sha256": slot_hash(asm.projector["triangle"].indices),
                     "K": _values(K.values), "b": _values(b), "u": _values(u), "l2_rel_error": err}
    print(wl.name, err, time.time() - t0)
    del asm, K

    t0 = time.time()
    wl = W.diffusion_mass_tet(64)
    rm = to_ref(wl.mesh)
    asm = KappaDiffusion.from_mesh(rm)
    K = asm(rm.points, element_data={"kappa": wl.data["kappa"]})
    M = tm.MassElementAssembler.from_assembler(asm)(rm.points)
    full[wl.name] = {"nnz": int(K.nnz), "hash": K.layout_hash, "slot_sha256": slot_hash(asm.projector["tetra"].indices),
                     "K": _values(K.values), "M": _values(M.values)}
    print(wl.name, time.time() - t0)
    del asm, K, M

    t0 = time.time()
    wl = W.inverse_diffusion_tet(48)
    rm = to_ref(wl.mesh)
    asm = KappaDiffusion.from_mesh(rm)
    K = asm(rm.points, element_data={"kappa": wl.data["kappa_true"]})
    b = Source.from_mesh(rm)(rm.points, point_data={"f": wl.data["f"]})
    full[wl.name] = {"nnz": int(K.nnz), "hash": K.layout_hash, "slot_sha256": slot_hash(asm.projector["tetra"].indices),
                     "K": _values(K.values), "b": _values(b)}
    print(wl.name, time.time() - t0)
    del asm, K

    t0 = time.time()
    wl = W.elasticity_p2tet(32)
    rm = to_ref(wl.mesh)
    asm = ElasticityE.from_mesh(rm)
    El = asm(rm.points, element_data={"E": wl.data["E"]})
    full[wl.name] = {"nnz_blocks": int(asm.edges.shape[1]), "nnz": int(El.nnz),
                     "hash_blocks": __import__("hashlib").sha256(
                         asm.edges[0].numpy().tobytes() + asm.edges[1].numpy().tobytes()).hexdigest(),
                     "slot_sha256": slot_hash(asm.projector["tetra10"].indices),
                     "K": _values(El.values)}
    print(wl.name, time.time() - t0)

    with open(os.path.join(HERE, "full_checksums.json"), "w") as fh:
        json.dump(full, fh, indent=1, sort_keys=True)
    print("wrote full_checksums.json")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--only=")]
    only = next((a.split("=", 1)[1] for a in sys.argv[1:] if a.startswith("--only=")), None)
    main(args[0] if args else os.environ.get("TENSORMESH_REF", "reference"), only)
