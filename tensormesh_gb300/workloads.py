"""Seeded synthetic workloads the benchmark and the parity tests run on.

Each builder returns the mesh and its coefficient fields, generated with
``numpy.random.default_rng`` so that the same seed gives the same inputs on
every machine.

* ``poisson_tri``: P1 triangles on the unit square, f = 2 pi^2 sin(pi x)
  sin(pi y) at the nodes, zero Dirichlet data on the boundary; the exact
  solution is sin(pi x) sin(pi y).  Default n = 256 (131,072 elements,
  66,049 nodes).
* ``diffusion_mass_tet``: Kuhn-split unit cube, interior nodes moved by
  U(-0.2h, 0.2h), per-element kappa ~ lognormal(0, 1).  Default n = 64
  (1,572,864 elements, 274,625 nodes).
* ``elasticity_p2tet``: P2 tetrahedra (10 nodes) on the Kuhn-split cube,
  per-element Young's modulus ~ U[0.5, 2], nu = 0.3, body force (0,0,-1),
  face z = 0 clamped.  Default n = 32 (196,608 elements, 274,625 nodes).
* ``inverse_diffusion_tet``: Kuhn-split cube, kappa_true ~ lognormal(0,
  0.5), f = 1, zero Dirichlet data.  Default n = 48 (663,552 elements).
* ``batched_poisson_tri``: many triangulated unit squares with n ~
  U{16..128} cells per side, interior nodes moved by U(-0.2h, 0.2h),
  kappa ~ lognormal(0, 1), nodal f ~ U[-1, 1], zero Dirichlet data.
"""
from dataclasses import dataclass, field
from typing import Dict, List

import math
import numpy as np
import torch

from .mesh import Mesh, gen_unit_square, gen_unit_cube

SEED_DIFFUSION = 20240601
SEED_ELASTIC = 20240602
SEED_INVERSE = 20240603
SEED_BATCH = 20240604


@dataclass
class Workload:
    name: str
    mesh: Mesh
    data: Dict[str, torch.Tensor] = field(default_factory=dict)
    params: Dict[str, float] = field(default_factory=dict)


def poisson_tri(n: int = 256) -> Workload:
    mesh = gen_unit_square(n)
    x, y = mesh.points[:, 0], mesh.points[:, 1]
    f = 2 * math.pi ** 2 * torch.sin(math.pi * x) * torch.sin(math.pi * y)
    exact = torch.sin(math.pi * x) * torch.sin(math.pi * y)
    return Workload(f"poisson_tri_{n}", mesh, {"f": f, "exact": exact})


def diffusion_mass_tet(n: int = 64, seed: int = SEED_DIFFUSION) -> Workload:
    mesh = gen_unit_cube(n, jitter=0.2, seed=seed)
    rng = np.random.default_rng(seed + 1)
    kappa = torch.from_numpy(rng.lognormal(0.0, 1.0, mesh.n_elements))
    return Workload(f"diffusion_mass_tet_{n}", mesh, {"kappa": kappa})


def elasticity_p2tet(n: int = 32, seed: int = SEED_ELASTIC) -> Workload:
    mesh = gen_unit_cube(n, order=2)
    rng = np.random.default_rng(seed)
    E = torch.from_numpy(rng.uniform(0.5, 2.0, mesh.n_elements))
    clamp = mesh.points[:, 2] == 0.0
    return Workload(f"elasticity_p2tet_{n}", mesh, {"E": E, "clamp": clamp},
                    {"nu": 0.3, "body_force_z": -1.0})


def inverse_diffusion_tet(n: int = 48, seed: int = SEED_INVERSE) -> Workload:
    mesh = gen_unit_cube(n)
    rng = np.random.default_rng(seed)
    kappa_true = torch.from_numpy(rng.lognormal(0.0, 0.5, mesh.n_elements))
    return Workload(f"inverse_diffusion_tet_{n}", mesh,
                    {"kappa_true": kappa_true, "f": torch.ones(mesh.n_points, dtype=torch.float64)})


def batched_poisson_tri(n_mesh: int = 512, n_min: int = 16, n_max: int = 128,
                        seed: int = SEED_BATCH) -> List[Workload]:
    rng = np.random.default_rng(seed)
    sizes = rng.integers(n_min, n_max + 1, size=n_mesh)
    out = []
    for i, n in enumerate(sizes):
        mesh = gen_unit_square(int(n), jitter=0.2, seed=seed * 1000 + i)
        kappa = torch.from_numpy(rng.lognormal(0.0, 1.0, mesh.n_elements))
        f = torch.from_numpy(rng.uniform(-1.0, 1.0, mesh.n_points))
        out.append(Workload(f"batched_poisson_tri_{i}_n{n}", mesh, {"kappa": kappa, "f": f}))
    return out
