"""Built-in forms (assemble/builtin.py of the reference) mapped to kernels.

* ``LaplaceElementAssembler``: grad u . grad v (builtin.py:24-62).  A
  per-element coefficient is taken from ``element_data["kappa"]`` (or a
  global one from ``scalar_data["kappa"]``), the diffusion form the
  reference's documentation writes as ``forward(gradu, gradv, kappa)``
  (examples/inverse_design/thermal_topology.py:51-52).
* ``DiffusionElementAssembler``: the same kernel, with that ``forward``.
* ``MassElementAssembler``: u v (builtin.py:64-100); ``scalar_data["rho"]``
  scales it.
* ``LinearElasticityElementAssembler(E=1.0, nu=0.3)``: B_i^T C B_j with
  isotropic C (builtin.py:102-217, functional/elasticity.py:132-284); a
  per-element Young's modulus comes from ``element_data["E"]``.
* ``const_node_assembler(c)``, ``func_node_assembler(f)`` (builtin.py:730-813)
  and ``LoadNodeAssembler`` (f v with nodal ``point_data["f"]``).
"""
import torch

from .assemble import ElementAssembler, NodeAssembler


class LaplaceElementAssembler(ElementAssembler):
    _tm_form = "diffusion"

    def forward(self, gradu, gradv):
        return gradu @ gradv

    def _tm_coefficients(self, ed, sd, E):
        if "_tm_modulus" in ed:                      # a per-node kappa, interpolated (assemble.py)
            return {"kappa": ed["_tm_modulus"]}
        return {"kappa": ed.get("kappa", sd.get("kappa"))}


class DiffusionElementAssembler(LaplaceElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return kappa * (gradu @ gradv)


class MassElementAssembler(ElementAssembler):
    _tm_form = "mass"

    def forward(self, u, v):
        return u * v

    def _tm_coefficients(self, ed, sd, E):
        return {"rho": sd.get("rho")}


class LinearElasticityElementAssembler(ElementAssembler):
    _tm_form = "elasticity"

    def __post_init__(self, E=1.0, nu=0.3):
        self.E = E
        self.nu = nu

    def forward(self, gradu, gradv):
        raise NotImplementedError("assembled by the elasticity kernel")

    def _tm_coefficients(self, ed, sd, E):
        nu = sd.get("nu", self.nu)
        return {"E": ed.get("E", sd.get("E", self.E)), "nu": nu if torch.is_tensor(nu) else float(nu)}


def const_node_assembler(c=1):
    class ConstNodeAssembler(NodeAssembler):
        def __post_init__(self, c=c):
            self.c = c

        def forward(self, v):
            return self.c * v

        @property
        def _tm_source(self):
            return ("const", self.c)

    return ConstNodeAssembler


def func_node_assembler(f=lambda x: x):
    class FuncNodeAssembler(NodeAssembler):
        def __post_init__(self, f=f):
            self.f = f

        def forward(self, x, v):
            return self.f(x) * v

    return FuncNodeAssembler


class LoadNodeAssembler(NodeAssembler):
    """b_i = int f phi_i with f given at the nodes (point_data["f"])."""

    _tm_source = ("nodal", "f")

    def forward(self, v, f):
        return f * v
