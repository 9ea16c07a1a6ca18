"""User ElementAssembler subclasses whose forward is one of the built-in
families, written the way the reference's documentation and examples write
them, assemble through the kernels and match the reference's golden values
(1e-12 relative Frobenius).

* ``SIMPLaplace``: the per-element-kappa diffusion form of the reference's
  inverse-design example (examples/inverse_design/thermal_topology.py:48-52),
  ``forward(gradu, gradv, kappa) = kappa * (gradu @ gradv)``; the golden
  ``q*_K`` values are the reference's assembly of that form.
* a mass form ``forward(u, v) = u * v`` (builtin.py:99-100): golden ``q*_M``.
* an elasticity form ``forward(gradu, gradv, E)`` returning the isotropic
  block with nu = 0.3: golden ``q*_El`` (the reference's Ba^T C(E) Bb).
A form whose modulus is a nonlinear function of its coefficient assembles
through the same kernels; a form that is none of these still raises
NotImplementedError."""
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import load_golden, rel_fro
from tensormesh_gb300.assemble import recognise_form

pytestmark = pytest.mark.gpu

ETYPE = {"tri3": "triangle", "tri6": "triangle6", "tet4": "tetra", "tet10": "tetra10", "quad": "quad",
         "quad9": "quad9"}


class SIMPLaplace(tg.ElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return kappa * (gradu @ gradv)


class PlainMass(tg.ElementAssembler):
    def forward(self, u, v):
        return u * v


class IsotropicElasticity(tg.ElementAssembler):
    def __post_init__(self, nu=0.3):
        self.nu = nu

    def forward(self, gradu, gradv, E):
        lam = E * self.nu / ((1 + self.nu) * (1 - 2 * self.nu))
        mu = E / (2 * (1 + self.nu))
        eye = torch.eye(gradu.shape[0], dtype=gradu.dtype)
        return lam * torch.outer(gradu, gradv) + mu * (torch.outer(gradv, gradu) + (gradu @ gradv) * eye)


class SquaredKappa(tg.ElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return kappa * kappa * (gradu @ gradv)


class Anisotropic(tg.ElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return kappa * gradu[0] * gradv[0]


@pytest.mark.parametrize("case", list(ETYPE))
def test_user_forms_match_reference(case, cuda):
    g = load_golden(case)
    mesh = tg.Mesh(torch.from_numpy(g["points"]), {ETYPE[case]: torch.from_numpy(g["conn"])}).to(cuda)
    kappa, E = (torch.from_numpy(g[k]).to(cuda) for k in ("kappa", "E"))
    for qo in g["qorders"]:
        asm = SIMPLaplace.from_mesh(mesh, quadrature_order=int(qo))
        K = asm(mesh.points, element_data={"kappa": kappa})
        assert rel_fro(K.values, g[f"q{qo}_K"]) <= 1e-12
        M = PlainMass.from_assembler(asm)(mesh.points)
        assert rel_fro(M.values, g[f"q{qo}_M"]) <= 1e-12
        El = IsotropicElasticity.from_assembler(asm)(mesh.points, element_data={"E": E})
        assert rel_fro(El.values, g[f"q{qo}_El"]) <= 1e-12
        # fused launch of the recognised diffusion and mass forms
        Kf, Mf = tg.assemble_forms([asm, PlainMass.from_assembler(asm)], mesh.points, {"kappa": kappa})
        assert torch.equal(Kf, K.values) and torch.equal(Mf, M.values)


def test_recognition(cuda):
    mesh = tg.gen_unit_cube(2, jitter=0.1, seed=5).to(cuda)
    r = recognise_form(SIMPLaplace.from_mesh(mesh))
    assert (r.form, r.coef) == ("diffusion", "kappa")
    assert recognise_form(PlainMass.from_mesh(mesh)).form == "mass"
    r = recognise_form(IsotropicElasticity.from_mesh(mesh, nu=0.25))
    assert r.form == "elasticity" and abs(r.nu - 0.25) < 1e-14
    # a modulus nonlinear in the coefficient: kappa^2 per element
    sq = SquaredKappa.from_mesh(mesh)
    r = recognise_form(sq)
    assert r.form == "diffusion" and r.cmap is not None
    k = torch.linspace(0.5, 2.0, mesh.n_elements, dtype=torch.float64, device=cuda)
    K2 = sq(mesh.points, element_data={"kappa": k})
    K1 = SIMPLaplace.from_assembler(sq)(mesh.points, element_data={"kappa": k * k})
    assert rel_fro(K2.values, K1.values) <= 1e-14
    bad = Anisotropic.from_mesh(mesh)
    assert recognise_form(bad) is None
    with pytest.raises(NotImplementedError):
        bad(mesh.points, element_data={"kappa": torch.ones(mesh.n_elements, dtype=torch.float64, device=cuda)})
    with pytest.raises(KeyError):
        SIMPLaplace.from_mesh(mesh)(mesh.points)
