"""Recognition of user forward integrands as built-in families (host only:
the probe runs forward on seeded random float64 arguments)."""
import torch

import tensormesh_gb300 as tg
from tensormesh_gb300.assemble import recognise_form


class SIMPLaplace(tg.ElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return kappa * (gradu @ gradv)


class Laplace(tg.ElementAssembler):
    def forward(self, gradu, gradv):
        return gradu @ gradv


class Mass(tg.ElementAssembler):
    def forward(self, u, v):
        return u * v


class Elastic(tg.ElementAssembler):
    def __post_init__(self, nu=0.3, E=1.0):
        self.nu, self.E = nu, E

    def forward(self, gradu, gradv):
        lam = self.E * self.nu / ((1 + self.nu) * (1 - 2 * self.nu))
        mu = self.E / (2 * (1 + self.nu))
        eye = torch.eye(gradu.shape[0], dtype=gradu.dtype)
        return lam * torch.outer(gradu, gradv) + mu * (torch.outer(gradv, gradu) + (gradu @ gradv) * eye)


class Nonlinear(tg.ElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return torch.exp(kappa) * (gradu @ gradv)


class Advection(tg.ElementAssembler):
    def forward(self, gradu, v):
        return gradu[0] * v


def test_recognised_families():
    mesh = tg.gen_unit_cube(2, jitter=0.1, seed=5)
    r = recognise_form(SIMPLaplace.from_mesh(mesh))
    assert (r.form, r.coef) == ("diffusion", "kappa")
    r = recognise_form(Laplace.from_mesh(mesh))
    assert (r.form, r.coef) == ("diffusion", None)
    assert recognise_form(Mass.from_mesh(mesh)).form == "mass"
    r = recognise_form(Elastic.from_mesh(mesh, nu=0.25, E=2.5))
    assert r.form == "elasticity" and r.coef is None
    assert abs(r.nu - 0.25) < 1e-14 and abs(r.scale - 2.5) < 1e-13
    tri = tg.gen_unit_square(3, jitter=0.1, seed=6)
    r = recognise_form(Elastic.from_mesh(tri, nu=0.3))
    assert r.form == "elasticity" and abs(r.nu - 0.3) < 1e-14


def test_custom_forms_are_not_recognised():
    mesh = tg.gen_unit_cube(2, jitter=0.1, seed=5)
    assert recognise_form(Nonlinear.from_mesh(mesh)) is None
    assert recognise_form(Advection.from_mesh(mesh)) is None
    assert recognise_form(tg.ElementAssembler.from_mesh(mesh)) is None
