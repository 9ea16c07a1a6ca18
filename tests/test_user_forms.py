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


class Anisotropic(tg.ElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return kappa * gradu[0] * gradv[0]


class SIMPElastic(tg.ElementAssembler):
    """The plane-stress SIMP form of the reference's compliance example
    (examples/inverse_design/compliance_topology.py:31-110), restated."""

    def __post_init__(self, E_max=70e3, E_min=70.0, nu=0.3, penal=3.0):
        self.E_max, self.E_min, self.nu, self.penal = E_max, E_min, nu, penal

    def forward(self, gradu, gradv, rho):
        E = self.E_min + (rho ** self.penal) * (self.E_max - self.E_min)
        d11, d12, d33 = E / (1 - self.nu ** 2), self.nu * E / (1 - self.nu ** 2), E / (2 * (1 + self.nu))
        ux, uy, vx, vy = gradu[0], gradu[1], gradv[0], gradv[1]
        return torch.stack([torch.stack([d11 * ux * vx + d33 * uy * vy, d12 * ux * vy + d33 * uy * vx]),
                            torch.stack([d12 * uy * vx + d33 * ux * vy, d11 * uy * vy + d33 * ux * vx])])


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
    assert abs(r.nu - 0.25) < 1e-14 and abs(r.scale - 2.5) < 1e-13 and r.cmap is None
    tri = tg.gen_unit_square(3, jitter=0.1, seed=6)
    r = recognise_form(Elastic.from_mesh(tri, nu=0.3))
    assert r.form == "elasticity" and abs(r.nu - 0.3) < 1e-14


def test_coefficient_maps():
    """A family whose modulus is a nonlinear function of the coefficient:
    the modulus per element from forward on probe arguments, with its
    derivative (the reference's autograd through forward)."""
    mesh = tg.gen_unit_cube(2, jitter=0.1, seed=5)
    r = recognise_form(Nonlinear.from_mesh(mesh))
    assert (r.form, r.coef) == ("diffusion", "kappa") and r.cmap is not None
    k = torch.tensor([-0.5, 0.0, 0.7], dtype=torch.float64, requires_grad=True)
    m = r.modulus(k)
    assert torch.allclose(m, torch.exp(k.detach()), rtol=1e-13, atol=0)
    m.sum().backward()
    assert torch.allclose(k.grad, torch.exp(k.detach()), rtol=1e-13, atol=0)
    quads = tg.gen_unit_square(3, cell="quad")
    r = recognise_form(SIMPElastic.from_mesh(quads))
    assert r.form == "elasticity" and r.coef == "rho" and r.cmap is not None
    # plane stress is the kernel's isotropic block with nu' = nu / (1 + nu)
    # and E' = E (1 + 2 nu) / (1 + nu)^2
    assert abs(r.nu - 0.3 / 1.3) < 1e-14
    rho = torch.tensor([0.2, 0.6, 1.0], dtype=torch.float64)
    E = 70.0 + rho ** 3 * (70e3 - 70.0)
    assert torch.allclose(r.modulus(rho), E * 1.6 / 1.69, rtol=1e-12, atol=0)


def test_custom_forms_are_not_recognised():
    mesh = tg.gen_unit_cube(2, jitter=0.1, seed=5)
    assert recognise_form(Anisotropic.from_mesh(mesh)) is None
    assert recognise_form(Advection.from_mesh(mesh)) is None
    assert recognise_form(tg.ElementAssembler.from_mesh(mesh)) is None
