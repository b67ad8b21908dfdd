"""Adjoint (backward) assembly: gradients of the compliance J = b^T u with
K(kappa, x) u = b (zero Dirichlet by static condensation) with respect to the
per-element kappa and the nodal coordinates, against the reference's own
autograd (golden fixture) and against central finite differences."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from oracle import fem

pytestmark = pytest.mark.gpu
DEV = "cuda"


class KappaLaplace(tg.ElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return kappa * (gradu @ gradv)


def compliance(mesh, x, kappa, rtol=1e-13):
    K = KappaLaplace.from_mesh(mesh, quadrature_order=1)(x, element_data={"kappa": kappa})
    b = tg.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=1)(x)
    cond = tg.Condenser(mesh.boundary_mask)
    K_ii, f_i = cond(K, b)
    u = cond.recover(K_ii.solve(f_i, rtol=rtol))
    return (b * u).sum()


def test_gradients_match_reference_autograd(golden):
    pts, el, bd = golden["adj/points"], golden["adj/elements"], golden["adj/boundary"]
    mesh = tg.Mesh(points=torch.tensor(pts, device=DEV), cells={"triangle": torch.tensor(el, device=DEV)},
                   point_data={"is_boundary": torch.tensor(bd, device=DEV)})
    x = torch.tensor(pts, device=DEV, requires_grad=True)
    kappa = torch.tensor(golden["adj/kappa"], device=DEV, requires_grad=True)
    J = compliance(mesh, x, kappa)
    J.backward()
    assert abs(J.item() - float(golden["adj/J"])) <= 1e-11 * abs(float(golden["adj/J"]))
    gk = kappa.grad.cpu().numpy()
    gx = x.grad.cpu().numpy()
    ref_k, ref_x = golden["adj/dJ_dkappa"], golden["adj/dJ_dx"]
    assert np.max(np.abs(gk - ref_k)) <= 1e-9 * np.max(np.abs(ref_k))
    interior = ~bd
    assert np.max(np.abs(gx[interior] - ref_x[interior])) <= 1e-9 * np.max(np.abs(ref_x[interior]))


@pytest.mark.parametrize("n", [32])
def test_gradients_match_central_differences(n):
    """64 seeded random directions, h = 1e-6, on kappa and on interior-node xy."""
    mesh = tg.Mesh.gen_unit_square(n, device=DEV)
    g = torch.Generator().manual_seed(3)
    kappa0 = torch.exp(torch.randn(mesh.n_elements, generator=g, dtype=torch.float64)).to(DEV)
    x0 = mesh.points.clone()
    x = x0.clone().requires_grad_(True)
    kappa = kappa0.clone().requires_grad_(True)
    compliance(mesh, x, kappa).backward()
    gk, gx = kappa.grad, x.grad
    interior = ~mesh.boundary_mask
    h = 1e-6
    errs_k, errs_x = [], []
    with torch.no_grad():
        for i in range(32):
            d = torch.randn(mesh.n_elements, generator=g, dtype=torch.float64).to(DEV)
            fd = (compliance(mesh, x0, kappa0 + h * d) - compliance(mesh, x0, kappa0 - h * d)) / (2 * h)
            an = (gk * d).sum()
            # relative to the magnitude of the terms (a direction can cancel)
            errs_k.append(abs(float(fd - an)) / float((gk * d).abs().sum()))
            dx = torch.randn(x0.shape, generator=g, dtype=torch.float64).to(DEV) * interior[:, None]
            fd = (compliance(mesh, x0 + h * dx, kappa0) - compliance(mesh, x0 - h * dx, kappa0)) / (2 * h)
            an = (gx * dx).sum()
            errs_x.append(abs(float(fd - an)) / float((gx * dx).abs().sum()))
    assert max(errs_k) <= 1e-5, max(errs_k)
    assert max(errs_x) <= 1e-5, max(errs_x)


@pytest.mark.parametrize("etype", ["triangle", "triangle6", "tetra", "tetra10"])
@pytest.mark.parametrize("form", ["laplace", "mass", "elasticity"])
def test_backward_kernel_matches_oracle_directional_fd(etype, form):
    """d/dt <G, K(x + t dX, c + t dc)> at t=0 through the backward kernel vs a
    central difference of the oracle's assembly (float64)."""
    base = tg.Mesh.gen_unit_square(4) if etype.startswith("tri") else tg.Mesh.gen_unit_cube(2)
    if etype.endswith(("6", "10")):
        base = base.to_p2()
    g = torch.Generator().manual_seed(9)
    pts = base.points + 0.1 * (torch.rand(base.points.shape, generator=g, dtype=torch.float64) - 0.5) / 4
    el = base.cells[etype]
    c0 = torch.exp(torch.randn(el.shape[0], generator=g, dtype=torch.float64))
    mesh = tg.Mesh(points=pts.to(DEV), cells={etype: el.to(DEV)})

    class F(tg.ElementAssembler):
        pass
    if form == "laplace":
        F.forward = lambda self, gradu, gradv, kappa: kappa * (gradu @ gradv)
    elif form == "mass":
        F.forward = lambda self, u, v, kappa: kappa * u * v
    else:
        lam, mu = tg.forms.reference_lame(1.0, 0.3)
        F.forward = lambda self, gradu, gradv, kappa: kappa * tg.forms.elasticity_block(gradu, gradv, lam, mu)
    x = pts.to(DEV).requires_grad_(True)
    c = c0.to(DEV).requires_grad_(True)
    K = F.from_mesh(mesh, quadrature_order=2)(x, element_data={"kappa": c})
    G = torch.randn(K.nnz, generator=g, dtype=torch.float64).to(DEV)
    (K.values * G).sum().backward()
    dX = torch.randn(pts.shape, generator=g, dtype=torch.float64)
    dc = torch.randn(el.shape[0], generator=g, dtype=torch.float64)
    an = float((x.grad.cpu() * dX).sum() + (c.grad.cpu() * dc).sum())
    h = 1e-6

    def ev(t):
        _, _, v = fem.assemble_csr((pts + t * dX).numpy(), el.numpy(), etype, form, 2, coef=(c0 + t * dc).numpy())
        return float((torch.from_numpy(v) * G.cpu()).sum())
    fd = (ev(h) - ev(-h)) / (2 * h)
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(an))
