"""The float64 default path (double-float arithmetic) against the oracle on
inputs that break a naive float-pair emulation: meshes in very small or very
large units, meshes far from the origin, coefficients far outside float's
range, and sliver elements.  The bar is the one of every float64 result:
values within 1e-12 relative (max-norm over nnz relative to max|K|) of the
oracle, CSR pattern bit-exact."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from oracle import fem

pytestmark = pytest.mark.gpu
DEV = "cuda"
TOL = 1e-12


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


class KappaLaplace(tg.ElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return kappa * (gradu @ gradv)


class KappaMass(tg.ElementAssembler):
    def forward(self, u, v, kappa):
        return kappa * u * v


class EElasticity(tg.ElementAssembler):
    def forward(self, gradu, gradv, E):
        lam, mu = tg.forms.reference_lame(1.0, 0.3)
        return E * tg.forms.elasticity_block(gradu, gradv, lam, mu)


FORMS = {"laplace": (KappaLaplace, "kappa"), "mass": (KappaMass, "kappa"), "elasticity": (EElasticity, "E")}


def jittered(etype, n, seed):
    base = tg.Mesh.gen_unit_square(n) if etype.startswith("tri") else tg.Mesh.gen_unit_cube(n)
    pts = base.points.clone()
    rng = np.random.default_rng(seed)
    pts += torch.tensor(rng.uniform(-0.2, 0.2, size=pts.shape) / n)
    mesh = tg.Mesh(points=pts, cells={base.default_element_type: base.cells[base.default_element_type]})
    return mesh.to_p2() if etype.endswith(("6", "10")) else mesh


def check(pts, el, etype, form, coef, tol=TOL, q=1, oracle_pts=None):
    """``oracle_pts``: the same geometry for the oracle when ``pts`` itself
    would make the oracle inexact (a translated mesh, see below)."""
    cls, key = FORMS[form]
    ip, ix, dv = fem.assemble_csr(pts if oracle_pts is None else oracle_pts, el, etype, form, q, coef=coef)
    mesh = tg.Mesh(points=torch.tensor(pts, device=DEV), cells={etype: torch.tensor(el, device=DEV)})
    K = cls.from_mesh(mesh, quadrature_order=q)(mesh.points, element_data={key: torch.tensor(coef, device=DEV)})
    assert np.array_equal(K.indptr.cpu().numpy(), ip) and np.array_equal(K.indices.cpu().numpy(), ix)
    err = rel_err(K.values.cpu().numpy(), dv)
    assert err <= tol, (etype, form, err)
    return err


@pytest.mark.parametrize("scale", [1e-9, 1e-3, 1e3, 1e9])
@pytest.mark.parametrize("etype", ["triangle", "triangle6", "tetra", "tetra10"])
@pytest.mark.parametrize("form", ["laplace", "mass", "elasticity"])
def test_mesh_units(scale, etype, form):
    """The same jittered mesh in units 1e-9 .. 1e9: stiffness scales as
    h^(D-2), mass as h^D; double-float products of such edge vectors leave
    float's exponent range unless the kernel works in a patch frame."""
    mesh = jittered(etype, 5, 7)
    pts = mesh.points.numpy() * scale
    el = mesh.cells[etype].numpy()
    coef = np.exp(np.random.default_rng(1).normal(size=el.shape[0]))
    check(pts, el, etype, form, coef)


@pytest.mark.parametrize("etype", ["triangle", "tetra", "tetra10"])
def test_mesh_far_from_origin(etype):
    """A mesh of cell size 1/5 translated by ~1e4: a float pair holds the raw
    coordinates to 2^-49 of 1e4, i.e. 1e-10 of an edge; the frame forms edge
    vectors exactly.  The oracle runs on the translated coordinates moved back
    (an exact subtraction), because its own Jacobian sum over P2 nodes,
    sum_b X_b dN_b, cancels ~1e4-sized terms down to an edge and is itself
    wrong by ~1e-10 on the translated values (as the reference would be)."""
    mesh = jittered(etype, 5, 3)
    shift = np.array([12345.0, -23456.0, 3456.0][: mesh.points.shape[1]])
    pts = mesh.points.numpy() + shift
    back = pts - shift                      # exact (Sterbenz): the geometry of pts, near the origin
    el = mesh.cells[etype].numpy()
    coef = np.exp(np.random.default_rng(2).normal(size=el.shape[0]))
    for form in ("laplace", "elasticity"):
        check(pts, el, etype, form, coef, oracle_pts=back)


def test_coefficients_beyond_float_range():
    """kappa around 1e+-150: double-float cannot hold the element values, so
    the kernel redoes those patches in native FP64."""
    mesh = jittered("tetra", 6, 5)
    pts, el = mesh.points.numpy(), mesh.cells["tetra"].numpy()
    g = np.random.default_rng(4).normal(size=el.shape[0])
    for mag in (1e150, 1e-150):
        check(pts, el, "tetra", "laplace", mag * np.exp(g))
    mixed = np.exp(g) * np.where(np.arange(el.shape[0]) % 97 == 0, 1e80, 1.0)
    check(pts, el, "tetra", "laplace", mixed)


@pytest.mark.parametrize("height", [20.0, 200.0])
def test_sliver_fan(height):
    """A bipyramid fan of 30 needles (ring radius 1, apexes at +-height):
    conditioning proxies of 1e4 .. 1e7, taken by the native-FP64 element path."""
    ring = 30
    t = np.arange(ring) * 2 * np.pi / ring
    pts = np.concatenate([[[0.0, 0.0, -height], [0.0, 0.0, height]],
                          np.stack([np.cos(t), np.sin(t), 0.1 * np.sin(3 * t)], 1)])
    el = np.array([[0, 2 + k, 2 + (k + 1) % ring, 1] for k in range(ring)], dtype=np.int64)
    kappa = np.exp(np.random.default_rng(ring).normal(size=ring))
    for form in ("laplace", "elasticity"):
        check(pts, el, "tetra", form, kappa)
