"""Neo-Hookean energy assembly on the GPU (``NeoHookeanModel.energy`` and the
u-gradient its backward returns) against the reference's own values (golden
fixtures of its energy and autograd) and against the numpy oracle."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from oracle import fem

pytestmark = pytest.mark.gpu
DEV = "cuda"
ETYPES = ["triangle", "triangle6", "tetra", "tetra10"]


def mesh_of(pts, el, etype, dtype=torch.float64):
    return tg.Mesh(points=torch.tensor(pts, dtype=dtype, device=DEV),
                   cells={etype: torch.tensor(el, dtype=torch.int64, device=DEV)})


@pytest.mark.parametrize("etype", ETYPES)
@pytest.mark.parametrize("q", [1, 2])
def test_energy_and_force_match_reference(golden, etype, q):
    pts, el, u0 = golden[f"{etype}/points"], golden[f"{etype}/elements"], golden[f"{etype}/nh/u"]
    mesh = mesh_of(pts, el, etype)
    model = tg.NeoHookeanModel.from_mesh(mesh, quadrature_order=q, E=2.0, nu=0.3)
    u = torch.tensor(u0, device=DEV, requires_grad=True)
    e = model.energy(u)
    e.backward()
    e_ref = float(golden[f"{etype}/nh/q{q}/energy"])
    g_ref = golden[f"{etype}/nh/q{q}/grad_u"]
    assert abs(float(e.detach()) - e_ref) <= 1e-12 * abs(e_ref)
    g = u.grad.cpu().numpy()
    assert np.max(np.abs(g - g_ref)) <= 1e-12 * np.max(np.abs(g_ref))


@pytest.mark.parametrize("etype,n", [("tetra", 6), ("triangle", 24), ("tetra10", 3)])
def test_energy_matches_oracle_on_larger_meshes(etype, n):
    dim = 3 if etype.startswith("tetra") else 2
    base = tg.Mesh.gen_unit_cube(n) if dim == 3 else tg.Mesh.gen_unit_square(n)
    pts = base.points.numpy()
    el = base.cells["tetra" if dim == 3 else "triangle"].numpy()
    rng = np.random.default_rng(5)
    pts = pts + rng.uniform(-0.15, 0.15, pts.shape) / n * (~np.isclose(pts, 0) & ~np.isclose(pts, 1))
    if etype == "tetra10":
        pts, el, _ = to_p2(pts, el)     # straight edges: midside nodes at the midpoints
    amp = (0.02 if etype == "tetra10" else 0.1) / n      # small against the element size: no inversion
    u0 = amp * rng.normal(size=(pts.shape[0], dim))
    mesh = mesh_of(pts, el, etype)
    model = tg.NeoHookeanModel.from_mesh(mesh, quadrature_order=2, E=3.0, nu=0.35)
    u = torch.tensor(u0, device=DEV, requires_grad=True)
    e = model.energy(u)
    e.backward()
    e_o, g_o = fem.neo_hookean(pts, el, etype, 2, u0, 3.0, 0.35)
    assert abs(float(e.detach()) - e_o) <= 1e-12 * abs(e_o)
    assert np.max(np.abs(u.grad.cpu().numpy() - g_o)) <= 1e-12 * np.max(np.abs(g_o))


def to_p2(pts, cells):
    """P2 tetrahedra: midside nodes appended per unique edge, in the oracle's
    (and the reference's) local edge order."""
    pairs = np.stack([np.sort(cells[:, [a, b]], axis=1) for a, b in fem._TET_EDGES], 1)
    flat = pairs.reshape(-1, 2)
    key = flat[:, 0] * len(pts) + flat[:, 1]
    uniq, inv = np.unique(key, return_inverse=True)
    u0, u1 = uniq // len(pts), uniq % len(pts)
    new_pts = np.concatenate([pts, 0.5 * (pts[u0] + pts[u1])], 0)
    new_cells = np.concatenate([cells, len(pts) + inv.reshape(cells.shape[0], len(fem._TET_EDGES))], 1)
    return new_pts, new_cells, None


def test_zero_displacement_zero_energy_and_deterministic(golden):
    """tests/assemble/test_builtin.py:116-125 of the reference; repeated calls
    give the same bits."""
    pts, el = golden["tetra/points"], golden["tetra/elements"]
    mesh = mesh_of(pts, el, "tetra")
    model = tg.NeoHookeanModel.from_mesh(mesh, quadrature_order=2, E=1.0, nu=0.3)
    u = torch.zeros(mesh.points.shape[0], 3, dtype=torch.float64, device=DEV, requires_grad=True)
    e = model.energy(u)
    e.backward()
    assert abs(float(e.detach())) <= 1e-14 and float(u.grad.abs().max()) <= 1e-14
    u2 = torch.tensor(golden["tetra/nh/u"], device=DEV)
    assert torch.equal(model.energy(u2), model.energy(u2))


def test_float32_energy_within_float_tolerance(golden):
    pts, el, u0 = golden["tetra/points"], golden["tetra/elements"], golden["tetra/nh/u"]
    mesh = mesh_of(pts, el, "tetra", dtype=torch.float32)
    model = tg.NeoHookeanModel.from_mesh(mesh, quadrature_order=2, E=2.0, nu=0.3)
    u = torch.tensor(u0, dtype=torch.float32, device=DEV, requires_grad=True)
    e = model.energy(u)
    e.backward()
    e_ref = float(golden["tetra/nh/q2/energy"])
    assert abs(float(e.detach()) - e_ref) <= 1e-5 * abs(e_ref)
    g_ref = golden["tetra/nh/q2/grad_u"]
    assert np.max(np.abs(u.grad.cpu().numpy() - g_ref)) <= 1e-5 * np.max(np.abs(g_ref))


def test_other_densities_raise():
    mesh = tg.Mesh.gen_unit_square(4, device=DEV)

    class Other(tg.ElementAssembler):
        def element_energy(self, graddisplacement):
            return (graddisplacement ** 2).sum()

    with pytest.raises(NotImplementedError):
        Other.from_mesh(mesh, quadrature_order=1).energy(point_data={"displacement": torch.zeros_like(mesh.points)})
