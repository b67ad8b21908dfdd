"""Parity of the CUDA assembly against the reference's own outputs (golden
fixtures) and the CPU oracle.

Bars: CSR indptr/indices bit-exact; values within 1e-12 relative (max-norm
over nnz relative to max|K|) for float64 (both the emulated double-float
path and native FP64), within 1e-5 relative for float32; bitwise
determinism run to run."""
import math

import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from oracle import fem

pytestmark = pytest.mark.gpu
DEV = "cuda"
ETYPES = ["triangle", "triangle6", "tetra", "tetra10"]
TOL = {torch.float64: 1e-12, torch.float32: 1e-5}


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def golden_mesh(golden, etype, dtype=torch.float64):
    pts = torch.tensor(golden[f"{etype}/points"], dtype=dtype, device=DEV)
    el = torch.tensor(golden[f"{etype}/elements"], device=DEV)
    return tg.Mesh(points=pts, cells={etype: el},
                   point_data={"is_boundary": torch.tensor(golden[f"{etype}/boundary"], device=DEV)})


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


def build_case(mesh, etype, case, q, coef):
    if case == "laplace":
        return tg.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=q)(mesh.points)
    if case == "mass":
        return tg.MassElementAssembler.from_mesh(mesh, quadrature_order=q)(mesh.points)
    if case == "elasticity":
        return tg.LinearElasticityElementAssembler.from_mesh(mesh, quadrature_order=q, E=2.5, nu=0.3)(mesh.points)
    cls = {"laplace_kappa": KappaLaplace, "mass_kappa": KappaMass, "elasticity_E": EElasticity}[case]
    key = "E" if case == "elasticity_E" else "kappa"
    return cls.from_mesh(mesh, quadrature_order=q)(mesh.points, element_data={key: coef})


@pytest.mark.parametrize("precision", ["emulated", "native"])
@pytest.mark.parametrize("etype", ETYPES)
@pytest.mark.parametrize("case", ["laplace", "mass", "elasticity", "laplace_kappa", "mass_kappa", "elasticity_E"])
@pytest.mark.parametrize("q", [1, 2, 3])
def test_assembly_matches_reference_fp64(golden, etype, case, q, precision):
    mesh = golden_mesh(golden, etype)
    coef = torch.tensor(golden[f"{etype}/coef"], device=DEV)
    tg.ElementAssembler.precision = precision
    try:
        K = build_case(mesh, etype, case, q, coef)
    finally:
        tg.ElementAssembler.precision = "emulated"
    key = f"{etype}/{case}/q{q}"
    np.testing.assert_array_equal(K.indptr.cpu().numpy(), golden[key + "/indptr"])
    np.testing.assert_array_equal(K.indices.cpu().numpy(), golden[key + "/indices"])
    err = rel_err(K.values.cpu().numpy(), golden[key + "/data"])
    assert err <= 1e-12, f"{key} {precision}: rel err {err:.3e}"


@pytest.mark.parametrize("etype", ETYPES)
@pytest.mark.parametrize("case", ["laplace", "mass", "elasticity_E"])
def test_assembly_fp32_variant(golden, etype, case):
    mesh = golden_mesh(golden, etype, torch.float32)
    coef = torch.tensor(golden[f"{etype}/coef"], device=DEV, dtype=torch.float32)
    K = build_case(mesh, etype, case, 2, coef)
    key = f"{etype}/{case}/q2"
    np.testing.assert_array_equal(K.indices.cpu().numpy(), golden[key + "/indices"])
    err = rel_err(K.values.cpu().numpy(), golden[key + "/data"])
    assert err <= 1e-5, f"{key}: fp32 rel err vs fp64 reference {err:.3e}"


@pytest.mark.parametrize("etype", ETYPES)
@pytest.mark.parametrize("q", [1, 2, 3])
def test_loads_match_reference(golden, etype, q):
    mesh = golden_mesh(golden, etype)
    dim = mesh.dim

    class PointLoad(tg.NodeAssembler):
        def forward(self, v, f):
            return v * f

    f_nodes = torch.tensor(golden[f"{etype}/f_nodes"], device=DEV)
    got = {
        "const": tg.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=q)(mesh.points),
        "func": tg.func_node_assembler(
            lambda x: 2 * math.pi ** 2 * torch.sin(math.pi * x[..., 0]) * torch.sin(math.pi * x[..., 1])
        ).from_mesh(mesh, quadrature_order=q)(mesh.points),
        "point": PointLoad.from_mesh(mesh, quadrature_order=q)(mesh.points, point_data={"f": f_nodes}),
        "vector": tg.const_node_assembler(torch.tensor([0.5, -1.0] if dim == 2 else [0.0, 0.3, -1.0],
                                                       dtype=torch.float64)).from_mesh(mesh, quadrature_order=q)(
            mesh.points),
    }
    for name, v in got.items():
        ref = golden[f"{etype}/load_{name}/q{q}"]
        assert tuple(v.shape) == ref.shape, name
        assert rel_err(v.cpu().numpy(), ref) <= 1e-12, name


@pytest.mark.parametrize("etype", ETYPES)
def test_assembly_matches_oracle_jittered_larger(etype):
    """A larger jittered mesh (more patches) against the oracle."""
    base = tg.Mesh.gen_unit_square(23) if etype.startswith("tri") else tg.Mesh.gen_unit_cube(7)
    if etype.endswith(("6", "10")):
        base = base.to_p2()
    g = torch.Generator().manual_seed(5)
    pts = base.points + 0.15 / 23 * (torch.rand(base.points.shape, generator=g, dtype=torch.float64) - 0.5)
    el = base.cells[etype]
    kappa = torch.exp(torch.randn(el.shape[0], generator=g, dtype=torch.float64))
    mesh = tg.Mesh(points=pts.to(DEV), cells={etype: el.to(DEV)})
    K = KappaLaplace.from_mesh(mesh, quadrature_order=2)(mesh.points, element_data={"kappa": kappa.to(DEV)})
    ip, ix, dv = fem.assemble_csr(pts.numpy(), el.numpy(), etype, "laplace", 2, coef=kappa.numpy())
    np.testing.assert_array_equal(K.indptr.cpu().numpy(), ip)
    np.testing.assert_array_equal(K.indices.cpu().numpy(), ix)
    assert rel_err(K.values.cpu().numpy(), dv) <= 1e-12


def test_assembly_is_bitwise_deterministic():
    mesh = tg.Mesh.gen_unit_cube(12, device=DEV)
    kappa = torch.exp(torch.randn(mesh.n_elements, device=DEV, dtype=torch.float64))
    asm = KappaLaplace.from_mesh(mesh, quadrature_order=1)
    ref = asm(mesh.points, element_data={"kappa": kappa}).values.clone()
    for _ in range(5):
        v = asm(mesh.points, element_data={"kappa": kappa}).values
        assert torch.equal(v, ref)


def test_unknown_form_raises():
    mesh = tg.Mesh.gen_unit_square(4, device=DEV)

    class Weird(tg.ElementAssembler):
        def forward(self, gradu, gradv):
            return (gradu @ gradv) ** 2

    with pytest.raises(NotImplementedError):
        Weird.from_mesh(mesh)(mesh.points)

    class BadKey(tg.ElementAssembler):
        def forward(self, gradu, gradv, nope):
            return gradu @ gradv

    with pytest.raises(ValueError):
        BadKey.from_mesh(mesh)(mesh.points)


def test_cpu_tensors_fail_loudly():
    mesh = tg.Mesh.gen_unit_square(4)
    with pytest.raises(RuntimeError):
        tg.LaplaceElementAssembler.from_mesh(mesh)(mesh.points)


@pytest.mark.parametrize("ring", [40, 250])
def test_high_valence_rows_match_oracle(ring):
    """A bipyramid fan of tetrahedra: both apexes touch every ring node, so
    their rows hold ring + 2 entries.  40 exceeds the 32-bit incidence record
    (64-bit records in the P1-tet kernel); 250 exceeds that kernel's shared
    memory (the generic kernel takes the launch).  The 250-fan's elements are
    slivers (ring edge 0.025 against height 1): the double-float default
    hands their patches to native FP64 and meets 1e-12; float32 meets 1e-3
    there (the element algebra amplifies its rounding by the aspect ratio)."""
    t = np.arange(ring) * 2 * np.pi / ring
    pts = np.concatenate([[[0.0, 0.0, -1.0], [0.0, 0.0, 1.0]],
                          np.stack([np.cos(t), np.sin(t), 0.1 * np.sin(3 * t)], 1)])
    el = np.array([[0, 2 + k, 2 + (k + 1) % ring, 1] for k in range(ring)], dtype=np.int64)
    g = np.random.default_rng(ring).normal(size=ring)
    kappa = np.exp(g)
    mesh = tg.Mesh(points=torch.tensor(pts, device=DEV), cells={"tetra": torch.tensor(el, device=DEV)})
    for cls, key, form in ((KappaLaplace, "kappa", "laplace"), (EElasticity, "E", "elasticity")):
        ip, ix, dv = fem.assemble_csr(pts, el, "tetra", form, 1, coef=kappa)
        sliver = ring > 40
        cases = [(torch.float64, "emulated", 1e-12),
                 (torch.float32, "emulated", 1e-3 if sliver else 1e-5)]
        if sliver:
            cases.append((torch.float64, "native", 1e-12))
        for dt, precision, tol in cases:
            asm = cls.from_mesh(mesh, quadrature_order=1)
            asm.precision = precision
            K = asm(mesh.points.to(dt), element_data={key: torch.tensor(kappa, dtype=dt, device=DEV)})
            assert np.array_equal(K.indptr.cpu().numpy(), ip) and np.array_equal(K.indices.cpu().numpy(), ix)
            assert rel_err(K.values.cpu().numpy(), dv) <= tol, (form, dt, precision)


@pytest.mark.parametrize("etype", ETYPES)
def test_pattern_kernels_match_host_definition(etype):
    """tm_pattern_count / tm_pattern_fill: indptr, indices and the slot map
    equal the host (torch) definition bit for bit, for shuffled element
    orders and rows with more candidate columns than the kernel keeps in
    registers (a 250-needle fan) or none at all (a node in no element)."""
    from tensormesh_gb300.plan import node_pattern
    base = tg.Mesh.gen_unit_square(13) if etype.startswith("tri") else tg.Mesh.gen_unit_cube(5)
    mesh = base.to_p2() if etype.endswith(("6", "10")) else base
    el = mesh.cells[etype]
    perm = torch.randperm(el.shape[0], generator=torch.Generator().manual_seed(1))
    cases = [(el, mesh.n_points), (el[perm], mesh.n_points)]
    if etype == "tetra":
        ring = 250
        fan = torch.tensor([[0, 2 + k, 2 + (k + 1) % ring, 1] for k in range(ring)])
        cases.append((fan, ring + 3))
    for e, n in cases:
        host = node_pattern(e, n)
        dev = node_pattern(e.to(DEV), n)
        assert torch.equal(dev.indptr.cpu(), host.indptr)
        assert torch.equal(dev.indices.cpu(), host.indices)
        assert torch.equal(dev.slots.cpu(), host.slots)


@pytest.mark.parametrize("dim", [2, 3])
def test_morton_key_kernel_matches_host_definition(dim):
    """tm_morton_keys against the torch definition of morton_keys on the
    host, bit for bit: random points, a regular grid (ties of the
    quantisation round half to even) and a degenerate axis (zero span)."""
    from tensormesh_gb300.plan import morton_keys, morton_parts
    g = torch.Generator().manual_seed(dim)
    grid = torch.stack(torch.meshgrid(*[torch.arange(9, dtype=torch.float64) / 8] * dim, indexing="ij"), -1)
    flat = torch.rand(500, dim, generator=g, dtype=torch.float64)
    flat[:, 0] = 0.25
    for c in (torch.rand(20000, dim, generator=g, dtype=torch.float64) * 7 - 3, grid.reshape(-1, dim), flat):
        lo, hi = c.min(0).values.contiguous(), c.max(0).values.contiguous()
        bits = 63 // dim
        host = morton_keys(c, lo, hi, bits)
        dev = morton_keys(c.to(DEV), lo.to(DEV), hi.to(DEV), bits)
        assert torch.equal(dev.cpu(), host)
        assert torch.equal(morton_parts(c.to(DEV), 64).cpu(), morton_parts(c, 64))
