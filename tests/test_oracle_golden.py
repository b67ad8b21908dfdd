"""Pin the CPU oracle to fixtures produced by the reference package itself
(tests/golden/make_golden.py): same CSR pattern, values within 1e-12
relative (max-norm over nnz, relative to max|K|)."""
import math

import numpy as np
import pytest

from oracle import fem

ETYPES = ["triangle", "triangle6", "tetra", "tetra10"]
CASES = ["laplace", "mass", "elasticity", "laplace_kappa", "mass_kappa", "elasticity_E"]


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("etype", ETYPES)
@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("q", [1, 2, 3])
def test_oracle_matches_reference_assembly(golden, etype, case, q):
    pts = golden[f"{etype}/points"]
    el = golden[f"{etype}/elements"]
    coef = golden[f"{etype}/coef"]
    form = case.split("_")[0]
    c = None
    if case == "elasticity":
        c = 2.5
    elif case != form:
        c = coef
    ip, ix, dv = fem.assemble_csr(pts, el, etype, form, q, coef=c, nu=0.3)
    key = f"{etype}/{case}/q{q}"
    np.testing.assert_array_equal(ip, golden[key + "/indptr"])
    np.testing.assert_array_equal(ix, golden[key + "/indices"])
    assert rel_err(dv, golden[key + "/data"]) <= 1e-12


@pytest.mark.parametrize("etype", ETYPES)
@pytest.mark.parametrize("q", [1, 2, 3])
def test_oracle_matches_reference_loads(golden, etype, q):
    pts = golden[f"{etype}/points"]
    el = golden[f"{etype}/elements"]
    dim = pts.shape[1]
    f = lambda x: 2 * math.pi ** 2 * np.sin(math.pi * x[..., 0]) * np.sin(math.pi * x[..., 1])  # noqa: E731
    got = {
        "const": fem.assemble_load(pts, el, etype, q, "const", 1.0),
        "func": fem.assemble_load(pts, el, etype, q, "func", f),
        "point": fem.assemble_load(pts, el, etype, q, "point", golden[f"{etype}/f_nodes"]),
        "vector": fem.assemble_load(pts, el, etype, q, "const", [0.5, -1.0] if dim == 2 else [0.0, 0.3, -1.0]),
    }
    for name, v in got.items():
        ref = golden[f"{etype}/load_{name}/q{q}"]
        assert v.shape == ref.shape, name
        assert rel_err(v, ref) <= 1e-12, name


def test_scalar_pattern_is_reference_edge_order(golden):
    """The reference's scalar ``edges`` are already canonical CSR order
    (element_assembler.py:851-856): row-major, sorted columns."""
    for etype in ETYPES:
        e = golden[f"{etype}/ref_edges"]
        ip, ix, _ = fem.node_pattern(golden[f"{etype}/elements"], golden[f"{etype}/points"].shape[0])
        rows = np.repeat(np.arange(ip.shape[0] - 1), np.diff(ip))
        np.testing.assert_array_equal(e[0], rows)
        np.testing.assert_array_equal(e[1], ix)


def test_oracle_c1_poisson_pipeline(golden):
    pts, el, bd = golden["c1/points"], golden["c1/elements"], golden["c1/boundary"]
    ip, ix, dv = fem.assemble_csr(pts, el, "triangle", "laplace", 1)
    np.testing.assert_array_equal(ip, golden["c1/K_indptr"])
    np.testing.assert_array_equal(ix, golden["c1/K_indices"])
    assert rel_err(dv, golden["c1/K_data"]) <= 1e-12
    f = lambda x: 2 * math.pi ** 2 * np.sin(math.pi * x[..., 0]) * np.sin(math.pi * x[..., 1])  # noqa: E731
    b = fem.assemble_load(pts, el, "triangle", 1, "func", f)
    assert rel_err(b, golden["c1/b"]) <= 1e-12
    iptr, iind, ival, fi = fem.condense(ip, ix, dv, bd, None, b)
    np.testing.assert_array_equal(iptr, golden["c1/Kii_indptr"])
    np.testing.assert_array_equal(iind, golden["c1/Kii_indices"])
    assert rel_err(ival, golden["c1/Kii_data"]) <= 1e-12
    assert rel_err(fi, golden["c1/f_i"]) <= 1e-12
    u = fem.recover(fem.spsolve(iptr, iind, ival, fi), bd)
    assert rel_err(u, golden["c1/u"]) <= 1e-10
    # PCG reaches the same solution
    x, it, res = fem.pcg_jacobi(iptr, iind, ival, fi, rtol=1e-12)
    assert res <= 1e-11
    assert rel_err(fem.recover(x, bd), golden["c1/u"]) <= 1e-9


def test_oracle_adjoint_kappa_matches_reference_autograd(golden):
    pts, el, bd, kappa = golden["adj/points"], golden["adj/elements"], golden["adj/boundary"], golden["adj/kappa"]
    u = golden["adj/u"]
    g = fem.compliance_gradients_kappa(pts, el, "triangle", 1, kappa, u)
    assert rel_err(g, golden["adj/dJ_dkappa"]) <= 1e-10


@pytest.mark.parametrize("etype", ETYPES)
@pytest.mark.parametrize("q", [1, 2])
def test_oracle_neo_hookean_matches_reference_energy_and_autograd(golden, etype, q):
    """NeoHookeanModel.energy(u) and u.grad from the reference's autograd."""
    pts, el, u = golden[f"{etype}/points"], golden[f"{etype}/elements"], golden[f"{etype}/nh/u"]
    e, g = fem.neo_hookean(pts, el, etype, q, u, 2.0, 0.3)
    e_ref = float(golden[f"{etype}/nh/q{q}/energy"])
    g_ref = golden[f"{etype}/nh/q{q}/grad_u"]
    assert abs(e - e_ref) <= 1e-12 * abs(e_ref)
    assert np.max(np.abs(g - g_ref)) <= 1e-12 * np.max(np.abs(g_ref))


def test_oracle_neo_hookean_zero_displacement_has_zero_energy(golden):
    """tests/assemble/test_builtin.py:116-125 of the reference, as an invariant."""
    pts, el = golden["triangle/points"], golden["triangle/elements"]
    e, g = fem.neo_hookean(pts, el, "triangle", 2, np.zeros_like(pts), 1.0, 0.3)
    assert abs(e) <= 1e-14 and np.max(np.abs(g)) <= 1e-14


FACET_MESHES = ["triangle", "triangle6", "tetra", "tetra10", "triangle6c", "tetra10c"]


def facet_cases(g, et):
    """(kind, value, mask) per fixture case (the forwards of make_golden.py's
    facet_fixtures)."""
    pts = g[f"{et}/points"]
    dim = pts.shape[1]
    bd, top = g[f"{et}/boundary"], g[f"{et}/top"]
    return {
        "const": ("const", 1.0, bd),
        "vector": ("const", [0.5, -1.0] if dim == 2 else [0.0, 0.3, -1.0], bd),
        "func": ("func", lambda x: np.sin(math.pi * x[..., 0]) + x[..., 1] ** 2, bd),
        "point": ("point", g[f"{et}/facet_g"], bd),
        "top": ("const", 1.0, top),
    }


@pytest.mark.parametrize("et", FACET_MESHES)
@pytest.mark.parametrize("q", [1, 2, 3, 4])
def test_oracle_facet_loads_match_reference(golden_facet, et, q):
    """With the reference's own float32 facet table the restatement reproduces
    the reference to rounding; with the exact float64 table (what the GPU path
    uses) the difference is the reference table's float32 rounding."""
    g = golden_facet
    etype = et.rstrip("c")
    fam = "triangle" if etype.startswith("tri") else "tetra"
    table = (g[f"facet_table/{fam}/q{q}/w"], g[f"facet_table/{fam}/q{q}/p"])
    pts, el = g[f"{et}/points"], g[f"{et}/elements"]
    for case, (kind, val, mask) in facet_cases(g, et).items():
        ref = g[f"{et}/facet_{case}/q{q}"]
        got = fem.facet_load(pts, el, etype, mask, q, kind, val, tables=table)
        assert rel_err(got, ref) <= 1e-12, (case, rel_err(got, ref))
        exact = fem.facet_load(pts, el, etype, mask, q, kind, val)
        assert rel_err(exact, ref) <= 1e-6, (case, rel_err(exact, ref))


def test_oracle_facet_selection_includes_interior_facets(golden_facet):
    """The reference selects every facet whose nodes are all flagged: on the
    4 x 4 square the corner-cell diagonals joining two boundary nodes are
    integrated from both sides (boundary length 4 + 2 * 2 * sqrt(2) / 4)."""
    g = golden_facet
    tot = fem.facet_load(g["triangle/points"], g["triangle/elements"], "triangle", g["triangle/boundary"], 2,
                         "const", 1.0).sum()
    assert abs(tot - (4 + math.sqrt(2))) < 1e-12
    assert abs(g["triangle/facet_const/q2"].sum() - tot) < 1e-12


def test_oracle_condenser_with_prescribed_values(golden_condense):
    """Nonzero Dirichlet values: f_i = f[inner] - K_io u_o, recover writes the
    values; update_dirichlet + condense_rhs re-condense with new values
    (operator/condense.py:222-236, 238-309, 388-458)."""
    g = golden_condense
    pts, el, bd = g["dir/points"], g["dir/elements"], g["dir/boundary"]
    ip, ix, dv = fem.assemble_csr(pts, el, "triangle", "laplace", 2)
    b = fem.assemble_load(pts, el, "triangle", 2, "const", 1.0)
    for val, f_key, u_key in ((g["dir/g_full"], "dir/f_i", "dir/u"), (g["dir/g2_outer"], "dir/f_i2", "dir/u2")):
        iptr, ic, iv, f_i = fem.condense(ip, ix, dv, bd, val, b)
        assert rel_err(f_i, g[f_key]) <= 1e-12
        u = fem.recover(fem.spsolve(iptr, ic, iv, f_i), bd, val)
        assert rel_err(u, g[u_key]) <= 1e-10


def test_oracle_clamped_elasticity_pipeline(golden_condense):
    """Per-element-E elasticity, all three dofs clamped on x = 0, body force
    (0, 0, -1): K, the condensed system and the displacement."""
    g = golden_condense
    pts, el, E, clamp = g["c2/points"], g["c2/elements"], g["c2/E"], g["c2/clamp"]
    ip, ix, dv = fem.assemble_csr(pts, el, "tetra", "elasticity", 1, coef=E)
    np.testing.assert_array_equal(ip, g["c2/K_indptr"])
    np.testing.assert_array_equal(ix, g["c2/K_indices"])
    assert rel_err(dv, g["c2/K_data"]) <= 1e-12
    f = fem.assemble_load(pts, el, "tetra", 1, "const", [0.0, 0.0, -1.0])
    assert rel_err(f, g["c2/f"]) <= 1e-12
    iptr, ic, iv, f_i = fem.condense(ip, ix, dv, clamp, None, f)
    np.testing.assert_array_equal(iptr, g["c2/Kii_indptr"])
    np.testing.assert_array_equal(ic, g["c2/Kii_indices"])
    assert rel_err(iv, g["c2/Kii_data"]) <= 1e-12
    assert rel_err(f_i, g["c2/f_i"]) <= 1e-12
    u = fem.recover(fem.spsolve(iptr, ic, iv, f_i), clamp)
    assert rel_err(u, g["c2/u"]) <= 1e-10


@pytest.mark.parametrize("et", FACET_MESHES)
@pytest.mark.parametrize("q", [1, 2, 3, 4])
def test_package_reference_facet_rule_is_the_reference_table(golden_facet, et, q):
    """The package's default facet rule carries the reference's float32 table
    (weights and points bit for bit), and the oracle run on the package's
    tables reproduces the reference's facet loads to rounding."""
    from tensormesh_gb300.facet import facet_tables
    g = golden_facet
    etype = et.rstrip("c")
    fam = "triangle" if etype.startswith("tri") else "tetra"
    w, _, _, xi = facet_tables(etype, q, "reference")
    assert np.array_equal(w, g[f"facet_table/{fam}/q{q}/w"])
    assert np.array_equal(xi, g[f"facet_table/{fam}/q{q}/p"])
    pts, el = g[f"{et}/points"], g[f"{et}/elements"]
    for case, (kind, val, mask) in facet_cases(g, et).items():
        got = fem.facet_load(pts, el, etype, mask, q, kind, val, tables=(w, xi))
        assert rel_err(got, g[f"{et}/facet_{case}/q{q}"]) <= 1e-12, case
