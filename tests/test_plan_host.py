"""Host-side logic on the CPU: structured meshes, the canonical pattern, the
block expansion and the patch plan.  The patch plan is checked by replaying
the kernel's gather order (phase B of the assembly kernel) in numpy with the
oracle's element matrices: it must reproduce the oracle CSR exactly in
pattern and to rounding in values."""
import numpy as np
import pytest
import torch

from oracle import fem
from tensormesh_gb300 import Mesh
from tensormesh_gb300.plan import PatchPlan, block_pattern, node_pattern


def _meshes():
    sq = Mesh.gen_unit_square(5)
    cu = Mesh.gen_unit_cube(3)
    return {"triangle": sq, "triangle6": sq.to_p2(), "tetra": cu, "tetra10": cu.to_p2()}


def test_structured_meshes_match_fixture_numbering(golden):
    """The generators reproduce the numbering of the golden meshes (built by
    the fixture script with its own code)."""
    c1 = Mesh.gen_unit_square(64)
    np.testing.assert_array_equal(c1.cells["triangle"].numpy(), golden["c1/elements"])
    np.testing.assert_allclose(c1.points.numpy(), golden["c1/points"], rtol=0, atol=0)
    np.testing.assert_array_equal(c1.boundary_mask.numpy(), golden["c1/boundary"])


def test_kuhn_cube_counts():
    m = Mesh.gen_unit_cube(4)
    assert m.cells["tetra"].shape == (6 * 64, 4)
    p = node_pattern(m.cells["tetra"], m.n_points)
    n = 4
    assert p.nnz == (n + 1) ** 3 + 2 * (3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1) + n ** 3)
    # every Kuhn tet has the same volume 1/(6 n^3) and covers the cube
    X = m.points[m.cells["tetra"]].double()
    vol = torch.det(X[:, 1:] - X[:, :1]).abs() / 6
    assert torch.allclose(vol, torch.full_like(vol, 1 / (6 * n ** 3)))


@pytest.mark.parametrize("etype", ["triangle", "triangle6", "tetra", "tetra10"])
def test_pattern_matches_oracle(etype):
    m = _meshes()[etype]
    el = m.cells[etype]
    p = node_pattern(el, m.n_points)
    ip, ix, slots = fem.node_pattern(el.numpy(), m.n_points)
    np.testing.assert_array_equal(p.indptr.numpy(), ip)
    np.testing.assert_array_equal(p.indices.numpy(), ix)
    np.testing.assert_array_equal(p.slots.numpy(), slots)
    for H in (2, 3):
        dp, di = block_pattern(p.indptr, p.indices, H)
        op, oi = fem.block_pattern(ip, ix, H)
        np.testing.assert_array_equal(dp.numpy(), op)
        np.testing.assert_array_equal(di.numpy(), oi)


def replay_plan(plan: PatchPlan, Ke: np.ndarray, nnz: int) -> np.ndarray:
    """numpy replay of the kernel's phase B + write-out for scalar forms."""
    out = np.full(nnz, np.nan)
    B = plan.n_basis
    rptr, rows, racc = plan.rptr.numpy(), plan.rows.numpy(), plan.racc.numpy()
    eptr, elem = plan.eptr.numpy(), plan.elem.numpy()
    iptr = plan.iptr.numpy()
    inc_elem = plan.inc_elem.numpy().astype(np.int64) & 0xFFFF
    inc_a = plan.inc_a.numpy()
    inc_pos = plan.inc_pos.numpy().reshape(-1, B)
    indptr = plan.indptr.numpy()
    for p in range(plan.n_patches):
        for lr in range(rptr[p], rptr[p + 1]):
            r = rows[lr]
            deg = indptr[r + 1] - indptr[r]
            acc = np.zeros(deg)
            prev = -1
            for k in range(iptr[lr], iptr[lr + 1]):
                le = inc_elem[k]
                assert le > prev  # sorted by element, as phase B requires
                prev = le
                e = elem[eptr[p] + le]
                a = inc_a[k]
                for b in range(B):
                    acc[inc_pos[k, b]] += Ke[e, a, b]
            out[indptr[r]:indptr[r + 1]] = acc
    return out


@pytest.mark.parametrize("etype", ["triangle", "triangle6", "tetra", "tetra10"])
@pytest.mark.parametrize("budget", [64, 300, 100000])
def test_patch_plan_replay_reproduces_oracle(etype, budget):
    m = _meshes()[etype]
    el = m.cells[etype]
    pts = m.points.numpy()
    p = node_pattern(el, m.n_points)
    plan = PatchPlan(el, m.points, p, slot_budget=budget)
    assert plan.n_incidences == el.shape[0] * el.shape[1]
    # every row owned exactly once
    assert sorted(plan.rows.tolist()) == list(range(m.n_points))
    # local connectivity round-trips to the global one
    econn = plan.econn.numpy().astype(np.int64) & 0xFFFF
    vptr, vtx, eptr = plan.vptr.numpy(), plan.vtx.numpy(), plan.eptr.numpy()
    for pp in range(plan.n_patches):
        for le in range(eptr[pp], eptr[pp + 1]):
            e = plan.elem[le].item()
            np.testing.assert_array_equal(vtx[vptr[pp] + econn[le]], el[e].numpy())
    Ke = fem.element_matrices(pts, el.numpy(), etype, "laplace", 2)
    ip, ix, dv = fem.assemble_csr(pts, el.numpy(), etype, "laplace", 2)
    got = replay_plan(plan, Ke, ix.shape[0])
    assert np.max(np.abs(got - dv)) <= 1e-13 * np.max(np.abs(dv))


def replay_packed(plan: PatchPlan, Ke: np.ndarray, nnz: int, bits32: bool) -> np.ndarray:
    """numpy replay of the P1-tet kernel's phase B from the packed records
    (inc_pack / inc_pack32 and rdiag), in the kernel's chunked order."""
    out = np.full(nnz, np.nan)
    rec = (plan.inc_pack32.numpy().astype(np.int64) & 0xFFFFFFFF) if bits32 else plan.inc_pack.numpy()
    emask, ash, psh, pw = (0x7FFF, 15, 17, 5) if bits32 else (0xFFFF, 16, 18, 8)
    rptr, rows, racc = plan.rptr.numpy(), plan.rows.numpy(), plan.racc.numpy()
    eptr, elem, iptr = plan.eptr.numpy(), plan.elem.numpy(), plan.iptr.numpy()
    rdiag, indptr = plan.rdiag.numpy(), plan.indptr.numpy()
    for p in range(plan.n_patches):
        for lr in range(rptr[p], rptr[p + 1]):
            r = rows[lr]
            acc = np.zeros(indptr[r + 1] - indptr[r])
            for k in range(iptr[lr], iptr[lr + 1]):
                w = int(rec[k])
                le, a = w & emask, (w >> ash) & 3
                e = elem[eptr[p] + le]
                acc[rdiag[lr]] += Ke[e, a, a]
                for j in range(3):
                    b = (a + 1 + j) % 4
                    acc[(w >> (psh + pw * j)) & ((1 << pw) - 1)] += Ke[e, a, b]
            out[indptr[r]:indptr[r + 1]] = acc
    return out


@pytest.mark.parametrize("budget", [64, 300, 100000])
def test_packed_tet_records_reproduce_oracle(budget):
    m = _meshes()["tetra"]
    el = m.cells["tetra"]
    pts = m.points.numpy()
    p = node_pattern(el, m.n_points)
    plan = PatchPlan(el, m.points, p, slot_budget=budget)
    assert plan.inc_pack is not None and plan.inc_pack32 is not None and plan.rdiag is not None
    assert plan.max_rows <= 256
    Ke = fem.element_matrices(pts, el.numpy(), "tetra", "laplace", 2)
    ip, ix, dv = fem.assemble_csr(pts, el.numpy(), "tetra", "laplace", 2)
    for bits32 in (False, True):
        got = replay_packed(plan, Ke, ix.shape[0], bits32)
        assert np.max(np.abs(got - dv)) <= 1e-13 * np.max(np.abs(dv))


def test_rcb_partition_any_number_of_parts_is_balanced():
    from tensormesh_gb300.plan import rcb_partition
    g = torch.Generator().manual_seed(0)
    c = torch.rand(20000, 3, generator=g, dtype=torch.float64)
    for P in (1, 3, 7, 64, 391):
        part = rcb_partition(c, n_parts=P)
        cnt = torch.bincount(part, minlength=P)
        assert int(part.max()) + 1 == P
        assert int(cnt.max()) - int(cnt.min()) <= 1


def test_morton_parts_are_octree_cells():
    from tensormesh_gb300.plan import morton_parts
    i = torch.arange(1, 32, dtype=torch.float64) / 32
    pts = torch.stack(torch.meshgrid(i, i, i, indexing="ij"), -1).reshape(-1, 3)
    part = morton_parts(pts, 64)
    cnt = torch.bincount(part)
    assert int(cnt.max()) <= 2 * 64 and int(part.max()) + 1 == cnt.shape[0]
    # every part is an axis-aligned box of grid points (a cell of the octree)
    for k in range(0, int(part.max()) + 1, 37):
        sel = pts[part == k] * 32
        ext = (sel.max(0).values - sel.min(0).values + 1).round().long()
        assert int(ext.prod()) == sel.shape[0]


def test_morton_keys_interleave_the_quantised_coordinates():
    """The host definition of the Z-order keys against a scalar restatement:
    q_d = round-half-even((x_d - lo_d) / (hi_d - lo_d) * (2^bits - 1)), bit b
    of q_d at key bit b D + d."""
    from tensormesh_gb300.plan import morton_keys
    g = torch.Generator().manual_seed(5)
    for D in (2, 3):
        c = torch.rand(300, D, generator=g, dtype=torch.float64) * 5 - 2
        lo, hi = c.min(0).values, c.max(0).values
        bits = 63 // D
        got = morton_keys(c, lo, hi, bits).tolist()
        scale = float((1 << bits) - 1)
        for i in range(c.shape[0]):
            key = 0
            for d in range(D):
                q = round(float((c[i, d] - lo[d]) / (hi[d] - lo[d])) * scale)   # Python round: half to even
                for b in range(bits):
                    key |= ((q >> b) & 1) << (b * D + d)
            assert got[i] == key
