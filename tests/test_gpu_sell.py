"""Jacobi-PCG over the SELL-32 copy (tm_sell_plan / tm_pcg_jacobi_sell, the
standard and the pipelined form) against the CSR kernel (tm_pcg_jacobi), the
oracle's PCG and the true FP64 residual, on ragged row counts (n not a multiple of 32, slices of uneven
rows) and the edge cases of the plan."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from tensormesh_gb300 import _lib, solve as S
from oracle import fem

pytestmark = pytest.mark.gpu
DEV = "cuda"


def poisson(n, dtype=torch.float64, seed=0):
    mesh = tg.Mesh.gen_unit_cube(n, device=DEV, dtype=dtype)
    g = torch.Generator().manual_seed(seed)
    kappa = torch.exp(torch.randn(mesh.n_elements, generator=g, dtype=torch.float64)).to(DEV, dtype)

    class KL(tg.ElementAssembler):
        def forward(self, gradu, gradv, kappa):
            return kappa * (gradu @ gradv)
    K = KL.from_mesh(mesh, quadrature_order=1)(mesh.points, element_data={"kappa": kappa})
    b = tg.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=1)(mesh.points)
    return tg.Condenser(mesh.boundary_mask)(K, b)


def random_spd(n, seed):
    """A ragged SPD CSR matrix: random sparse symmetric pattern with row
    lengths from 1 to ~40 and a dominant diagonal."""
    rng = np.random.default_rng(seed)
    A = np.zeros((n, n))
    for i in range(n):
        k = int(rng.integers(0, min(n, 20)))
        cols = rng.choice(n, size=k, replace=False)
        A[i, cols] = rng.normal(size=k)
    A = A + A.T
    np.fill_diagonal(A, 0.0)
    np.fill_diagonal(A, np.abs(A).sum(1) + rng.uniform(0.5, 2.0, size=n))
    ip = [0]
    ix, dv = [], []
    for i in range(n):
        nz = np.nonzero(A[i])[0]
        ix.extend(nz.tolist())
        dv.extend(A[i, nz].tolist())
        ip.append(len(ix))
    return np.array(ip, np.int64), np.array(ix, np.int32), np.array(dv)


def slice_plan_reference(indptr, n):
    lens = np.diff(indptr)
    ns = (n + 31) // 32
    w = np.zeros(ns + 1, np.int64)
    for s in range(ns):
        w[s + 1] = 32 * lens[32 * s:32 * s + 32].max()
    return np.cumsum(w)


@pytest.mark.parametrize("n", [1, 31, 33, 100, 257])
def test_sell_plan_and_solve_on_ragged_matrices(n):
    ip, ix, dv = random_spd(n, seed=n)
    indptr = torch.from_numpy(ip).to(DEV)
    indices = torch.from_numpy(ix).to(DEV)
    sp, n_pad, narrow = S.sell_plan(indptr, indices)
    ref = slice_plan_reference(ip, n)
    np.testing.assert_array_equal(sp.cpu().numpy(), ref)
    assert n_pad == int(ref[-1]) and narrow
    b = np.random.default_rng(n + 1).normal(size=n)
    values = torch.from_numpy(dv).to(DEV)
    x = torch.zeros(n, dtype=torch.float64, device=DEV)
    info = S.pcg_jacobi_raw(indptr, indices, values, torch.from_numpy(b).to(DEV), x, rtol=1e-12)
    assert info.status == 0 and info.residual <= 1e-12, info
    xo, _, _ = fem.pcg_jacobi(ip, ix.astype(np.int64), dv, b, rtol=1e-13)
    assert np.max(np.abs(x.cpu().numpy() - xo)) <= 1e-9 * np.max(np.abs(xo))


@pytest.mark.parametrize("dtype,rtol", [(torch.float64, 1e-10), (torch.float32, 1e-5)])
def test_sell_matches_csr_kernel(dtype, rtol, monkeypatch):
    """Standard PCG over the SELL copy runs the CSR kernel's recurrence:
    same iteration count up to rounding, same solution."""
    K_ii, f_i = poisson(20, dtype)
    out = {}
    for layout in ("csr", "sell"):
        monkeypatch.setattr(S, "LAYOUT", layout)
        x = torch.zeros_like(f_i)
        info = S.pcg_jacobi_raw(K_ii.indptr, K_ii.indices, K_ii.values, f_i, x, rtol=rtol)
        assert info.status == 0 and info.residual <= rtol * 1.0001, (layout, info)
        out[layout] = (x.double(), info)
    # same Krylov method: iteration counts agree up to rounding
    assert abs(out["sell"][1].iterations - out["csr"][1].iterations) <= 2 + out["csr"][1].iterations // 50
    xs, xc = out["sell"][0], out["csr"][0]
    tol = 1e-7 if dtype == torch.float64 else 1e-3
    assert float((xs - xc).abs().max() / xc.abs().max()) <= tol


def test_sell_nonzero_initial_guess_and_iteration_cap():
    K_ii, f_i = poisson(12)
    x0 = torch.randn_like(f_i)
    x = x0.clone()
    info = S.pcg_jacobi_raw(K_ii.indptr, K_ii.indices, K_ii.values, f_i, x, rtol=1e-11)
    assert info.status == 0 and info.residual <= 1e-11
    sp, n_pad, _ = S.sell_plan(K_ii.indptr, K_ii.indices)
    n = f_i.shape[0]
    ws = S.SellWorkspace(n, n_pad, torch.float64, f_i.device)
    x = torch.zeros_like(f_i)
    st = _lib.load().tm_pcg_jacobi_sell(_lib.TM_F64, n, K_ii.indptr.data_ptr(), K_ii.indices.data_ptr(),
                                        K_ii.values.data_ptr(), sp.data_ptr(), n_pad, f_i.data_ptr(),
                                        x.data_ptr(), 1e-14, 0.0, 3, _lib.TM_PCG_STANDARD, ws.buf.data_ptr(),
                                        ws.nbytes,
                                        _lib.stream_handle(f_i.device))
    assert st == 0
    it = _lib.ctypes.c_int32(0)
    res = _lib.ctypes.c_double(0.0)
    bn = _lib.ctypes.c_double(0.0)
    status = _lib.load().tm_pcg_result(ws.buf.data_ptr(), _lib.ctypes.byref(it), _lib.ctypes.byref(res),
                                       _lib.ctypes.byref(bn), _lib.stream_handle(f_i.device))
    assert status == _lib.TM_ERR_MAXITER and it.value == 3
    assert abs(bn.value - float(torch.linalg.vector_norm(f_i))) <= 1e-12 * bn.value


def test_sell_plan_of_another_pattern_is_rejected():
    """A slice plan whose widths do not cover the rows returns TM_ERR_INDEX
    through the solver record; the kernel writes and iterates nothing."""
    K_ii, f_i = poisson(8)
    n = f_i.shape[0]
    sp, n_pad, _ = S.sell_plan(K_ii.indptr, K_ii.indices)
    bad = sp.clone()
    bad[1:] = bad[1:] // 2 // 32 * 32       # half the widths: rows no longer fit
    bad[-1] = n_pad
    ws = S.SellWorkspace(n, n_pad, torch.float64, f_i.device)
    x = torch.zeros_like(f_i)
    lib = _lib.load()
    s = _lib.stream_handle(f_i.device)
    assert lib.tm_pcg_jacobi_sell(_lib.TM_F64, n, K_ii.indptr.data_ptr(), K_ii.indices.data_ptr(),
                                  K_ii.values.data_ptr(), bad.data_ptr(), n_pad, f_i.data_ptr(), x.data_ptr(),
                                  1e-8, 0.0, 100, 0, ws.buf.data_ptr(), ws.nbytes, s) == 0
    status = lib.tm_pcg_result(ws.buf.data_ptr(), None, None, None, s)
    assert status == _lib.TM_ERR_INDEX
    assert int(torch.count_nonzero(x)) == 0
    # a column index outside [0, n): rejected the same way, without a gather
    bad_idx = K_ii.indices.clone()
    bad_idx[5] = n + 7
    assert lib.tm_pcg_jacobi_sell(_lib.TM_F64, n, K_ii.indptr.data_ptr(), bad_idx.data_ptr(),
                                  K_ii.values.data_ptr(), sp.data_ptr(), n_pad, f_i.data_ptr(), x.data_ptr(),
                                  1e-8, 0.0, 100, 0, ws.buf.data_ptr(), ws.nbytes, s) == 0
    assert lib.tm_pcg_result(ws.buf.data_ptr(), None, None, None, s) == _lib.TM_ERR_INDEX
    assert int(torch.count_nonzero(x)) == 0
    # argument checks on the host
    assert lib.tm_pcg_jacobi_sell(_lib.TM_F64, n, K_ii.indptr.data_ptr(), K_ii.indices.data_ptr(),
                                  K_ii.values.data_ptr(), sp.data_ptr(), n_pad, f_i.data_ptr(), x.data_ptr(),
                                  1e-8, 0.0, 100, 0, ws.buf.data_ptr(), ws.nbytes - 1, s) == _lib.TM_ERR_INDEX
    assert lib.tm_pcg_jacobi_sell(7, n, K_ii.indptr.data_ptr(), K_ii.indices.data_ptr(),
                                  K_ii.values.data_ptr(), sp.data_ptr(), n_pad, f_i.data_ptr(), x.data_ptr(),
                                  1e-8, 0.0, 100, 0, ws.buf.data_ptr(), ws.nbytes, s) == _lib.TM_ERR_INVALID
    assert lib.tm_pcg_jacobi_sell(_lib.TM_F64, n, K_ii.indptr.data_ptr(), K_ii.indices.data_ptr(),
                                  K_ii.values.data_ptr(), sp.data_ptr(), n_pad, f_i.data_ptr(), x.data_ptr(),
                                  1e-8, 0.0, 100, 4, ws.buf.data_ptr(), ws.nbytes, s) == _lib.TM_ERR_INVALID


def test_sell_solve_is_bitwise_repeatable():
    K_ii, f_i = poisson(16)
    xs = []
    for _ in range(2):
        x = torch.zeros_like(f_i)
        S.pcg_jacobi_raw(K_ii.indptr, K_ii.indices, K_ii.values, f_i, x, rtol=1e-10)
        xs.append(x)
    assert torch.equal(xs[0], xs[1])


def test_pipelined_form_converges_in_double_float(monkeypatch):
    """The one-barrier pipelined form on an FP64 Poisson system: converged to
    the target true residual (restarting from its iterate after a breakdown)."""
    K_ii, f_i = poisson(20)
    monkeypatch.setattr(S, "LAYOUT", "sell-pipelined")
    x = torch.zeros_like(f_i)
    info = S.pcg_jacobi_raw(K_ii.indptr, K_ii.indices, K_ii.values, f_i, x, rtol=1e-10)
    assert info.status == 0 and info.residual <= 1e-10 * 1.0001, info
    monkeypatch.setattr(S, "LAYOUT", "sell")
    xr = torch.zeros_like(f_i)
    S.pcg_jacobi_raw(K_ii.indptr, K_ii.indices, K_ii.values, f_i, xr, rtol=1e-10)
    assert float((x - xr).abs().max() / xr.abs().max()) <= 1e-7


def test_wide_couplings_keep_32_bit_columns(monkeypatch):
    """A coupling farther than 32767 rows from the diagonal: the plan reports
    the pattern as wide, the solve takes 32-bit columns and converges; a
    caller that claims 16-bit columns anyway gets TM_ERR_INDEX."""
    n = 40000
    rows = np.arange(n)
    ip = np.zeros(n + 1, np.int64)
    cols, vals = [], []
    for i in range(n):           # tridiagonal, plus a coupling of rows 0 and n - 1
        row_c = [c for c in (i - 1, i, i + 1) if 0 <= c < n]
        if i == 0:
            row_c.append(n - 1)
        if i == n - 1:
            row_c.insert(0, 0)
        cols.extend(row_c)
        vals.extend([4.0 if c == i else -1.0 for c in row_c])
        ip[i + 1] = len(cols)
    indptr = torch.from_numpy(ip).to(DEV)
    indices = torch.tensor(cols, dtype=torch.int32, device=DEV)
    values = torch.tensor(vals, dtype=torch.float64, device=DEV)
    sp, n_pad, narrow = S.sell_plan(indptr, indices)
    assert not narrow
    b = torch.ones(n, dtype=torch.float64, device=DEV)
    x = torch.zeros_like(b)
    info = S.pcg_jacobi_raw(indptr, indices, values, b, x, rtol=1e-10)
    assert info.status == 0 and info.residual <= 1e-10
    ws = S.SellWorkspace(n, n_pad, torch.float64, b.device)
    lib = _lib.load()
    s = _lib.stream_handle(b.device)
    x = torch.zeros_like(b)
    assert lib.tm_pcg_jacobi_sell(_lib.TM_F64, n, indptr.data_ptr(), indices.data_ptr(), values.data_ptr(),
                                  sp.data_ptr(), n_pad, b.data_ptr(), x.data_ptr(), 1e-8, 0.0, 100,
                                  _lib.TM_PCG_NARROW, ws.buf.data_ptr(), ws.nbytes, s) == 0
    assert lib.tm_pcg_result(ws.buf.data_ptr(), None, None, None, s) == _lib.TM_ERR_INDEX
    assert int(torch.count_nonzero(x)) == 0


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_plain_sell_copy_and_product(dtype):
    """tm_sell_fill / tm_spmv_sell: y = A x on the plain SELL-32 copy equals
    the CSR product, with 16-bit offsets and with 32-bit columns."""
    K_ii, f_i = poisson(14)
    n = f_i.shape[0]
    sp, n_pad, narrow = S.sell_plan(K_ii.indptr, K_ii.indices)
    assert narrow
    vals = K_ii.values.to(dtype).contiguous()
    x = torch.randn(n, dtype=torch.float64, device=DEV).to(dtype)
    ref = S.spmv_raw(K_ii.indptr, K_ii.indices, vals, x)
    lib = _lib.load()
    s = _lib.stream_handle(f_i.device)
    code = _lib.TM_F64 if dtype == torch.float64 else _lib.TM_F32
    for nar in (1, 0):
        scol = torch.empty(n_pad, dtype=torch.int16 if nar else torch.int32, device=DEV)
        sval = torch.empty(n_pad, dtype=dtype, device=DEV)
        bad = torch.zeros(1, dtype=torch.int32, device=DEV)
        assert lib.tm_sell_fill(code, n, K_ii.indptr.data_ptr(), K_ii.indices.data_ptr(), vals.data_ptr(),
                                sp.data_ptr(), n_pad, nar, scol.data_ptr(), sval.data_ptr(), bad.data_ptr(), s) == 0
        assert int(bad.item()) == 0
        y = torch.empty_like(x)
        assert lib.tm_spmv_sell(code, n, sp.data_ptr(), nar, scol.data_ptr(), sval.data_ptr(), x.data_ptr(),
                                y.data_ptr(), s) == 0
        tol = 1e-14 if dtype == torch.float64 else 1e-6
        assert float((y - ref).abs().max() / ref.abs().max()) <= tol
    # a column outside [0, n) raises the flag
    bad_idx = K_ii.indices.clone()
    bad_idx[3] = -1
    bad = torch.zeros(1, dtype=torch.int32, device=DEV)
    assert lib.tm_sell_fill(code, n, K_ii.indptr.data_ptr(), bad_idx.data_ptr(), vals.data_ptr(), sp.data_ptr(),
                            n_pad, 1, scol.data_ptr(), sval.data_ptr(), bad.data_ptr(), s) == 0
    assert int(bad.item()) == 1
