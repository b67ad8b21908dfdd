"""Error behaviour of the C ABI that needs no GPU: sizing queries, and calls
whose arguments are rejected before any device work (negative sizes, NULL
pointers, unknown dtypes or flags) return TM_ERR_INVALID (or its negative for
the size queries), as include/tensormesh_gb300.h documents."""
import pytest

from tensormesh_gb300 import _lib

INV = _lib.TM_ERR_INVALID
FAKE = 1 << 20      # a non-NULL pointer value that a rejected call never dereferences


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def test_size_queries(lib):
    assert lib.tm_fcg_workspace_doubles() == 2 * 304 + 8
    a256 = lambda b: (b + 255) // 256 * 256
    for dt, es in ((_lib.TM_F64, 8), (_lib.TM_F32, 4)):
        n, n_pad = 1000, 1024 * 16
        assert lib.tm_pcg_sell_workspace_bytes(dt, n, n_pad) == (
            256 + a256(7 * 4096 * 8) + 9 * a256(n * es) + a256(n_pad * es) + a256(n_pad * 4))
    assert lib.tm_pcg_sell_workspace_bytes(99, 10, 32) == -INV
    assert lib.tm_pcg_sell_workspace_bytes(_lib.TM_F64, -1, 32) == -INV
    assert lib.tm_pcg_workspace_bytes(_lib.TM_F64, -1, 10, 8) == -INV
    assert lib.tm_pcg_workspace_bytes(7, 10, 10, 8) == -INV
    assert lib.tm_pcg_workspace_bytes(_lib.TM_F32, 10, 40, 8) == 256 + 4 * (6 * 10 + 3 * 8)
    assert lib.tm_sell_plan(-1, FAKE, FAKE, FAKE, None, None) == -INV
    assert lib.tm_sell_plan(10, FAKE, FAKE, None, None, None) == -INV


def test_negative_sizes_are_rejected(lib):
    f64 = _lib.TM_F64
    assert lib.tm_gather(f64, -3, FAKE, FAKE, FAKE, None) == INV
    assert lib.tm_scatter(f64, -3, FAKE, FAKE, FAKE, None) == INV
    assert lib.tm_csr_diagonal_inverse(f64, -3, FAKE, FAKE, FAKE, FAKE, None) == INV
    assert lib.tm_spmv_csr(f64, -3, 10, FAKE, FAKE, FAKE, FAKE, FAKE, None) == INV
    assert lib.tm_spmv_sell(f64, -3, FAKE, 1, FAKE, FAKE, FAKE, FAKE, None) == INV
    assert lib.tm_kp_count(-3, FAKE, FAKE, FAKE, FAKE, None) == INV
    assert lib.tm_morton_keys(-3, 3, FAKE, FAKE, FAKE, 21, FAKE, None) == INV
    assert lib.tm_pcg_jacobi(f64, -3, FAKE, FAKE, FAKE, FAKE, FAKE, 1e-8, 0.0, 10, FAKE, 1 << 20, None) == INV


def test_null_pointers_unknown_dtypes_and_flags_are_rejected(lib):
    f64 = _lib.TM_F64
    assert lib.tm_gather(f64, 5, None, FAKE, FAKE, None) == INV
    assert lib.tm_spmv_csr(f64, 5, 10, FAKE, FAKE, FAKE, None, FAKE, None) == INV
    assert lib.tm_spmv_csr(42, 5, 10, FAKE, FAKE, FAKE, FAKE, FAKE, None) == INV
    assert lib.tm_spmv_sell(42, 5, FAKE, 1, FAKE, FAKE, FAKE, FAKE, None) == INV
    assert lib.tm_morton_keys(5, 4, FAKE, FAKE, FAKE, 15, FAKE, None) == INV    # dim > 3
    assert lib.tm_morton_keys(5, 3, FAKE, FAKE, FAKE, 22, FAKE, None) == INV    # 66 key bits
    assert lib.tm_morton_keys(5, 3, None, FAKE, FAKE, 21, FAKE, None) == INV
    assert lib.tm_pcg_jacobi_sell(f64, 5, FAKE, FAKE, FAKE, FAKE, 160, FAKE, FAKE, 1e-8, 0.0, 10,
                                  7, FAKE, 1 << 20, None) == INV                # unknown method bits
    assert lib.tm_twolevel_apply(None, FAKE, FAKE, None) == INV
    assert lib.tm_fcg_twolevel_iterations(None, 0, FAKE, FAKE, FAKE, None, 0, None, None, FAKE, FAKE, FAKE,
                                          FAKE, FAKE, FAKE, FAKE, 1, None) == INV
    t = _lib.TwoLevel()
    t.n, t.nc = 10, 0                                                            # no aggregates
    assert lib.tm_twolevel_apply(t, FAKE, FAKE, None) == INV


def test_network_entries_reject_negative_sizes(lib):
    assert lib.tm_mpnn_input_fwd(-1, FAKE, FAKE, FAKE, FAKE, FAKE, FAKE, FAKE, None) == INV
    assert lib.tm_gather_axpy_f32(-1, FAKE, FAKE, FAKE, FAKE, FAKE, FAKE, FAKE, None) == INV
