"""The allocation-free PCG entry point (tm_pcg_jacobi_noalloc) against the
workspace entry point (tm_pcg_jacobi), through the C ABI.

Callers that cannot allocate device memory when they solve use the
allocation-free variant; its scratch lives in a fixed array inside the
library, shared by every call.  This file is collected last on purpose: if it
fails, a run that stops at the first failure has already run every other
test.  It is self-contained, so it also passes alone in a fresh process."""
import ctypes

import pytest
import torch

import tensormesh_gb300 as tg
from tensormesh_gb300 import _lib

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _system():
    mesh = tg.Mesh.gen_unit_cube(20, device=DEV, dtype=torch.float32)
    g = torch.Generator().manual_seed(17)
    kappa = torch.exp(torch.randn(mesh.n_elements, generator=g)).to(DEV)

    class KL(tg.ElementAssembler):
        def forward(self, gradu, gradv, kappa):
            return kappa * (gradu @ gradv)
    K = KL.from_mesh(mesh, quadrature_order=1)(mesh.points, element_data={"kappa": kappa})
    b = tg.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=1)(mesh.points)
    return tg.Condenser(mesh.boundary_mask)(K, b)


def test_noalloc_pcg_matches_workspace_pcg_twice():
    K, f = _system()
    assert K.dtype == torch.float32
    rtol = 1e-5
    x_ref = K.solve(f, rtol=rtol)
    assert K.last_solve_info.status == 0
    lib = _lib.load()
    for call in range(2):  # second call reuses the same scratch array
        x = torch.zeros_like(f)
        iters = ctypes.c_int32(0)
        res = ctypes.c_double(0.0)
        st = lib.tm_pcg_jacobi_noalloc(K.shape[0], K.indptr.data_ptr(), K.indices.data_ptr(),
                                       K.values.data_ptr(), f.data_ptr(), x.data_ptr(), rtol, 0.0, 20000,
                                       ctypes.byref(iters), ctypes.byref(res), _lib.stream_handle(x.device))
        assert st == _lib.TM_OK, f"call {call}: status {st}"
        assert iters.value > 0
        err = float((x - x_ref).abs().max() / x_ref.abs().max())
        assert err <= rtol, f"call {call}: rel diff {err:.3e}"
        true_res = float(torch.linalg.vector_norm(f.double() - (K @ x).double()) / torch.linalg.vector_norm(f.double()))
        assert true_res <= 10 * rtol


def test_noalloc_rejects_sizes_beyond_its_limit():
    lib = _lib.load()
    one = torch.zeros(1, device=DEV)
    ip = torch.zeros(2, dtype=torch.int64, device=DEV)
    ix = torch.zeros(1, dtype=torch.int32, device=DEV)
    st = lib.tm_pcg_jacobi_noalloc(2_000_000, ip.data_ptr(), ix.data_ptr(), one.data_ptr(), one.data_ptr(),
                                   one.data_ptr(), 1e-6, 0.0, 10, None, None, _lib.stream_handle(one.device))
    assert st == _lib.TM_ERR_INDEX
