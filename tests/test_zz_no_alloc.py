"""The no-allocation coupling-gradient entry point (edgpu_coupling_grad_device_noalloc).

Callers whose device memory belongs to another allocator (a Julia or PyTorch memory pool), or that
keep cudaMalloc/cudaFree out of a time-step loop, cannot let the library allocate.  This entry point
takes its scratch from a fixed array inside the library instead.  The test calls it through the C
ABI twice in a row and checks both results against the allocating entry point,
edgpu_coupling_grad_device, which also builds the operator's gradient tables the variant requires.
This file is collected last so that a run stopping at the first failure has run everything else."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_gradient_matches_allocating_entry_point():
    import torch
    import edgpu
    from edgpu import _lib, lattice
    from edgpu.representation import _torch_stream
    assert torch.cuda.is_available()
    L = 12
    rng = np.random.default_rng(21)
    J = 0.5 + rng.random(L)
    hs, _ = edgpu.spin_half_system(L)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0))
    m, r, c, a, ids = lattice.heisenberg_coupled(hs, lattice.chain_bonds(L))
    opr = edgpu.OperatorRepresentation.from_terms(hsr, m, r, c, a, coupling_ids=ids, couplings=J)
    N = hsr.dimension
    lib = _lib.lib()
    for prec, dtype, tol in ((_lib.FP64, torch.complex128, 1e-12), (_lib.MIXED, torch.complex64, 1e-5)):
        x = edgpu.random_state(N, 5, "fp64").to(dtype)
        gy = edgpu.random_state(N, 6, "fp64").to(dtype)
        y_ref = torch.empty_like(x)
        g_ref = edgpu.coupling_grad(opr, x, gy, precision=prec, y=y_ref)
        torch.cuda.synchronize()
        for call in range(2):
            y = torch.full_like(x, 7.0)
            g = np.full(L, np.nan)
            st = lib.edgpu_coupling_grad_device_noalloc(opr.handle, prec, ctypes.c_void_p(x.data_ptr()),
                                                        ctypes.c_void_p(gy.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                                        N, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                        _torch_stream())
            _lib.check(st)
            torch.cuda.synchronize()
            assert np.allclose(g, g_ref, rtol=tol, atol=tol), (call, g, g_ref)
            dy = torch.linalg.vector_norm((y - y_ref).to(torch.complex128)).item()
            assert dy <= tol * max(1.0, torch.linalg.vector_norm(y_ref.to(torch.complex128)).item()), (call, dy)
    # a length mismatch is rejected before anything runs
    g = np.zeros(L)
    st = lib.edgpu_coupling_grad_device_noalloc(opr.handle, _lib.FP64, ctypes.c_void_p(x.data_ptr()),
                                                ctypes.c_void_p(gy.data_ptr()), ctypes.c_void_p(y.data_ptr()), N + 1,
                                                g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
    assert st == _lib.ERR_DIM
