"""The no-allocation coupling-gradient entry point (edgpu_coupling_grad_device_noalloc).

Callers whose device memory belongs to another allocator (a Julia or PyTorch memory pool), or that
keep cudaMalloc/cudaFree out of a time-step loop, cannot let the library allocate.  This entry point
takes its scratch from a fixed array inside the library instead.  The test calls it through the C
ABI twice in a row and checks both results against the allocating entry point,
edgpu_coupling_grad_device (which also builds the operator's tables the variant requires), on the
kernels the allocating entry point chooses: the pair-flip gradient kernel through a target table,
and the term scan; that the device's free memory does not change across the calls, also after new
coupling values (rewritten in place); that an operator whose tables were never built is refused
with EDGPU_ERR_STATE; and, with enough couplings and rows, that the block count is limited to what
the scratch array holds.  This file is collected last so that a run stopping at the first failure
has run everything else."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, _lib, opr, prec, x, gy, y, n, g, stream):
    return lib.edgpu_coupling_grad_device_noalloc(opr.handle, prec, ctypes.c_void_p(x.data_ptr()),
                                                  ctypes.c_void_p(gy.data_ptr()), ctypes.c_void_p(y.data_ptr()), n,
                                                  g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), stream)


def _chain_operator(L, table, reduced):
    import edgpu
    from edgpu import lattice
    rng = np.random.default_rng(21)
    J = 0.5 + rng.random(L)
    hs, _ = edgpu.spin_half_system(L)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0))
    sp = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, 0)) if reduced else hsr
    m, r, c, a, ids = lattice.heisenberg_coupled(hs, lattice.chain_bonds(L))
    opr = edgpu.OperatorRepresentation.from_terms(sp, m, r, c, a, coupling_ids=ids, couplings=J)
    if table:
        assert opr.build_targets(1 << 30)
    return opr, J


@pytest.mark.parametrize("table,reduced", [(False, False), (True, False), (True, True)])
def test_noalloc_gradient_matches_allocating_entry_point(table, reduced):
    import torch
    import edgpu
    from edgpu import _lib
    from edgpu.representation import _torch_stream
    assert torch.cuda.is_available()
    L = 14
    opr, J = _chain_operator(L, table, reduced)
    N = opr.dimension
    lib = _lib.lib()
    for prec, dtype, tol in ((_lib.FP64, torch.complex128, 1e-12), (_lib.MIXED, torch.complex64, 1e-5)):
        x = edgpu.random_state(N, 5, "fp64").to(dtype)
        gy = edgpu.random_state(N, 6, "fp64").to(dtype)
        y_ref = torch.empty_like(x)
        g_ref = edgpu.coupling_grad(opr, x, gy, precision=prec, y=y_ref)
        y = torch.full_like(x, 7.0)
        ny = torch.linalg.vector_norm(y_ref.to(torch.complex128)).item()
        torch.cuda.synchronize()
        free0 = None
        for call in range(3):
            g = np.full(L, np.nan)
            _lib.check(_noalloc(lib, _lib, opr, prec, x, gy, y, N, g, _torch_stream()))
            torch.cuda.synchronize()
            assert np.allclose(g, g_ref, rtol=tol, atol=tol), (call, g, g_ref)
            dy = torch.linalg.vector_norm((y - y_ref).to(torch.complex128)).item()
            assert dy <= tol * max(1.0, ny), (call, dy)
            if free0 is None:
                # the first call on a device may make the driver place the library's device globals
                # (the scratch array) in memory; the later calls must change nothing
                free0 = torch.cuda.mem_get_info()[0]
        assert torch.cuda.mem_get_info()[0] == free0, "the no-allocation entry point changed the free device memory"
        # new coupling values are written into the existing tables: still no allocation, new results
        J2 = J[::-1].copy()
        opr.set_couplings(J2)
        g2_ref = edgpu.coupling_grad(opr, x, gy, precision=prec, y=y_ref)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        opr.set_couplings(J)
        opr.set_couplings(J2)
        g2 = np.full(L, np.nan)
        _lib.check(_noalloc(lib, _lib, opr, prec, x, gy, y, N, g2, _torch_stream()))
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free1
        assert np.allclose(g2, g2_ref, rtol=tol, atol=tol)
        opr.set_couplings(J)
    # a length mismatch is rejected before anything runs
    g = np.zeros(L)
    st = _noalloc(lib, _lib, opr, _lib.FP64, x, gy, y, N + 1, g, None)
    assert st == _lib.ERR_DIM


def test_noalloc_refuses_an_operator_without_tables():
    import torch
    import edgpu
    from edgpu import _lib
    opr, _ = _chain_operator(10, False, False)
    N = opr.dimension
    x = edgpu.random_state(N, 1, "fp64")
    y = torch.empty_like(x)
    g = np.zeros(10)
    st = _noalloc(_lib.lib(), _lib, opr, _lib.FP64, x, x, y, N, g, None)
    assert st == _lib.ERR_STATE
    assert "not built" in _lib.lib().edgpu_last_error().decode()


def test_noalloc_limits_blocks_to_the_scratch():
    """About a thousand couplings (one per term) over 705,432 rows: the allocating launch uses more blocks than the
    2 MiB scratch holds partial sums for, so the no-allocation launch runs with fewer blocks (a
    different summation order of the same terms)."""
    import torch
    import edgpu
    from edgpu import _lib, lattice
    from edgpu.representation import _torch_stream
    L = 22
    hs, _ = edgpu.spin_half_system(L)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0))
    bonds = lattice.chain_bonds(L) + [(i, (i + 2) % L) for i in range(L)]
    H = lattice.xxz_hamiltonian(hs, bonds, 1.0, 0.7)
    m, r, c, a = edgpu.term_arrays(H)
    # four copies of every term, each with its own coupling: about a thousand couplings, so the scratch
    # holds the partial sums of at most 2^18 / T - 1 (below 300) blocks, fewer than the allocating
    # launch uses
    m, r, c, a = np.tile(m, 4), np.tile(r, 4), np.tile(c, 4), np.tile(a, 4)
    T = len(m)
    assert T >= 880
    rng = np.random.default_rng(3)
    J = 0.5 + rng.random(T)
    opr = edgpu.OperatorRepresentation.from_terms(hsr, m, r, c, a, coupling_ids=np.arange(T), couplings=J)
    N = opr.dimension
    x = edgpu.random_state(N, 5, "fp64")
    gy = edgpu.random_state(N, 6, "fp64")
    y_ref = torch.empty_like(x)
    g_ref = edgpu.coupling_grad(opr, x, gy, precision="fp64", y=y_ref)
    y = torch.empty_like(x)
    for _ in range(2):
        g = np.full(T, np.nan)
        _lib.check(_noalloc(_lib.lib(), _lib, opr, _lib.FP64, x, gy, y, N, g, _torch_stream()))
        torch.cuda.synchronize()
        assert np.allclose(g, g_ref, rtol=1e-10, atol=1e-10)
        assert torch.allclose(y, y_ref, rtol=1e-12, atol=1e-12)
