"""The differentiable product edgpu.apply_hamiltonian (torch.autograd.Function, the counterpart of a
ChainRulesCore.rrule for mul!): torch.autograd.gradcheck in FP64 against finite differences, for
terms that do not commute with the translations (per-bond couplings in a momentum sector, the
adjoint's scatter path) and terms that do (complex characters), plus the mixed-precision flavour
against the FP64 gradients."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _coupled(L, k, seed):
    import edgpu
    from edgpu import lattice
    hs, _ = edgpu.spin_half_system(L)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0))
    rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, k))
    m, r, c, a, ids = lattice.heisenberg_coupled(hs, lattice.chain_bonds(L))
    J = 0.5 + np.random.default_rng(seed).random(L)
    return edgpu.OperatorRepresentation.from_terms(rh, m, r, c, a, coupling_ids=ids, couplings=J), J


@pytest.mark.parametrize("L,k,invariant", [(10, 0, False), (12, 1, False), (12, 3, True)])
def test_gradcheck(L, k, invariant):
    import torch
    import edgpu
    opr, J = _coupled(L, k, 4)
    if invariant:   # equal couplings: the terms commute with the translations
        J[:] = 0.9
        opr.set_couplings(J)
    else:           # the adjoint through the adjoint target table
        assert opr.build_targets(1 << 28) and opr.build_adjoint_targets(1 << 28)
    N = opr.dimension
    g = torch.Generator(device="cpu").manual_seed(L + k)
    x = torch.randn(N, dtype=torch.complex128, generator=g).cuda().requires_grad_(True)
    Jt = torch.tensor(J, dtype=torch.float64, device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(lambda xx, jj: edgpu.apply_hamiltonian(opr, xx, jj), (x, Jt),
                                    eps=1e-6, atol=1e-7, rtol=1e-6, nondet_tol=1e-12)


def test_backward_matches_library_gradients_and_mixed():
    import torch
    import edgpu
    opr, J = _coupled(14, 0, 6)
    N = opr.dimension
    x64 = edgpu.random_state(N, 5, "fp64")
    gy = edgpu.random_state(N, 6, "fp64")
    x = x64.clone().requires_grad_(True)
    Jt = torch.tensor(J, dtype=torch.float64, device="cuda", requires_grad=True)
    y = edgpu.apply_hamiltonian(opr, x, Jt)
    loss = (gy.conj() * y).real.sum()
    loss.backward()
    want_J = edgpu.coupling_grad(opr, x64, gy, precision="fp64")
    want_x = torch.empty_like(gy)
    edgpu.mul_adjoint_(want_x, opr, gy, precision="fp64")
    torch.cuda.synchronize()
    assert np.allclose(Jt.grad.cpu().numpy(), want_J, rtol=1e-12, atol=1e-12)
    assert torch.allclose(x.grad, want_x, rtol=1e-12, atol=1e-12)
    # a second forward with other couplings, differentiated after the first: each backward uses its own J
    J2 = J[::-1].copy()
    J2t = torch.tensor(J2, dtype=torch.float64, device="cuda", requires_grad=True)
    x2 = x64.clone().requires_grad_(True)
    y2 = edgpu.apply_hamiltonian(opr, x2, J2t)
    x1 = x64.clone().requires_grad_(True)
    J1t = torch.tensor(J, dtype=torch.float64, device="cuda", requires_grad=True)
    y1 = edgpu.apply_hamiltonian(opr, x1, J1t)
    (gy.conj() * y2).real.sum().backward()
    (gy.conj() * y1).real.sum().backward()
    assert torch.allclose(x1.grad, want_x, rtol=1e-12, atol=1e-12)
    opr.set_couplings(J2)
    want_x2 = torch.empty_like(gy)
    edgpu.mul_adjoint_(want_x2, opr, gy, precision="fp64")
    torch.cuda.synchronize()
    assert torch.allclose(x2.grad, want_x2, rtol=1e-12, atol=1e-12)
    # mixed precision (complex64 vectors, FP32 accumulation) against the FP64 gradients
    x32 = x64.to(torch.complex64).requires_grad_(True)
    J3t = torch.tensor(J, dtype=torch.float64, device="cuda", requires_grad=True)
    y32 = edgpu.apply_hamiltonian(opr, x32, J3t)
    (gy.to(torch.complex64).conj() * y32).real.sum().backward()
    assert np.allclose(J3t.grad.cpu().numpy(), want_J, rtol=1e-4, atol=1e-4)
    assert torch.allclose(x32.grad.to(torch.complex128), want_x, rtol=1e-4, atol=1e-5)
