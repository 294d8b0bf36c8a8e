"""symmetry_unreduce / symmetry_reduce(rhsr, v) on the device (edgpu_symmetry_unreduce_device,
edgpu_symmetry_reduce_device): against the oracle's parent-table restatement
(symmetry_reduce.jl:38-56, :208-225) for chains at every momentum, tori, translation x spin-flip
groups, materialised and lazy parents, FP64 and mixed precision; and the round trip at the 6x6
sector's full size (a parent vector of 9,075,135,300 entries), where the reference's parent-sized
tables do not fit."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _check(E, rh, red, seed):
    import torch
    N, Np = red.dim, red.parent.size
    rng = np.random.default_rng(seed)
    s = rng.normal(size=N) + 1j * rng.normal(size=N)
    lv = rng.normal(size=Np) + 1j * rng.normal(size=Np)
    want_large = O.unreduce(red, s)
    want_small = O.reduce_vector(red, lv)
    for dt, tol in ((torch.complex128, 1e-13), (torch.complex64, 1e-6)):
        big = E.symmetry_unreduce(rh, torch.from_numpy(s).to(dt).cuda())
        sm = E.symmetry_reduce(rh, torch.from_numpy(lv).to(dt).cuda())
        torch.cuda.synchronize()
        assert np.max(np.abs(big.cpu().numpy() - want_large)) < tol * max(1.0, np.max(np.abs(want_large)))
        assert np.max(np.abs(sm.cpu().numpy() - want_small)) < tol * max(1.0, np.max(np.abs(want_small)))
    # host arrays (complex128 through the device)
    assert np.allclose(E.symmetry_unreduce(rh, s), want_large, atol=1e-13)
    assert np.allclose(E.symmetry_reduce(rh, lv), want_small, atol=1e-12)


@pytest.mark.parametrize("lazy", [False, True])
def test_chain_all_momenta(lazy):
    import edgpu as E
    L = 14
    hs, _ = E.spin_half_system(L)
    hsr = E.represent(E.HilbertSpaceSector(hs, 0), lazy=lazy)
    parent = O.popcount_basis(L, L // 2)
    bw, off = O.bit_layout(O.spin_half_sites(L))
    for m in range(L):
        rh = E.symmetry_reduce(hsr, E.translation_symops(L, m))
        maps, amps = O.translation_symops((L, 1), (m, 0))
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        _check(E, rh, red, m)


@pytest.mark.parametrize("shape,k", [((4, 4), (1, 2)), ((6, 3), (3, 1)), ((5, 4), (0, 0))])
def test_torus(shape, k):
    import edgpu as E
    L1, L2 = shape
    n = L1 * L2
    hs, _ = E.spin_half_system(n)
    hsr = E.represent(E.HilbertSpaceSector(hs, 0), lazy=True)
    rh = E.symmetry_reduce(hsr, E.translation_symops(shape, k))
    parent = O.popcount_basis(n, n // 2)
    bw, off = O.bit_layout(O.spin_half_sites(n))
    maps, amps = O.translation_symops(shape, k)
    red = O.symmetry_reduce(parent, bw, off, maps, amps)
    _check(E, rh, red, 7)


def test_translation_times_spin_flip():
    """A general group (site permutations with a global bit flip): translations of a 10-site ring
    times the spin flip, in the 2Sz = 0 sector."""
    import edgpu as E
    L = 10
    hs, _ = E.spin_half_system(L)
    hsr = E.represent(E.HilbertSpaceSector(hs, 0))
    parent = O.popcount_basis(L, L // 2)
    bw, off = O.bit_layout(O.spin_half_sites(L))
    full = (1 << L) - 1
    for m, par in ((0, 1), (3, -1), (5, 1)):
        ops, maps, flips, amps = [], [], [], []
        for t, a in E.translation_symops(L, m):
            for f, chi in ((False, 1), (True, par)):
                ops.append((t * E.GlobalBitFlip(f) if f else t, chi * a))
                maps.append(t.map)
                flips.append(full if f else 0)
                amps.append(chi * a)
        rh = E.symmetry_reduce(hsr, ops)
        red = O.symmetry_reduce(parent, bw, off, np.array(maps, dtype=np.int32), np.array(amps),
                                flips=np.array(flips, dtype=np.uint64))
        assert np.array_equal(rh.basis_list, red.basis_list)
        _check(E, rh, red, m + 3)


def test_round_trip_6x6_full_size():
    """The 6x6 k=(0,0) sector: unreduce then reduce is the identity (mixed precision; a 73 GB parent
    vector on the device), and the unreduced vector has the norm of the reduced one."""
    import gc
    import torch
    import edgpu as E
    gc.collect()
    torch.cuda.empty_cache()
    hs, _ = E.spin_half_system(36)
    hsr = E.represent(E.HilbertSpaceSector(hs, 0), lazy=True)
    rh = E.symmetry_reduce(hsr, E.translation_symops((6, 6), (0, 0)))
    s = E.random_state(rh.dimension, 11, "mixed")
    big = E.symmetry_unreduce(rh, s)
    assert big.numel() == 9075135300
    nb = torch.linalg.vector_norm(big).item()
    assert abs(nb - 1.0) < 1e-3
    back = E.symmetry_reduce(rh, big)
    del big
    torch.cuda.synchronize()
    err = torch.linalg.vector_norm((back - s).to(torch.complex128)).item()
    assert err < 1e-5
