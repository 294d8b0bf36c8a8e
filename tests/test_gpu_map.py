"""Parent-state maps (edgpu_space_build_map): the product that looks targets up in the map equals the
product that canonicalises and searches them, bit for bit, and the oracle within tolerance."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-5


@pytest.fixture(scope="module")
def edgpu():
    import torch
    assert torch.cuda.is_available()
    import edgpu as E
    return E


def relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def products(E, opr, x_np, lprs=(-1, -2, -4)):
    """{(precision, schedule): device result} for a seeded input."""
    import torch
    out = {}
    for prec, dt in (("fp64", torch.complex128), ("mixed", torch.complex64)):
        x = torch.from_numpy(x_np).to(dt).cuda()
        for sched in lprs:
            opr.set_tiling(prec, sched)
            y = torch.empty_like(x)
            E.mul_(y, opr, x, precision=prec)
            out[(prec, sched)] = y
        opr.set_tiling(prec, 0)
    return out


def check_mapped(E, rh, opr, red, terms, seed):
    import torch
    x = O.complex_gaussian(rh.dimension, seed)
    plain = products(E, opr, x)
    assert rh.build_map(1 << 30)
    n, b = rh.map_info
    assert n > 0 and b in (4, 8)
    mapped = products(E, opr, x)
    want = O.apply_rows(red, terms, x)
    for key, y in mapped.items():
        assert torch.equal(y, plain[key]), key
        tol = FP64_TOL if key[0] == "fp64" else MIXED_TOL
        assert relerr(y.cpu().numpy().astype(np.complex128), want) < tol, key
    rh.free_map()
    assert rh.map_info == (0, 0)
    again = products(E, opr, x, lprs=(-1,))
    assert torch.equal(again[("fp64", -1)], plain[("fp64", -1)])


def test_map_chain_all_momenta(edgpu):
    from edgpu import lattice
    L = 16
    hs, _ = edgpu.spin_half_system(L)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0))
    bonds = lattice.chain_bonds(L) + [(i, (i + 2) % L) for i in range(L)]
    jxy = [1.0] * L + [0.3] * L
    jz = [0.8] * L + [0.24] * L
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    terms = O.heisenberg_terms(L, bonds, jxy, jz)
    sites = O.spin_half_sites(L)
    parent = O.hs_get_basis_list(sites, [(0,)])
    bw, off = O.bit_layout(sites)
    for m in range(L):
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m))
        maps, amps = O.translation_symops((L, 1), (m, 0))
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        check_mapped(edgpu, rh, edgpu.represent(rh, H), red, terms, seed=m + 1)


@pytest.mark.parametrize("shape,sector", [((4, 4), 0), ((4, 5), 0), ((6, 3), 2), ((6, 5), 24)])
def test_map_torus(edgpu, shape, sector):
    from edgpu import lattice
    L1, L2 = shape
    n = L1 * L2
    hs, _ = edgpu.spin_half_system(n)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, sector), lazy=True)
    b1 = lattice.torus_bonds(L1, L2, lattice.TRIANGULAR_NN)
    b2 = lattice.torus_bonds(L1, L2, lattice.TRIANGULAR_NNN)
    bonds = b1 + b2
    jxy = [1.0] * len(b1) + [0.125] * len(b2)
    jz = [0.8 * j for j in jxy]
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    terms = O.heisenberg_terms(n, bonds, jxy, jz)
    sites = O.spin_half_sites(n)
    parent = O.hs_get_basis_list(sites, [(sector,)])
    bw, off = O.bit_layout(sites)
    for k in [(0, 0), (1, 0), (0, 1), (L1 - 1, L2 - 1)]:
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(shape, k))
        maps, amps = O.translation_symops(shape, k)
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        check_mapped(edgpu, rh, edgpu.represent(rh, H), red, terms, seed=k[0] + 7 * k[1])


def test_map_generic_group_and_limits(edgpu):
    from edgpu import lattice
    L = 10
    hs, _ = edgpu.spin_half_system(L)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0))
    H = lattice.xxz_hamiltonian(hs, lattice.chain_bonds(L), 1.0, 1.0)
    terms = O.heisenberg_terms(L, lattice.chain_bonds(L), [1.0] * L, [1.0] * L)
    sites = O.spin_half_sites(L)
    parent = O.hs_get_basis_list(sites, [(0,)])
    bw, off = O.bit_layout(sites)
    full = (1 << L) - 1
    for m, par in ((0, 1), (3, -1)):
        ops, maps, flips, amps = [], [], [], []
        for t, a in edgpu.translation_symops(L, m):
            for f, chi in ((False, 1), (True, par)):
                ops.append((t * edgpu.GlobalBitFlip(f) if f else t, chi * a))
                maps.append(t.map)
                flips.append(full if f else 0)
                amps.append(chi * a)
        rh = edgpu.symmetry_reduce(hsr, ops)
        red = O.symmetry_reduce(parent, bw, off, np.array(maps, dtype=np.int32), np.array(amps),
                                flips=np.array(flips, dtype=np.uint64))
        check_mapped(edgpu, rh, edgpu.represent(rh, H), red, terms, seed=5 + m)
    rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, 0))
    assert not rh.build_map(16)                       # too large for the limit: nothing built
    assert rh.map_info == (0, 0)


def test_map_batched_sectors(edgpu):
    import torch
    from edgpu import lattice
    L1, L2 = 4, 3
    n = L1 * L2
    hs, _ = edgpu.spin_half_system(n)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0), lazy=True)
    bonds = lattice.torus_bonds(L1, L2, lattice.TRIANGULAR_NN)
    H = lattice.xxz_hamiltonian(hs, bonds, 1.0, 0.8)
    spaces = [edgpu.symmetry_reduce(hsr, edgpu.translation_symops((L1, L2), (a, b)))
              for b in range(L2) for a in range(L1)]
    oprs = [edgpu.represent(sp, H) for sp in spaces]
    xs = [edgpu.random_state(o.dimension, 40 + i, "mixed") for i, o in enumerate(oprs)]
    ref = []
    for o, x in zip(oprs, xs):
        y = torch.empty_like(x)
        edgpu.mul_(y, o, x, precision="mixed")
        ref.append(y)
    b = edgpu.Batch(oprs)
    for sp in spaces:
        assert sp.build_map(1 << 26)
    for use_graph in (False, True):
        ys = [torch.empty_like(x) for x in xs]
        b.mul_(ys, xs, precision="mixed", use_graph=use_graph)
        torch.cuda.synchronize()
        for y, r in zip(ys, ref):
            assert torch.equal(y, r)
    for sp in spaces:
        sp.free_map()
    ys = [torch.empty_like(x) for x in xs]
    b.mul_(ys, xs, precision="mixed", use_graph=True)
    torch.cuda.synchronize()
    for y, r in zip(ys, ref):
        assert torch.equal(y, r)
