"""Batched sectors (edgpu_batch_*: one persistent launch, or per-sector launches on one to three
streams) against the oracle and against the single-sector product.

Every momentum sector of one Hamiltonian goes through one launch; each sector's result must equal
the single-sector product with the same lanes per row bit for bit, and the oracle's reduced product
within 1e-12 (FP64) or 1e-5 (mixed) relative.
"""
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


def triangular_sectors(E, L1, L2, sector, momenta=None):
    """J1-J2 XXZ model on the L1 x L2 triangular torus (Jz/Jxy = 0.8, J2/J1 = 0.125), every momentum
    sector: (GPU representations, oracle reduced tables, oracle terms)."""
    from edgpu import lattice
    n = L1 * L2
    hs, _ = E.spin_half_system(n)
    bonds1 = lattice.torus_bonds(L1, L2, lattice.TRIANGULAR_NN)
    bonds2 = lattice.torus_bonds(L1, L2, lattice.TRIANGULAR_NNN)
    bonds = bonds1 + bonds2
    jxy = [1.0] * len(bonds1) + [0.125] * len(bonds2)
    jz = [0.8 * j for j in jxy]
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    terms = O.heisenberg_terms(n, bonds, jxy, jz)
    hsr = E.represent(E.HilbertSpaceSector(hs, sector), lazy=True)
    sites = O.spin_half_sites(n)
    parent = O.hs_get_basis_list(sites, [(sector,)])
    bw, off = O.bit_layout(sites)
    if momenta is None:
        momenta = [(m1, m2) for m2 in range(L2) for m1 in range(L1)]
    oprs, reds = [], []
    for k in momenta:
        rh = E.symmetry_reduce(hsr, E.translation_symops((L1, L2), k))
        oprs.append(E.represent(rh, H))
        maps, amps = O.translation_symops((L1, L2), k)
        reds.append(O.symmetry_reduce(parent, bw, off, maps, amps))
    return oprs, reds, terms


def run_batch_checks(E, oprs, reds, terms):
    import torch
    b = E.Batch(oprs)
    xs_np = [O.complex_gaussian(o.dimension, 3 + i) for i, o in enumerate(oprs)]
    want = [O.apply_rows(r, terms, x) for r, x in zip(reds, xs_np)]
    for prec, tol, dt in (("fp64", FP64_TOL, torch.complex128), ("mixed", MIXED_TOL, torch.complex64)):
        xs = [torch.from_numpy(x).to(dt).cuda() for x in xs_np]
        for lpr in (1, 2, 4):
            b.set_tiling(prec, lpr)
            ref = []
            for o, x in zip(oprs, xs):
                o.set_tiling(prec, -lpr)
                y = torch.empty_like(x)
                E.mul_(y, o, x, precision=prec)
                ref.append(y)
                o.set_tiling(prec, 0)
            # one persistent launch; with one lane per row also per-sector launches on 1 to 3 streams
            for launch in ((0, 1, 2, 3) if lpr == 1 else (0,)):
                b.set_launch(prec, launch)
                assert b.launch(prec) == launch
                for use_graph in (False, True, True):
                    ys = [torch.full_like(x, float("nan")) for x in xs]
                    b.mul_(ys, xs, precision=prec, use_graph=use_graph)
                    torch.cuda.synchronize()
                    for k, (y, r, w) in enumerate(zip(ys, ref, want)):
                        assert torch.equal(y, r), (prec, lpr, launch, use_graph, k)
                        assert relerr(y.cpu().numpy().astype(np.complex128), w) < tol, (prec, lpr, k)
            b.set_launch(prec, 0)
        b.set_tiling(prec, 0)
    return b


def test_batch_triangular_all_momenta(edgpu):
    oprs, reds, terms = triangular_sectors(edgpu, 4, 3, 0)
    assert sum(o.dimension for o in oprs) == 924
    run_batch_checks(edgpu, oprs, reds, terms)


def test_batch_triangular_6x5_wide_words(edgpu):
    # 30 sites + 3 orbit-index bits: 64-bit basis words; 2Sz = 24 (three down spins), all 30 momenta
    oprs, reds, terms = triangular_sectors(edgpu, 6, 5, 24)
    assert sum(o.dimension for o in oprs) == 4060
    run_batch_checks(edgpu, oprs, reds, terms)


def test_batch_chain_ring_with_empty_sectors(edgpu):
    # chain L=8, 2Sz=6 (one down spin): one state per momentum; 2Sz=8 sector has one orbit (k=0 only)
    from edgpu import lattice
    L = 8
    hs, _ = edgpu.spin_half_system(L)
    H = lattice.xxz_hamiltonian(hs, lattice.chain_bonds(L), 1.0, 0.8)
    terms = O.heisenberg_terms(L, lattice.chain_bonds(L), [1.0] * L, [0.8] * L)
    sites = O.spin_half_sites(L)
    bw, off = O.bit_layout(sites)
    for q in (6, 8, 4):
        hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, q))
        parent = O.hs_get_basis_list(sites, [(q,)])
        oprs, reds = [], []
        for m in range(L):
            oprs.append(edgpu.represent(edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m)), H))
            maps, amps = O.translation_symops((L, 1), (m, 0))
            reds.append(O.symmetry_reduce(parent, bw, off, maps, amps))
        if q == 8:
            assert [o.dimension for o in oprs] == [1] + [0] * (L - 1)
        run_batch_checks(edgpu, oprs, reds, terms)


def test_batch_generic_group(edgpu):
    # translations x global spin flip (sign-carrying group, table-driven canonicalisation)
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
    oprs, reds = [], []
    for m in range(L):
        for par in (1, -1):
            ops, maps, flips, amps = [], [], [], []
            for t, a in edgpu.translation_symops(L, m):
                for f, chi in ((False, 1), (True, par)):
                    ops.append((t * edgpu.GlobalBitFlip(f) if f else t, chi * a))
                    maps.append(t.map)
                    flips.append(full if f else 0)
                    amps.append(chi * a)
            oprs.append(edgpu.represent(edgpu.symmetry_reduce(hsr, ops), H))
            reds.append(O.symmetry_reduce(parent, bw, off, np.array(maps, dtype=np.int32), np.array(amps),
                                          flips=np.array(flips, dtype=np.uint64)))
    run_batch_checks(edgpu, oprs, reds, terms)


def test_batch_per_sector_own_schedules(edgpu):
    """Per-sector launches with each operator's own schedule (launch modes 5 to 7), here the slab
    product for some sectors and the target table for the others: every sector's result equals that
    operator's own product bit for bit, and the oracle within tolerance."""
    import torch
    oprs, reds, terms = triangular_sectors(edgpu, 4, 3, 0)
    b = edgpu.Batch(oprs)
    for i, o in enumerate(oprs):
        if o.dimension:
            assert o.build_targets(1 << 26)
            if i % 2 == 0:
                assert o.build_slabs(slab_bytes=8, max_bytes=1 << 26)
    xs_np = [O.complex_gaussian(o.dimension, 30 + i) for i, o in enumerate(oprs)]
    want = [O.apply_rows(r, terms, x) for r, x in zip(reds, xs_np)]
    for prec, tol, dt in (("fp64", FP64_TOL, torch.complex128), ("mixed", MIXED_TOL, torch.complex64)):
        xs = [torch.from_numpy(x).to(dt).cuda() for x in xs_np]
        ref = []
        for o, x in zip(oprs, xs):
            y = torch.empty_like(x)
            edgpu.mul_(y, o, x, precision=prec)
            ref.append(y)
        for launch in (5, 6, 7):
            b.set_launch(prec, launch)
            assert b.launch(prec) == launch
            for use_graph in (False, True, True):
                ys = [torch.full_like(x, float("nan")) for x in xs]
                b.mul_(ys, xs, precision=prec, use_graph=use_graph)
                torch.cuda.synchronize()
                for k, (y, r, w) in enumerate(zip(ys, ref, want)):
                    assert torch.equal(y, r), (prec, launch, use_graph, k)
                    assert relerr(y.cpu().numpy().astype(np.complex128), w) < tol, (prec, launch, k)
    lpr, ms = b.autotune("mixed")
    assert b.launch("mixed") in (0, 1, 2, 3, 5, 6, 7)


def test_batch_rejects_different_operators(edgpu):
    import torch
    from edgpu import lattice
    L = 8
    hs, _ = edgpu.spin_half_system(L)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0))
    H1 = lattice.xxz_hamiltonian(hs, lattice.chain_bonds(L), 1.0, 1.0)
    H2 = lattice.xxz_hamiltonian(hs, lattice.chain_bonds(L), 1.0, 0.5)
    o1 = edgpu.represent(edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, 0)), H1)
    o2 = edgpu.represent(edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, 1)), H2)
    b = edgpu.Batch([o1, o2])
    xs = [edgpu.random_state(o.dimension, 1, "mixed") for o in (o1, o2)]
    ys = [torch.empty_like(x) for x in xs]
    with pytest.raises(edgpu.ArgumentError):
        b.mul_(ys, xs)
    with pytest.raises(edgpu.DimensionMismatch):
        edgpu.Batch([o1, o1]).mul_(ys, xs)
    with pytest.raises(edgpu.ArgumentError):
        b.set_tiling("mixed", 3)
    with pytest.raises(edgpu.ArgumentError):
        b.set_launch("mixed", 4)
    with pytest.raises(edgpu.ArgumentError):
        b.set_launch("mixed", 8)


def test_batch_follows_coupling_changes_and_autotune(edgpu):
    import torch
    from edgpu import lattice
    L = 12
    bonds = lattice.chain_bonds(L)
    hs, _ = edgpu.spin_half_system(L)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0), lazy=True)
    masks, rows, cols, amps, ids = lattice.heisenberg_coupled(hs, bonds)
    J = 0.5 + np.random.default_rng(4).random(L)
    oprs = [edgpu.OperatorRepresentation.from_terms(edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m)),
                                                    masks, rows, cols, amps, ids, J) for m in range(L)]
    b = edgpu.Batch(oprs)
    lpr, ms = b.autotune("mixed")
    assert lpr in (1, 2, 4) and ms > 0
    assert b.launch("mixed") in (0, 1, 2, 3)
    xs = [edgpu.random_state(o.dimension, 10 + i, "mixed") for i, o in enumerate(oprs)]
    for step in range(2):
        ys = [torch.empty_like(x) for x in xs]
        b.mul_(ys, xs, use_graph=True)
        for o, x, y in zip(oprs, xs, ys):
            o.set_tiling("mixed", -lpr)
            r = torch.empty_like(x)
            edgpu.mul_(r, o, x, precision="mixed")
            o.set_tiling("mixed", 0)
            assert torch.equal(y, r)
        for o in oprs:
            o.set_couplings(J * (1.5 + step))
