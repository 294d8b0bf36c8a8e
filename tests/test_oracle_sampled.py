"""The orbit-by-orbit oracle (oracle.OrbitTables) against the parent-table oracle.

OrbitTables evaluates the reference's mapping tables (symmetry_reduce_generic.jl:22-106) for one
orbit at a time, so that rows of sectors whose parent-sized tables do not fit in host memory (the
6x6 torus) can still be checked against the reference's row formula
(reduced_operator_representation.jl:57-85).  Here, at sizes where the parent-sized tables are cheap,
it must give exactly what the table-based restatement gives: the same representatives, mapping
amplitudes, rows and nonzero counts.  The Burnside count of sector dimensions is checked against the
representative lists too.  CPU only."""
import numpy as np
import pytest

from oracle import oracle as O


def _torus_terms(shape, nn, nnn, j1, j2, aniso, rng=None):
    L1, L2 = shape
    bonds, jxy, jz = [], [], []
    for vecs, j in ((nn, j1), (nnn, j2)):
        for dx, dy in vecs:
            for y in range(L2):
                for x in range(L1):
                    bonds.append((x + L1 * y, (x + dx) % L1 + L1 * ((y + dy) % L2)))
                    jj = j if rng is None else j * (0.5 + rng.random())
                    jxy.append(jj)
                    jz.append(jj * aniso)
    return O.heisenberg_terms(L1 * L2, bonds, jxy, jz)


CASES = [
    # (shape, momentum, nn, nnn, j2, aniso, n_up, random couplings)
    ((12, 1), (0, 0), [(1, 0)], [], 0.0, 1.0, 6, False),
    ((12, 1), (5, 0), [(1, 0)], [(2, 0)], 0.3, 0.7, 6, True),
    ((14, 1), (7, 0), [(1, 0)], [], 0.0, 1.0, 7, False),
    ((13, 1), (3, 0), [(1, 0)], [(2, 0)], 0.5, 1.0, 6, False),
    ((4, 4), (0, 0), [(1, 0), (0, 1)], [(1, 1), (1, -1)], 0.5, 1.0, 8, False),
    ((4, 4), (1, 2), [(1, 0), (0, 1)], [(1, 1), (1, -1)], 0.5, 1.0, 8, False),
    ((5, 4), (2, 1), [(1, 0), (1, 1), (0, 1)], [(2, 1), (1, 2), (-1, 1)], 0.125, 0.8, 10, False),
    ((6, 3), (3, 1), [(1, 0), (1, 1), (0, 1)], [(2, 1), (1, 2), (-1, 1)], 0.125, 0.8, 9, True),
    ((4, 4), (2, 0), [(1, 0), (0, 1)], [], 0.0, 1.0, 5, False),
]


@pytest.mark.parametrize("shape,k,nn,nnn,j2,aniso,n_up,rand", CASES)
def test_orbit_tables_match_parent_tables(shape, k, nn, nnn, j2, aniso, n_up, rand):
    L1, L2 = shape
    n = L1 * L2
    parent = O.popcount_basis(n, n_up)
    sites = O.spin_half_sites(n)
    bw, off = O.bit_layout(sites)
    maps, amps = O.translation_symops(shape, k)
    red = O.symmetry_reduce(parent, bw, off, maps, amps)
    terms = _torus_terms(shape, nn, nnn, 1.0, j2, aniso, np.random.default_rng(3) if rand else None)
    x = O.complex_gaussian(red.dim, 11)
    y_ref = O.apply_rows(red, terms, x)

    ot = O.OrbitTables(n, n_up, maps, amps, red.basis_list)
    # mapping tables: every parent state's representative index and amplitude
    rep, kept, nd, am = ot.orbit_info(parent)
    idx = np.where(kept, O.lookup(red.basis_list, rep), -1)
    assert np.array_equal(idx, red.basis_mapping_index)
    assert np.allclose(am[kept], red.basis_mapping_amplitude[kept], rtol=0, atol=1e-15)
    # representatives are their own orbit minima, kept; orbit sizes divide the group order
    rrep, rkept, rnd, _ = ot.orbit_info(red.basis_list)
    assert np.array_equal(rrep, red.basis_list) and rkept.all()
    assert np.all(maps.shape[0] % rnd == 0)
    # every row of the product, and its nonzero count
    vals, st, nnz = ot.rows(terms, x, np.arange(red.dim))
    assert (st == 0).all()
    assert np.max(np.abs(vals - y_ref)) <= 1e-13 * max(1.0, np.max(np.abs(y_ref)))
    sampler = O.RowSampler(red, terms, x)
    assert int(nnz.sum()) == sampler.run(0, red.dim, count=True)
    # Burnside's count of the sector dimension
    num = np.rint(-np.angle(amps) / (2 * np.pi) * n).astype(np.int64) % n
    assert np.allclose(np.exp(-2j * np.pi * num / n), amps)
    assert O.sector_dimension(maps, num, n, n_up) == red.dim


def test_orbit_tables_flag_a_bad_table():
    """A representative table with an entry removed is caught (status 3 on rows that reach it), and
    a non-representative entry is flagged (status 1)."""
    n, n_up = 12, 6
    parent = O.popcount_basis(n, n_up)
    sites = O.spin_half_sites(n)
    bw, off = O.bit_layout(sites)
    maps, amps = O.translation_symops((n, 1), (0, 0))
    red = O.symmetry_reduce(parent, bw, off, maps, amps)
    terms = _torus_terms((n, 1), [(1, 0)], [], 1.0, 0.0, 1.0)
    bad = np.delete(red.basis_list, 5)
    ot = O.OrbitTables(n, n_up, maps, amps, bad)
    x = O.complex_gaussian(bad.size, 1)
    _, st, _ = ot.rows(terms, x, np.arange(bad.size))
    assert (st == 3).any()
    bad2 = red.basis_list.copy()
    bad2[3] = O.symmetry_apply(bw, off, maps[1], int(bad2[3]))
    bad2.sort()
    ot2 = O.OrbitTables(n, n_up, maps, amps, bad2)
    _, st2, _ = ot2.rows(terms, O.complex_gaussian(bad2.size, 1), np.arange(bad2.size))
    assert (st2 == 1).any()


def test_sector_dimensions_sum_to_parent():
    """Burnside counts over all momenta of the 6x6 torus and the 30-site triangular torus add up to
    the 2Sz = 0 parent dimension, and give the exact sector sizes of the benchmark sectors."""
    from math import comb
    for shape, check in (((6, 6), {(0, 0): 252091362}), ((6, 5), {}), ((24, 1), {(0, 0): 112720}),
                         ((28, 1), {(0, 0): 1432860})):
        L1, L2 = shape
        n = L1 * L2
        tot = 0
        for m2 in range(L2):
            for m1 in range(L1):
                maps, amps = O.translation_symops(shape, (m1, m2))
                G = maps.shape[0]
                num = np.rint(-np.angle(amps) / (2 * np.pi) * G * 1.0).astype(np.int64)
                den = G
                # amplitudes are exp(-2 pi i (m1 a / L1 + m2 b / L2)): numerators over L1 * L2
                num = np.array([(m1 * (g % L1) * L2 + m2 * (g // L1) * L1) % den for g in range(G)])
                assert np.allclose(np.exp(-2j * np.pi * num / den), amps)
                d = O.sector_dimension(maps, num, den, n // 2)
                if (m1, m2) in check:
                    assert d == check[(m1, m2)]
                tot += d
        assert tot == comb(n, n // 2)


@pytest.mark.parametrize("shape,k,n_up", [((6, 4), (0, 0), 12), ((6, 4), (1, 2), 11), ((5, 4), (2, 1), 10),
                                          ((12, 1), (5, 0), 6), ((4, 4), (1, 1), 7), ((6, 3), (3, 1), 9)])
def test_torus_representatives_match_the_sweep(shape, k, n_up):
    """oracle.torus_representatives (orbit minima with trivial stabiliser character, enumerated
    without a parent basis) equals the visited-flag sweep's representative list."""
    L1, L2 = shape
    n = L1 * L2
    parent = O.popcount_basis(n, n_up)
    sites = O.spin_half_sites(n)
    bw, off = O.bit_layout(sites)
    maps, amps = O.translation_symops(shape, k)
    red = O.symmetry_reduce(parent, bw, off, maps, amps)
    assert np.array_equal(O.torus_representatives(shape, n_up, k), red.basis_list)


@pytest.mark.parametrize("shape,k", [((6, 4), (1, 2)), ((5, 4), (0, 0)), ((6, 3), (3, 1))])
def test_orbit_tables_torus_rotations_equal_site_loop(shape, k):
    """The torus variant of the orbit-by-orbit rows (elements applied by word rotations, used where the
    host restatement is timed) gives exactly the rows of the site-permutation loop."""
    L1, L2 = shape
    n = L1 * L2
    basis = O.torus_representatives(shape, n // 2, k)
    maps, amps = O.translation_symops(shape, k)
    terms = _torus_terms(shape, [(1, 0), (0, 1)], [(1, 1)], 1.0, 0.4, 0.8, np.random.default_rng(2))
    x = O.complex_gaussian(basis.size, 5)
    rows = np.arange(basis.size)
    a = O.OrbitTables(n, n // 2, maps, amps, basis).rows(terms, x, rows)
    b = O.OrbitTables(n, n // 2, maps, amps, basis, torus=shape).rows(terms, x, rows)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
