"""Parity of the CUDA path (through the C ABI) against the oracle.

Integer work (basis, representatives, indices) must match bit for bit; FP64 products within 1e-12
relative (the reference's own tolerance for this path is 1e-10); mixed precision within 1e-5.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_tests.json")))
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


def chain_case(E, L, sector=0):
    hs, _ = E.spin_half_system(L)
    hsr = E.represent(E.HilbertSpaceSector(hs, sector))
    sites = O.spin_half_sites(L)
    parent = O.hs_get_basis_list(sites, [(sector,)])
    bw, off = O.bit_layout(sites)
    return hs, hsr, parent, bw, off


# ---------------------------------------------------------------------------------------------------
# sector basis and lookup
# ---------------------------------------------------------------------------------------------------

@pytest.mark.parametrize("L", [1, 4, 9, 16, 20])
def test_sector_bases_bitexact(edgpu, L):
    hs, _ = edgpu.spin_half_system(L)
    sites = O.spin_half_sites(L)
    for q in O.quantum_number_sectors(sites):
        hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, q))
        want = O.popcount_basis(L, (L - q[0]) // 2)
        assert np.array_equal(hsr.basis_list, want)
    full = edgpu.represent(hs)
    assert np.array_equal(full.basis_list, np.arange(2 ** L, dtype=np.uint64))


def test_golden_spinhalf_and_tJ(edgpu):
    g = GOLD["spinhalf_L4_sectors"]
    hs, _ = edgpu.spin_half_system(4)
    for q, basis in g["sectors"].items():
        assert edgpu.represent(edgpu.HilbertSpaceSector(hs, int(q))).basis_list.tolist() == basis
    t = GOLD["tJ"]
    sites = [edgpu.Site([edgpu.State(f"s{i}", tuple(q)) for i, q in enumerate(s)]) for s in t["sites"]]
    hs = edgpu.HilbertSpace(sites)
    assert hs.quantum_number_sectors() == [tuple(q) for q in t["sectors"]]
    assert edgpu.represent(hs).basis_list.tolist() == t["all_basis"]
    assert edgpu.represent(edgpu.HilbertSpaceSector(hs, [tuple(q) for q in t["sectors"]])).basis_list.tolist() == \
        t["all_basis"]
    for qn, basis in t["qn_basis"]:
        hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, tuple(qn)))
        assert hsr.basis_list.tolist() == basis
        assert [hsr.basis_lookup(b) for b in basis] == list(range(len(basis)))
        assert hsr == edgpu.represent(hs, np.array(basis, dtype=np.uint64))
    u = edgpu.represent(edgpu.HilbertSpaceSector(hs, [tuple(q) for q in t["union_qns"]]))
    assert u.basis_list.tolist() == t["union_basis"]
    assert edgpu.represent(hs, np.array(t["unsorted_input"], dtype=np.uint64)).basis_list.tolist() == \
        t["union_basis"]
    assert edgpu.represent(edgpu.HilbertSpaceSector(hs, [])).basis_list.tolist() == []


def test_basis_errors(edgpu):
    hs, _ = edgpu.spin_half_system(4)
    with pytest.raises(edgpu.ArgumentError):
        edgpu.represent(hs, np.array([3, 3, 5], dtype=np.uint64))
    big = edgpu.HilbertSpace([edgpu.Site([edgpu.State("Up", 1), edgpu.State("Dn", -1)])] * 64)
    with pytest.raises(edgpu.ArgumentError):
        edgpu.represent(edgpu.HilbertSpaceSector(big, 0))


def test_lookup_matches_oracle(edgpu):
    hs, hsr, parent, _, _ = chain_case(edgpu, 16)
    rng = np.random.default_rng(3)
    keys = np.concatenate([parent[rng.integers(0, parent.size, 500)],
                           rng.integers(0, 2 ** 16, 500).astype(np.uint64),
                           np.array([0, 2 ** 16 - 1, 2 ** 40], dtype=np.uint64)])
    assert np.array_equal(hsr.lookup(keys), O.lookup(parent, keys))
    with pytest.raises(KeyError):
        hsr.basis_lookup(0)


# ---------------------------------------------------------------------------------------------------
# representatives, mapping tables, phase convention
# ---------------------------------------------------------------------------------------------------

@pytest.mark.parametrize("L", [4, 7, 8, 12, 16, 20])
def test_chain_reps_and_mapping(edgpu, L):
    hs, hsr, parent, bw, off = chain_case(edgpu, L, 0 if L % 2 == 0 else 1)
    total = 0
    for m in range(L):
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m))
        maps, amps = O.translation_symops((L, 1), (m, 0))
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        assert np.array_equal(rh.basis_list, red.basis_list)
        assert np.array_equal(rh.basis_mapping_index, red.basis_mapping_index)
        assert np.abs(rh.basis_mapping_amplitude - red.basis_mapping_amplitude).max() < 1e-13
        total += rh.dimension
    assert total == parent.size


TORI = [(2, 2), (4, 2), (3, 3), (4, 4), (6, 3), (5, 4)]


@pytest.mark.parametrize("shape", TORI)
def test_torus_reps_and_mapping(edgpu, shape):
    L1, L2 = shape
    n = L1 * L2
    hs, hsr, parent, bw, off = chain_case(edgpu, n, 0 if n % 2 == 0 else 1)
    total = 0
    for m2 in range(L2):
        for m1 in range(L1):
            rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(shape, (m1, m2)))
            maps, amps = O.translation_symops(shape, (m1, m2))
            red = O.symmetry_reduce(parent, bw, off, maps, amps)
            assert np.array_equal(rh.basis_list, red.basis_list)
            assert np.array_equal(rh.basis_mapping_index, red.basis_mapping_index)
            assert np.abs(rh.basis_mapping_amplitude - red.basis_mapping_amplitude).max() < 1e-13
            total += rh.dimension
    assert total == parent.size


def test_golden_translation_point_symmorphic_L4(edgpu):
    hs, hsr, parent, bw, off = chain_case(edgpu, 4)
    for idx, reps in GOLD["translation_L4"]["reps_by_irrep_index"].items():
        assert edgpu.symmetry_reduce(hsr, edgpu.translation_symops(4, int(idx) - 1)).basis_list.tolist() == reps
    g = GOLD["point_L4"]
    E = edgpu.SitePermutation([0, 1, 2, 3])
    inv = edgpu.SitePermutation(g["inversion_map"])
    for irr in g["irreps"]:
        rh = edgpu.symmetry_reduce(hsr, [(E, irr["chars"][0]), (inv, irr["chars"][1])])
        assert rh.basis_list.tolist() == irr["reps"]
    for sign, key in ((1, "k0_even_reps"), (-1, "k0_odd_reps")):
        ops = []
        for t, a in edgpu.translation_symops(4, 0):
            for p, chi in ((E, 1), (inv, sign)):
                ops.append((edgpu.SitePermutation([p.map[t.map[i]] for i in range(4)]), chi * a))
        assert edgpu.symmetry_reduce(hsr, ops).basis_list.tolist() == GOLD["symmorphic_L4"][key]


def test_generic_group_with_bitflip_matches_oracle(edgpu):
    # translations x global spin flip on an L=10 chain, every (k, flip parity)
    L = 10
    hs, hsr, parent, bw, off = chain_case(edgpu, L)
    full = (1 << L) - 1
    for m in (0, 1, 5):
        for par in (1, -1):
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
            assert np.array_equal(rh.basis_list, red.basis_list)
            assert np.array_equal(rh.basis_mapping_index, red.basis_mapping_index)
            assert np.abs(rh.basis_mapping_amplitude - red.basis_mapping_amplitude).max() < 1e-13


def test_phase_convention_L7(edgpu):
    g = GOLD["convention_L7"]
    hs, _ = edgpu.spin_half_system(7)
    for case in ("particle", "hole"):
        c = g[case]
        hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, c["sector"]))
        assert hsr.basis_list.tolist() == c["basis"]
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(7, g["irrep_index"] - 1))
        assert rh.basis_list.tolist() == c["reps"]
        psi = edgpu.symmetry_unreduce(rh, np.array([1.0 + 0j]))
        want = [np.exp(c["phase_sign"] * 2j * np.pi * i / 7) / np.sqrt(7) for i in range(7)]
        assert np.allclose(psi, want, atol=1e-14)


def test_reduce_unreduce_roundtrip(edgpu):
    hs, hsr, parent, _, _ = chain_case(edgpu, 12)
    rng = np.random.default_rng(5)
    for m in range(12):
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(12, m))
        sv = rng.random(rh.dimension) + 1j * rng.random(rh.dimension)
        assert np.allclose(edgpu.symmetry_reduce(rh, edgpu.symmetry_unreduce(rh, sv)), sv, atol=1e-13)
        with pytest.raises(edgpu.DimensionMismatch):
            edgpu.symmetry_unreduce(rh, np.zeros(rh.dimension + 1))
        with pytest.raises(edgpu.DimensionMismatch):
            edgpu.symmetry_reduce(rh, np.zeros(parent.size + 1))


def test_symmetry_argument_errors(edgpu):
    hs, hsr, _, _, _ = chain_case(edgpu, 6)
    ops = edgpu.translation_symops(6, 1)
    with pytest.raises(edgpu.ArgumentError):
        edgpu.symmetry_reduce(hsr, [(op, 2.0 * a) for op, a in ops])            # non-unit amplitudes
    with pytest.raises(edgpu.ArgumentError):
        edgpu.symmetry_reduce(hsr, ops[:3])                                     # not a group
    with pytest.raises(edgpu.ArgumentError):
        edgpu.symmetry_reduce(hsr, [ops[1], ops[0]] + ops[2:])                  # identity not first
    with pytest.raises(edgpu.ArgumentError):
        edgpu.symmetry_reduce(hsr, [(op, a if i != 1 else 1j) for i, (op, a) in enumerate(ops)])  # not a rep


# ---------------------------------------------------------------------------------------------------
# the product
# ---------------------------------------------------------------------------------------------------

def xxz_terms_both(E, n, bonds, jxy, jz):
    from edgpu import lattice
    hs, _ = E.spin_half_system(n)
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    return H, O.heisenberg_terms(n, bonds, jxy, jz)


SCHEDULES = (-1, -2, -4, 32, 8)   # 1, 2, 4 lanes per row; queued with 32 and 8 rows per warp tile


def check_product(E, opr, space_oracle, terms, N, seed=11):
    x = O.complex_gaussian(N, seed)
    want = O.apply_rows(space_oracle, terms, x)
    for sched in SCHEDULES:
        opr.set_tiling("fp64", sched)
        opr.set_tiling("mixed", sched)
        y = np.zeros(N, dtype=np.complex128)
        E.mul_(y, opr, x, precision="fp64")
        assert relerr(y, want) < FP64_TOL, sched
        y32 = np.zeros(N, dtype=np.complex128)
        E.mul_(y32, opr, x, precision="mixed")
        assert relerr(y32, want) < MIXED_TOL, sched
    opr.set_tiling("fp64", 0)
    opr.set_tiling("mixed", 0)
    # apply! adds; mul! overwrites
    y2 = y.copy()
    E.apply_(y2, opr, x)
    assert relerr(y2, 2 * want) < FP64_TOL
    E.mul_(y2, opr, x)
    assert relerr(y2, want) < FP64_TOL
    # transpose product (row vector times the matrix)
    yt = np.zeros(N, dtype=np.complex128)
    E.apply_(yt, x, opr)
    assert relerr(yt, O.apply_cols(space_oracle, terms, x)) < FP64_TOL


@pytest.mark.parametrize("L", [6, 12, 16, 20])
def test_unreduced_product(edgpu, L):
    hs, hsr, parent, _, _ = chain_case(edgpu, L)
    rng = np.random.default_rng(L)
    bonds = [(i, (i + 1) % L) for i in range(L)] + [(i, (i + 2) % L) for i in range(L)]
    jxy = list(rng.uniform(0.5, 1.5, len(bonds)))
    jz = list(rng.uniform(-1.0, 1.0, len(bonds)))
    H, terms = xxz_terms_both(edgpu, L, bonds, jxy, jz)
    check_product(edgpu, edgpu.represent(hsr, H), parent, terms, parent.size)


@pytest.mark.parametrize("L", [8, 12, 16, 20])
def test_reduced_chain_product_all_momenta(edgpu, L):
    hs, hsr, parent, bw, off = chain_case(edgpu, L)
    bonds = [(i, (i + 1) % L) for i in range(L)] + [(i, (i + 2) % L) for i in range(L)]
    H, terms = xxz_terms_both(edgpu, L, bonds, [1.0] * L + [0.3] * L, [0.8] * L + [0.24] * L)
    for m in range(L):
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m))
        maps, amps = O.translation_symops((L, 1), (m, 0))
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        check_product(edgpu, edgpu.represent(rh, H), red, terms, rh.dimension, seed=m + 1)


@pytest.mark.parametrize("shape", [(3, 3), (4, 4), (6, 3), (4, 5)])
def test_reduced_torus_product(edgpu, shape):
    L1, L2 = shape
    n = L1 * L2
    sector = 0 if n % 2 == 0 else 1
    hs, hsr, parent, bw, off = chain_case(edgpu, n, sector)
    bonds, jxy, jz = [], [], []
    for (dx, dy), j in (((1, 0), 1.0), ((0, 1), 1.0), ((1, 1), 0.5), ((1, -1), 0.5)):
        for y in range(L2):
            for x in range(L1):
                bonds.append((x + L1 * y, (x + dx) % L1 + L1 * ((y + dy) % L2)))
                jxy.append(j)
                jz.append(0.8 * j)
    H, terms = xxz_terms_both(edgpu, n, bonds, jxy, jz)
    for (m1, m2) in [(0, 0), (1, 0), (0, 1), (L1 // 2, L2 // 2), (L1 - 1, 1)]:
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(shape, (m1, m2)))
        maps, amps = O.translation_symops(shape, (m1, m2))
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        check_product(edgpu, edgpu.represent(rh, H), red, terms, rh.dimension, seed=m1 + 7 * m2)


def test_generic_group_product(edgpu):
    L = 10
    hs, hsr, parent, bw, off = chain_case(edgpu, L)
    full = (1 << L) - 1
    H, terms = xxz_terms_both(edgpu, L, [(i, (i + 1) % L) for i in range(L)], [1.0] * L, [1.0] * L)
    for m in (0, 3):
        for par in (1, -1):
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
            check_product(edgpu, edgpu.represent(rh, H), red, terms, rh.dimension)


def test_complex_and_non_hermitian_terms(edgpu):
    # sigma_+ sigma_- with complex amplitudes (a Dzyaloshinskii-Moriya-like chirality) and a
    # non-Hermitian sigma_+ sigma_+ sigma_- sigma_- pair term, reduced at several momenta
    L = 12
    hs, hsr, parent, bw, off = chain_case(edgpu, L)
    _, offs = O.bit_layout(O.spin_half_sites(L))
    op_o = []
    for i in range(L):
        j = (i + 1) % L
        op_o += O.op_scale(0.7 + 0.3j, O.op_mul(O.pauli_matrix(offs, i, "+"), O.pauli_matrix(offs, j, "-")))
        op_o += O.op_scale(0.2, O.op_mul(O.pauli_matrix(offs, i, "z"), O.pauli_matrix(offs, j, "z")))
        k = (i + 2) % L
        op_o += O.op_scale(0.1j, O.op_mul(O.op_mul(O.pauli_matrix(offs, i, "+"), O.pauli_matrix(offs, j, "+")),
                                         O.op_mul(O.pauli_matrix(offs, k, "-"), O.pauli_matrix(offs, (i + 3) % L, "-"))))
    m_, r_, c_, a_ = O.term_arrays(op_o)
    for m in range(0, L, 3):
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m))
        maps, amps = O.translation_symops((L, 1), (m, 0))
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        opr = edgpu.OperatorRepresentation.from_terms(rh, m_, r_, c_, a_)
        check_product(edgpu, opr, red, op_o, rh.dimension)
        # adjoint product on the device: H^dagger x = conj(transpose(H) conj(x))
        import torch
        x = O.complex_gaussian(rh.dimension, 9)
        want = np.conj(O.apply_cols(red, op_o, np.conj(x)))
        xd = torch.from_numpy(x).cuda()
        yd = torch.empty_like(xd)
        edgpu.mul_adjoint_(yd, opr, xd, precision="fp64")
        torch.cuda.synchronize()
        assert relerr(yd.cpu().numpy(), want) < FP64_TOL


def test_invalid_targets_are_dropped(edgpu):
    g = GOLD["oprep_iterator"]
    hs, _ = edgpu.spin_half_system(4)
    hsr = edgpu.represent(hs, np.array(g["basis"], dtype=np.uint64))
    t = np.array(g["terms"], dtype=object)
    opr = edgpu.OperatorRepresentation.from_terms(hsr, t[:, 0].astype(np.uint64), t[:, 1].astype(np.uint64),
                                                  t[:, 2].astype(np.uint64), t[:, 3].astype(complex))
    y = np.ones(2, dtype=complex)
    edgpu.mul_(y, opr, np.array([1.0 + 0j, 2.0]))
    assert np.allclose(y, 0)
    go = GOLD["out_of_sector"]
    hs, hsr, parent, _, _ = chain_case(edgpu, go["n_sites"])
    sx = edgpu.pauli_matrix(hs, go["site"], "x")
    opr = edgpu.represent(hsr, sx)
    st = np.full(parent.size, complex(*go["state_value"]))
    out = np.ones(parent.size, dtype=complex)
    edgpu.mul_(out, opr, st)
    assert np.allclose(out, 0)
    edgpu.apply_(out, st, opr)
    assert np.allclose(out, 0)


def test_dimension_mismatch(edgpu):
    hs, hsr, parent, _, _ = chain_case(edgpu, 6)
    opr = edgpu.represent(hsr, edgpu.pauli_matrix(hs, 0, "z"))
    n = parent.size
    for out, st in ((np.zeros(n + 1, complex), np.zeros(n, complex)), (np.zeros(n, complex), np.zeros(n + 1, complex))):
        with pytest.raises(edgpu.DimensionMismatch):
            edgpu.mul_(out, opr, st)
        with pytest.raises(edgpu.DimensionMismatch):
            edgpu.apply_(out, opr, st)
        with pytest.raises(edgpu.DimensionMismatch):
            edgpu.apply_(out, st, opr)


def test_golden_reduced_hamiltonian_L4(edgpu):
    g = GOLD["reduced_H_L4"]
    hs, hsr, parent, bw, off = chain_case(edgpu, 4)
    j1 = sum((edgpu.pauli_matrix(hs, i, s) * edgpu.pauli_matrix(hs, (i + 1) % 4, s)
              for i in range(4) for s in "xyz"), edgpu.NullOperator())
    full = np.zeros((6, 6), complex)
    opr_full = edgpu.represent(hsr, j1)
    for c in range(6):
        e = np.zeros(6, complex)
        e[c] = 1
        full[:, c] = opr_full @ e
    psis = [np.array(p) / np.linalg.norm(p) for p in g["psis"]]
    H = np.array([[psis[i] @ (full @ psis[j]) for j in range(2)] for i in range(2)])
    rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(4, 0))
    assert rh.basis_list.tolist() == g["reps"]
    opr = edgpu.represent(rh, j1)
    M = np.zeros((2, 2), complex)
    for c in range(2):
        e = np.zeros(2, complex)
        e[c] = 1
        M[:, c] = opr @ e
    assert np.allclose(M, H, atol=1e-14)


@pytest.mark.parametrize("L", [8, 12])
def test_spectrum_union_over_momenta(edgpu, L):
    hs, hsr, parent, _, _ = chain_case(edgpu, L)
    H, terms = xxz_terms_both(edgpu, L, [(i, (i + 1) % L) for i in range(L)], [1.0] * L, [1.0] * L)
    full = O.dense_matrix(parent, terms)
    ev = []
    for m in range(L):
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m))
        opr = edgpu.represent(rh, H)
        n = rh.dimension
        M = np.zeros((n, n), complex)
        for c in range(n):
            e = np.zeros(n, complex)
            e[c] = 1
            M[:, c] = opr @ e
        assert np.allclose(M, M.conj().T, atol=1e-13)
        ev += list(np.linalg.eigvalsh(M))
    assert np.allclose(sorted(ev), np.linalg.eigvalsh(full), atol=1e-10)


def test_random_vector_matches_oracle(edgpu):
    for n, seed in ((1, 3), (1000, 7), (112720, 2)):
        v = edgpu.random_state(n, seed, "fp64").cpu().numpy()
        assert relerr(v, O.complex_gaussian(n, seed)) < 1e-13
        v32 = edgpu.random_state(n, seed, "mixed").cpu().numpy()
        assert relerr(v32, O.complex_gaussian(n, seed)) < 1e-6
