"""Pins the oracle (CPU restatement of the reference) against the golden vectors the reference's own
tests assert (tests/golden/reference_tests.json, transcribed from test/*.jl).  CPU only."""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_tests.json")))
TOL = math.sqrt(np.finfo(float).eps)


def test_spinhalf_sectors():
    g = GOLD["spinhalf_L4_sectors"]
    sites = O.spin_half_sites(g["n_sites"])
    assert O.quantum_number_sectors(sites) == sorted((int(k),) for k in g["sectors"])
    for q, basis in g["sectors"].items():
        assert O.hs_get_basis_list(sites, [(int(q),)]).tolist() == basis
    assert O.hs_get_basis_list(sites).tolist() == GOLD["spinhalf_L4_full"]["basis"]


def test_tJ_multibit_sites():
    g = GOLD["tJ"]
    sites = [[tuple(q) for q in s] for s in g["sites"]]
    assert O.quantum_number_sectors(sites) == [tuple(q) for q in g["sectors"]]
    assert O.hs_get_basis_list(sites).tolist() == g["all_basis"]
    for qn, basis in g["qn_basis"]:
        assert O.hs_get_basis_list(sites, [tuple(qn)]).tolist() == basis
    assert O.hs_get_basis_list(sites, [tuple(q) for q in g["union_qns"]]).tolist() == g["union_basis"]
    assert O.hs_get_basis_list(sites, []).tolist() == []


def test_br_too_small():
    g = GOLD["br_too_small"]
    with pytest.raises(O.ArgumentError):
        O.hs_get_basis_list(O.spin_half_sites(g["n_sites"]), [(0,)], nbits_type=g["word_bits"])


def test_frozen_sorted_checks():
    g = GOLD["frozen_sorted"]
    with pytest.raises(O.ArgumentError):
        O.check_frozen_sorted(np.array(g["unsorted"]))
    with pytest.raises(O.ArgumentError):
        O.check_frozen_sorted(np.array(g["duplicates"]))
    keys = np.array([1, 2, 3, 4, 5], dtype=np.uint64)
    assert O.lookup(keys, np.array([1, 5, 6, 0], dtype=np.uint64)).tolist() == [0, 4, -1, -1]


def _l4():
    sites = O.spin_half_sites(4)
    parent = O.hs_get_basis_list(sites, [(0,)])
    bw, off = O.bit_layout(sites)
    return sites, parent, bw, off


def test_translation_reps_L4():
    _, parent, bw, off = _l4()
    for idx, reps in GOLD["translation_L4"]["reps_by_irrep_index"].items():
        maps, amps = O.translation_symops((4, 1), (int(idx) - 1, 0))
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        assert red.basis_list.tolist() == reps


def test_mapping_invariants_and_roundtrip():
    # test_symmetry_reduce.jl:52-99
    _, parent, bw, off = _l4()
    total = 0
    rng = np.random.default_rng(0)
    for m in range(4):
        maps, amps = O.translation_symops((4, 1), (m, 0))
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        total += red.dim
        for ip, b in enumerate(parent):
            if b in red.basis_list:
                assert 0 <= red.basis_mapping_index[ip] < red.dim
                assert red.basis_list[red.basis_mapping_index[ip]] == b
                assert abs(red.basis_mapping_amplitude[ip].imag) <= TOL
        for ip, ir in enumerate(red.basis_mapping_index):
            if ir == -1:
                assert parent[ip] not in red.basis_list
        sv = rng.random(red.dim) + 1j * rng.random(red.dim)
        lv = O.unreduce(red, sv)
        assert np.allclose(O.reduce_vector(red, lv), sv, atol=TOL)
    assert total == parent.size


def test_point_and_symmorphic_reps_L4():
    _, parent, bw, off = _l4()
    g = GOLD["point_L4"]
    ident = list(range(4))
    for irr in g["irreps"]:
        maps = np.array([ident, g["inversion_map"]], dtype=np.int32)
        red = O.symmetry_reduce(parent, bw, off, maps, np.array(irr["chars"], dtype=complex))
        assert red.basis_list.tolist() == irr["reps"]
    # translations x inversion (dihedral group of order 8), k = 0, inversion character +1 / -1
    tmaps, tamps = O.translation_symops((4, 1), (0, 0))
    inv = g["inversion_map"]
    for sign, key in ((1, "k0_even_reps"), (-1, "k0_odd_reps")):
        maps, amps = [], []
        for t in range(4):
            for p, chi in ((ident, 1), (inv, sign)):
                maps.append([p[tmaps[t][i]] for i in range(4)])      # p * t
                amps.append(chi * tamps[t])
        red = O.symmetry_reduce(parent, bw, off, np.array(maps, dtype=np.int32), np.array(amps))
        assert red.basis_list.tolist() == GOLD["symmorphic_L4"][key]


def test_momentum_phase_convention_L7():
    g = GOLD["convention_L7"]
    sites = O.spin_half_sites(g["n_sites"])
    bw, off = O.bit_layout(sites)
    maps, amps = O.translation_symops((7, 1), (g["irrep_index"] - 1, 0))
    for case in ("particle", "hole"):
        c = g[case]
        parent = O.hs_get_basis_list(sites, [(c["sector"],)])
        assert parent.tolist() == c["basis"]
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        assert red.basis_list.tolist() == c["reps"]
        psi = O.unreduce(red, np.array([1.0 + 0j]))
        want = [np.exp(c["phase_sign"] * 2j * np.pi * i / 7) / np.sqrt(7) for i in range(7)]
        assert np.allclose(psi, want, atol=TOL)


def test_reduced_hamiltonian_explicit_L4():
    g = GOLD["reduced_H_L4"]
    _, parent, bw, off = _l4()
    assert parent.tolist() == g["parent_basis"]
    _, offs = O.bit_layout(O.spin_half_sites(4))
    j1 = []
    for i in range(4):
        for s in "xyz":
            j1 += O.op_mul(O.pauli_matrix(offs, i, s), O.pauli_matrix(offs, (i + 1) % 4, s))
    full = O.dense_matrix(parent, j1)
    psis = [np.array(p) / np.linalg.norm(p) for p in g["psis"]]
    H = np.array([[psis[i] @ (full @ psis[j]) for j in range(2)] for i in range(2)])
    maps, amps = O.translation_symops((4, 1), (0, 0))
    red = O.symmetry_reduce(parent, bw, off, maps, amps)
    assert red.basis_list.tolist() == g["reps"]
    assert np.allclose(O.dense_matrix(red, j1), H, atol=TOL)
    # row and column iterators agree (no dropped weight): transpose product of unit vectors
    M = O.dense_matrix(red, j1)
    for c in range(2):
        e = np.zeros(2, dtype=complex)
        e[c] = 1
        assert np.allclose(O.apply_cols(red, j1, e), M[c, :], atol=TOL)


def test_spectrum_union_over_momenta_L4_and_L8():
    for L in (4, 8):
        sites = O.spin_half_sites(L)
        parent = O.hs_get_basis_list(sites, [(0,)])
        bw, off = O.bit_layout(sites)
        terms = O.heisenberg_terms(L, [(i, (i + 1) % L) for i in range(L)], [1.0] * L, [1.0] * L)
        full = O.dense_matrix(parent, terms)
        assert np.allclose(full, full.conj().T, atol=TOL)
        ev = []
        for m in range(L):
            maps, amps = O.translation_symops((L, 1), (m, 0))
            red = O.symmetry_reduce(parent, bw, off, maps, amps)
            Hr = O.dense_matrix(red, terms)
            assert np.allclose(Hr, Hr.conj().T, atol=TOL)
            ev += list(np.linalg.eigvalsh(Hr))
        assert np.allclose(sorted(ev), np.linalg.eigvalsh(full), atol=1e-10)


def test_unreduced_rows_equal_columns_L7():
    sites = O.spin_half_sites(7)
    parent = O.hs_get_basis_list(sites, [(1,)])
    terms = O.heisenberg_terms(7, [(i, (i + 1) % 7) for i in range(7)], [1.0] * 7, [1.0] * 7)
    M = O.dense_matrix(parent, terms)
    for c in range(parent.size):
        e = np.zeros(parent.size, dtype=complex)
        e[c] = 1
        assert np.allclose(O.apply_cols(parent, terms, e), M[c, :], atol=1e-12)


def test_symmetry_apply_and_bitflip_bits():
    g = GOLD["symmetry_apply"]
    bw, off = O.bit_layout(O.spin_half_sites(4))
    for b, want in g["state_cases"]:
        assert O.symmetry_apply(bw, off, g["transop"], b) == want
    gb = GOLD["bitflip"]
    full = 0b1111
    ident = [0, 1, 2, 3]
    assert O.symmetry_apply(bw, off, ident, gb["cases"]["b0"][0]) == gb["cases"]["b0"][1]
    assert O.symmetry_apply(bw, off, ident, gb["cases"]["b1"][0], flip=full) == gb["cases"]["b1"][1]
    assert O.symmetry_apply(bw, off, gb["perm"], gb["cases"]["p_b0"][0]) == gb["cases"]["p_b0"][1]
    assert O.symmetry_apply(bw, off, gb["perm"], gb["cases"]["p_b1"][0], flip=full) == gb["cases"]["p_b1"][1]


def test_invalid_targets_dropped():
    g = GOLD["oprep_iterator"]
    basis = np.array(g["basis"], dtype=np.uint64)
    terms = [(m, r, c, complex(a)) for m, r, c, a in g["terms"]]
    x = np.array([1.0 + 0j, 2.0])
    assert np.allclose(O.apply_rows(basis, terms, x), 0)
    go = GOLD["out_of_sector"]
    sites = O.spin_half_sites(go["n_sites"])
    parent = O.hs_get_basis_list(sites, [(0,)])
    _, offs = O.bit_layout(sites)
    sx = O.pauli_matrix(offs, go["site"], "x")
    st = np.full(parent.size, complex(*go["state_value"]))
    assert np.allclose(O.apply_rows(parent, sx, st), 0)
    assert np.allclose(O.apply_cols(parent, sx, st), 0)


def test_apply_semantics_full_space():
    # apply! adds, mul! overwrites; transpose product (test_operator_representation.jl:181-272)
    sites = O.spin_half_sites(4)
    basis = O.hs_get_basis_list(sites)
    _, offs = O.bit_layout(sites)
    sp = O.pauli_matrix(offs, 1, "+")
    s_plus = np.array([[0, 1], [0, 0]])
    s0 = np.eye(2)
    dense = np.kron(np.kron(np.kron(s0, s0), s_plus), s0)   # Julia kron(s0,s0,s+,s0): site 1 is the fastest index
    rng = np.random.default_rng(1)
    state = rng.random(16) + 1j * rng.random(16)
    out = O.apply_rows(basis, sp, state)
    assert np.allclose(out, dense @ state)
    out2 = O.apply_rows(basis, sp, state, out=out.copy(), accumulate=True)
    assert np.allclose(out2, 2 * dense @ state)
    assert np.allclose(O.apply_cols(basis, sp, state), state @ dense)


def test_heisenberg_simplify_structure():
    # test_operator_simplify.jl:75-90: simplify of sum sigma.sigma has the terms of 2 s+s- + 2 s-s+ + sz sz
    n = 4
    _, offs = O.bit_layout(O.spin_half_sites(n))
    h1 = []
    for i in range(n):
        j = (i + 1) % n
        h1 += O.op_scale(2, O.op_mul(O.pauli_matrix(offs, i, "+"), O.pauli_matrix(offs, j, "-")))
        h1 += O.op_scale(2, O.op_mul(O.pauli_matrix(offs, i, "-"), O.pauli_matrix(offs, j, "+")))
        h1 += O.op_mul(O.pauli_matrix(offs, i, "z"), O.pauli_matrix(offs, j, "z"))
    h2 = []
    for i in range(n):
        for s in "xyz":
            h2 += O.op_mul(O.pauli_matrix(offs, i, s), O.pauli_matrix(offs, (i + 1) % n, s))
    assert set(O.simplify(h1)) == set(O.simplify(h2))
    assert len(O.simplify(h2)) == 6 * n


def test_popcount_basis_matches_dp():
    for n, k in [(10, 5), (14, 7), (12, 3)]:
        assert np.array_equal(O.popcount_basis(n, k), O.hs_get_basis_list(O.spin_half_sites(n), [(n - 2 * k,)]))


def test_lanczos_oracle_matches_dense():
    L = 10
    sites = O.spin_half_sites(L)
    parent = O.hs_get_basis_list(sites, [(0,)])
    terms = O.heisenberg_terms(L, [(i, (i + 1) % L) for i in range(L)], [1.0] * L, [1.0] * L)
    e_dense = np.linalg.eigvalsh(O.dense_matrix(parent, terms))[0]
    e0, _, _ = O.lanczos_e0(lambda v: O.apply_rows(parent, terms, v), parent.size, 80, seed=1)
    assert abs(e0 - e_dense) < 1e-10 * abs(e_dense)
