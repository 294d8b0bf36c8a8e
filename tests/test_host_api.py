"""Host-side mirror of the reference API (no GPU): layouts, quantum numbers, operator algebra,
symmetry bookkeeping.  Checked against the golden vectors and the oracle."""
import json
import math
import os

import numpy as np
import pytest

import edgpu
from edgpu import lattice
from edgpu.representation import _as_map_flip, _roots_of_unity
from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_tests.json")))


def test_site_and_space_layout():
    up, dn = edgpu.State("Up", 1), edgpu.State("Dn", -1)
    assert up.quantum_number == (1,)
    s = edgpu.Site([up, dn])
    assert edgpu.bitwidth(s) == 1
    assert edgpu.bitwidth(edgpu.Site([up, edgpu.State("Ze", 0), dn])) == 2
    hs = edgpu.HilbertSpace([s] * 3)
    assert hs.bitwidths == [1, 1, 1] and hs.bitoffsets == [0, 1, 2, 3]
    assert edgpu.bitwidth(hs) == 3
    assert hs.get_bitmask(1) == 0b010 and hs.get_bitmask() == 0b111
    assert hs.compress((1, 1, 0)) == 0b011 and hs.extract(0b011) == (1, 1, 0)
    assert hs.get_quantum_number(0b011) == (-1,)


def test_tJ_sectors_and_sector_intersection():
    t = GOLD["tJ"]
    sites = [edgpu.Site([edgpu.State(f"s{i}", tuple(q)) for i, q in enumerate(s)]) for s in t["sites"]]
    hs = edgpu.HilbertSpace(sites)
    assert hs.bitwidths == [2, 1, 1]
    assert hs.quantum_number_sectors() == [tuple(q) for q in t["sectors"]]
    hss = edgpu.HilbertSpaceSector(hs, [(3, 3), (9, 9)])
    assert hss.allowed_quantum_numbers == {(3, 3)}
    assert edgpu.HilbertSpaceSector(hs).allowed_quantum_numbers == set(tuple(q) for q in t["sectors"])


def test_pure_operator_invariant_and_algebra():
    with pytest.raises(edgpu.ArgumentError):
        edgpu.PureOperator(0b01, 0b10, 0b00, 1.0)
    with pytest.raises(edgpu.ArgumentError):
        edgpu.PureOperator(0b01, 0b00, 0b10, 1.0)
    hs, pauli = edgpu.spin_half_system(4)
    sp, sm = pauli(0, "+"), pauli(0, "-")
    prod = sp * sm                                  # |Up><Dn| |Dn><Up| = |Up><Up|
    assert isinstance(prod, edgpu.PureOperator) and (prod.bitrow, prod.bitcol) == (0, 0)
    assert isinstance(sp * sp, edgpu.NullOperator)
    assert edgpu.simplify(sp - sp) == edgpu.NullOperator()
    x = edgpu.simplify(pauli(0, "x") + pauli(0, "x"))
    assert isinstance(x, edgpu.SumOperator) and all(t.amplitude == 2 for t in x.terms)


def dense_1site(op):
    M = np.zeros((2, 2), complex)
    for t in op.terms:
        M[t.bitrow, t.bitcol] += t.amplitude
    return M


def test_pauli_matrices():
    hs, pauli = edgpu.spin_half_system(1)
    assert np.allclose(dense_1site(pauli(0, "x")), [[0, 1], [1, 0]])
    assert np.allclose(dense_1site(pauli(0, "y")), [[0, -1j], [1j, 0]])
    assert np.allclose(dense_1site(pauli(0, "z")), [[1, 0], [0, -1]])
    assert np.allclose(dense_1site(pauli(0, "+")), [[0, 1], [0, 0]])
    assert np.allclose(dense_1site(pauli(0, "-")), [[0, 0], [1, 0]])
    with pytest.raises(edgpu.ArgumentError):
        pauli(0, "q")
    with pytest.raises(edgpu.ArgumentError):
        edgpu.spin_half_system(65)


@pytest.mark.parametrize("n", [4, 7, 12])
def test_xxz_terms_equal_oracle(n):
    hs, _ = edgpu.spin_half_system(n)
    bonds = lattice.chain_bonds(n) + [(i, (i + 2) % n) for i in range(n)]
    rng = np.random.default_rng(n)
    jxy, jz = rng.random(len(bonds)), rng.random(len(bonds))
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    want = O.heisenberg_terms(n, bonds, list(jxy), list(jz))
    got = [(t.bitmask, t.bitrow, t.bitcol, t.amplitude) for t in H.terms]
    assert len(got) == len(want)
    for a, b in zip(sorted(got, key=lambda t: t[:3]), sorted(want, key=lambda t: t[:3])):
        assert a[:3] == b[:3] and abs(a[3] - b[3]) < 1e-15


def test_symmetry_apply_golden():
    g = GOLD["symmetry_apply"]
    hs, _ = edgpu.spin_half_system(4)
    P = edgpu.SitePermutation(g["transop"])
    for b, want in g["state_cases"]:
        assert edgpu.symmetry_apply(hs, P, b) == (want, 1)
    gb = GOLD["bitflip"]
    p = edgpu.SitePermutation(gb["perm"])
    for key, op in (("b0", edgpu.GlobalBitFlip(False)), ("b1", edgpu.GlobalBitFlip(True)),
                    ("p_b0", p * edgpu.GlobalBitFlip(False)), ("p_b1", p * edgpu.GlobalBitFlip(True))):
        b, want = gb["cases"][key]
        assert edgpu.symmetry_apply(hs, op, b)[0] == want


def test_translation_symops_convention_matches_oracle():
    for shape, k in (((7, 1), (2, 0)), ((6, 5), (1, 3)), ((4, 4), (2, 1))):
        ops = edgpu.translation_symops(shape, k)
        maps, amps = O.translation_symops(shape, k)
        assert [op.map for op, _ in ops] == maps.tolist()
        assert np.allclose([a for _, a in ops], amps)
        assert ops[0][0].map == list(range(shape[0] * shape[1])) and ops[0][1] == 1


def test_roots_of_unity():
    amps = [np.exp(2j * np.pi * k / 12) for k in range(12)]
    num, den = _roots_of_unity(amps, 1e-8)
    assert den == 12 and num == list(range(12))
    num, den = _roots_of_unity([1, -1, 1j, -1j], 1e-8)
    assert den == 4 and num == [0, 2, 1, 3]
    with pytest.raises(edgpu.ArgumentError):
        _roots_of_unity([1, 2.0], 1e-8)
    with pytest.raises(edgpu.ArgumentError):
        _roots_of_unity([1, np.exp(2j * np.pi * 0.123456789)], 1e-13)


def test_direct_product_bit_action():
    hs, _ = edgpu.spin_half_system(4)
    p = edgpu.SitePermutation([1, 2, 3, 0])
    m, f = _as_map_flip(hs, p * edgpu.GlobalBitFlip(True))
    assert m == [1, 2, 3, 0] and f == 0b1111


def test_representation_algebra_host_side():
    """opr + opr, opr - opr, number * opr, opr / number, -opr and ishermitian re-represent the combined,
    simplified operators (abstract_operator_representation.jl:55-107); checked on the host term tables
    without touching the device."""
    import edgpu
    from edgpu import operators as ops
    hs, _ = edgpu.spin_half_system(4)
    a = edgpu.pauli_matrix(hs, 0, "x") * edgpu.pauli_matrix(hs, 1, "x")
    b = edgpu.pauli_matrix(hs, 1, "+") * edgpu.pauli_matrix(hs, 2, "-")
    assert isinstance(ops.simplify(a - a), ops.NullOperator)
    s = ops.simplify(a + 2.0 * a)
    assert all(abs(t.amplitude - 3.0 * u.amplitude) < 1e-15 for t, u in zip(s.terms, ops.simplify(a).terms))
    h = ops.simplify(b + b.adjoint())
    assert isinstance(ops.simplify(h - h.adjoint()), ops.NullOperator)
    assert not isinstance(ops.simplify(b - b.adjoint()), ops.NullOperator)
