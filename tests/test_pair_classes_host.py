"""Host side of the pair-flip schedule, without a GPU: the bond classes the library builds for a
term table (edgpu_pair_classes_of_terms) satisfy their invariants, and a plain-Python walk of a row's
targets through them (the product kernel's algorithm: x_s = b ^ rotr_n(b, s), D = OR_s (x_s & A_s) |
(~x_s & P_s), amplitude by b_i and parallel/antiparallel) reproduces the oracle's row iterator
(operator_iterator.jl:48-54 through reduced_operator_representation.jl:57-85) on unreduced sectors."""
import ctypes

import numpy as np
import pytest

from edgpu import _lib, lattice
from edgpu._lib import ptr
from oracle import oracle as O

MAXC = 4


def classes_of(n, terms):
    m, r, c, a = O.term_arrays(terms)
    amps = np.ascontiguousarray(np.stack([a.real, a.imag], axis=1).reshape(-1))
    L = _lib.lib()
    nc = ctypes.c_int32()
    _lib.check(L.edgpu_pair_classes_of_terms(n, len(m), ptr(m, ctypes.c_uint64), ptr(r, ctypes.c_uint64),
                                             ptr(c, ctypes.c_uint64), ptr(amps, ctypes.c_double), 0,
                                             ctypes.byref(nc), None, None, None, None))
    k = nc.value
    if k == 0:
        return []
    info = np.zeros(k, np.int32)
    comps = np.zeros(k * MAXC * 3, np.uint64)
    flips = np.zeros(k * n, np.uint64)
    camps = np.zeros(k * n * 8, np.float64)
    _lib.check(L.edgpu_pair_classes_of_terms(n, len(m), ptr(m, ctypes.c_uint64), ptr(r, ctypes.c_uint64),
                                             ptr(c, ctypes.c_uint64), ptr(amps, ctypes.c_double), k,
                                             ctypes.byref(nc), ptr(info, ctypes.c_int32), ptr(comps, ctypes.c_uint64),
                                             ptr(flips, ctypes.c_uint64), ptr(camps, ctypes.c_double)))
    out = []
    for ci in range(k):
        nco = int(info[ci]) & 0xFF
        comp = [tuple(int(v) for v in comps[(ci * MAXC + j) * 3:(ci * MAXC + j) * 3 + 3]) for j in range(nco)]
        fl = [int(v) for v in flips[ci * n:(ci + 1) * n]]
        am = camps[ci * n * 8:(ci + 1) * n * 8].reshape(n, 4, 2)
        out.append(dict(par=bool(int(info[ci]) >> 8), comps=comp, flips=fl, amps=am[..., 0] + 1j * am[..., 1]))
    return out


def walk(n, cls, basis, diag_terms, x):
    """y = H x over an unreduced basis by the pair-flip walk through the classes."""
    full = (1 << n) - 1
    index = {int(b): i for i, b in enumerate(basis)}
    y = np.zeros(len(basis), complex)
    for r, b in enumerate(basis):
        b = int(b)
        acc = sum(a for (mk, rw, cl, a) in diag_terms if (b & mk) == rw) * x[r]
        for C in cls:
            D = 0
            for s, A, P in C["comps"]:
                xs = b ^ (((b >> s) | (b << (n - s))) & full)
                D |= (xs & A) | (~xs & P)
            while D:
                i = (D & -D).bit_length() - 1
                D &= D - 1
                f = C["flips"][i]
                v = (b >> i) & 1
                if C["par"]:
                    v |= int(bin(b & f).count("1") != 1) << 1
                c = index.get(b ^ f, -1)
                if c >= 0:
                    acc += C["amps"][i][v] * x[c]
        y[r] = acc
    return y


def check_classes(n, cls):
    for C in cls:
        assert 1 <= len(C["comps"]) <= MAXC
        starts = 0
        for s, A, P in C["comps"]:
            assert 1 <= s < n
            assert (A | P) & starts == 0                 # each start bit in one component only
            starts |= A | P
            for i in range(n):
                if (A | P) >> i & 1:
                    assert C["flips"][i] == (1 << i) | (1 << ((i + s) % n))


@pytest.mark.parametrize("shape,vectors,expected", [
    ((12, 1), [(1, 0)], (1, 1)),
    ((12, 1), [(1, 0), (2, 0)], (2, 2)),
    ((4, 4), lattice.SQUARE_NN + lattice.SQUARE_NNN, (4, 5)),
    ((6, 6), lattice.SQUARE_NN + lattice.SQUARE_NNN, (4, 5)),
    ((6, 5), lattice.TRIANGULAR_NN + lattice.TRIANGULAR_NNN, None),
])
def test_class_counts_and_invariants(shape, vectors, expected):
    L1, L2 = shape
    n = L1 * L2
    bonds = lattice.torus_bonds(L1, L2, vectors)
    terms = O.heisenberg_terms(n, bonds, [1.0] * len(bonds), [0.5] * len(bonds))
    cls = classes_of(n, terms)
    check_classes(n, cls)
    assert sum(bin(A | P).count("1") for C in cls for _, A, P in C["comps"]) == len(set(
        tuple(sorted(b)) for b in bonds))
    if expected:
        assert (len(cls), sum(len(C["comps"]) for C in cls)) == expected


@pytest.mark.parametrize("n,sector", [(10, 0), (12, 2)])
def test_walk_matches_oracle_xxz(n, sector):
    bonds = lattice.chain_bonds(n) + [(i, (i + 3) % n) for i in range(n)]
    rng = np.random.default_rng(n)
    jxy, jz = 0.5 + rng.random(len(bonds)), rng.random(len(bonds))
    terms = O.heisenberg_terms(n, bonds, jxy, jz)
    cls = classes_of(n, terms)
    check_classes(n, cls)
    sites = O.spin_half_sites(n)
    basis = O.hs_get_basis_list(sites, [(sector,)])
    x = O.complex_gaussian(len(basis), 3)
    y = walk(n, cls, basis, [t for t in terms if t[1] == t[2]], x)
    want = O.apply_rows(basis, terms, x)
    assert np.linalg.norm(y - want) <= 1e-12 * np.linalg.norm(want)


def test_walk_matches_oracle_complex_and_pair_terms():
    n = 8
    _, offs = O.bit_layout(O.spin_half_sites(n))
    op = []
    for i in range(n):
        j = (i + 1) % n
        op += O.op_scale(0.6 + 0.35j, O.op_mul(O.pauli_matrix(offs, i, "+"), O.pauli_matrix(offs, j, "-")))
        op += O.op_scale(0.6 - 0.35j, O.op_mul(O.pauli_matrix(offs, i, "-"), O.pauli_matrix(offs, j, "+")))
        op += O.op_scale(0.25, O.op_mul(O.pauli_matrix(offs, i, "+"), O.pauli_matrix(offs, j, "+")))
        op += O.op_scale(0.25, O.op_mul(O.pauli_matrix(offs, i, "-"), O.pauli_matrix(offs, j, "-")))
        op += O.op_scale(0.3, O.op_mul(O.pauli_matrix(offs, i, "z"), O.pauli_matrix(offs, j, "z")))
    op = O.simplify(op)
    cls = classes_of(n, op)
    assert len(cls) == 1 and cls[0]["par"]
    basis = O.hs_get_basis_list(O.spin_half_sites(n))
    x = O.complex_gaussian(len(basis), 5)
    y = walk(n, cls, basis, [t for t in op if t[1] == t[2]], x)
    want = O.apply_rows(basis, op, x)
    assert np.linalg.norm(y - want) <= 1e-12 * np.linalg.norm(want)


def test_terms_outside_the_schedule():
    n = 6
    _, offs = O.bit_layout(O.spin_half_sites(n))
    field = O.pauli_matrix(offs, 0, "x")                          # one-site flip
    assert classes_of(n, O.heisenberg_terms(n, lattice.chain_bonds(n), [1.0] * n, [1.0] * n) + field) == []
    half = O.op_mul(O.pauli_matrix(offs, 0, "+"), O.pauli_matrix(offs, 1, "-"))   # no Hermitian partner
    assert classes_of(n, half) == []


def test_argument_errors():
    L = _lib.lib()
    nc = ctypes.c_int32()
    z = np.zeros(1, np.uint64)
    a = np.zeros(2, np.float64)
    for n_bits in (0, 65):
        assert L.edgpu_pair_classes_of_terms(n_bits, 0, None, None, None, None, 0, ctypes.byref(nc),
                                             None, None, None, None) == _lib.ERR_ARG
    assert L.edgpu_pair_classes_of_terms(8, 1, None, None, None, None, 0, ctypes.byref(nc),
                                         None, None, None, None) == _lib.ERR_ARG
    assert L.edgpu_pair_classes_of_terms(8, 1, ptr(z, ctypes.c_uint64), ptr(z, ctypes.c_uint64),
                                         ptr(z, ctypes.c_uint64), ptr(a, ctypes.c_double), 0, None,
                                         None, None, None, None) == _lib.ERR_ARG
    # no terms at all: no classes
    assert L.edgpu_pair_classes_of_terms(8, 0, None, None, None, None, 0, ctypes.byref(nc),
                                         None, None, None, None) == 0
    assert nc.value == 0
