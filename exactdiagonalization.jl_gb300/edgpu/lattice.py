"""Lattice bond lists and spin-1/2 Hamiltonians built through the reference API
(pauli_matrix products + simplify), as used by the benchmark configurations.

Site (x, y) of an L1 x L2 torus has index x + L1*y (0-based), as in
examples/spinhalfsquare_large.jl:35 (1 + x + L1*y, 1-based).
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np

from .operators import NullOperator, SumOperator, pauli_matrix, simplify


def chain_bonds(L: int) -> List[Tuple[int, int]]:
    """Nearest-neighbour bonds (i, i+1 mod L) of a periodic chain."""
    return [(i, (i + 1) % L) for i in range(L)]


def torus_bonds(L1: int, L2: int, vectors: Sequence[Tuple[int, int]]) -> List[Tuple[int, int]]:
    """Bonds (x, y) -- (x + dx, y + dy) for every site and every displacement vector (periodic)."""
    out = []
    for dx, dy in vectors:
        for y in range(L2):
            for x in range(L1):
                out.append((x + L1 * y, (x + dx) % L1 + L1 * ((y + dy) % L2)))
    return out


TRIANGULAR_NN = [(1, 0), (1, 1), (0, 1)]          # examples/spinhalf_triangular.jl:20
TRIANGULAR_NNN = [(2, 1), (1, 2), (-1, 1)]        # examples/spinhalf_triangular.jl:21
SQUARE_NN = [(1, 0), (0, 1)]
SQUARE_NNN = [(1, 1), (1, -1)]


def xxz_hamiltonian(hs, bonds, jxy, jz, coupling_of_bond=None):
    """H = sum_b (Jxy_b/4 (sx sx + sy sy) + Jz_b/4 sz sz) with sigma = pauli_matrix, then simplify
    (6 terms per bond).  jxy/jz: scalars or per-bond sequences.

    With coupling_of_bond (bond -> coupling index) also returns the per-term coupling ids and the
    per-unit amplitudes for gradients: (H, ids, unit_terms) where unit_terms is H with every bond's
    couplings set to 1 and ids[t] the coupling of term t."""
    nb = len(bonds)
    jxy = np.broadcast_to(np.asarray(jxy, dtype=np.float64), (nb,))
    jz = np.broadcast_to(np.asarray(jz, dtype=np.float64), (nb,))
    op = NullOperator()
    for (i, j), a, b in zip(bonds, jxy, jz):
        bond = (a / 4.0) * (pauli_matrix(hs, i, "x") * pauli_matrix(hs, j, "x") +
                            pauli_matrix(hs, i, "y") * pauli_matrix(hs, j, "y")) + \
               (b / 4.0) * (pauli_matrix(hs, i, "z") * pauli_matrix(hs, j, "z"))
        op = op + bond
    return simplify(op)


def heisenberg_coupled(hs, bonds):
    """Per-bond Heisenberg terms with unit coupling: (masks, rows, cols, amps, coupling_ids) for
    H(J) = sum_b J_b S_b.S_b' (S = sigma/2), one coupling per bond."""
    masks, rows, cols, amps, ids = [], [], [], [], []
    for c, (i, j) in enumerate(bonds):
        t = simplify(0.25 * (pauli_matrix(hs, i, "x") * pauli_matrix(hs, j, "x") +
                             pauli_matrix(hs, i, "y") * pauli_matrix(hs, j, "y") +
                             pauli_matrix(hs, i, "z") * pauli_matrix(hs, j, "z")))
        for p in t.terms:
            masks.append(p.bitmask)
            rows.append(p.bitrow)
            cols.append(p.bitcol)
            amps.append(p.amplitude)
            ids.append(c)
    return (np.array(masks, dtype=np.uint64), np.array(rows, dtype=np.uint64), np.array(cols, dtype=np.uint64),
            np.array(amps, dtype=np.complex128), np.array(ids, dtype=np.int32))


# C4v about site (0, 0) of an L x L torus: (class, (x, y) -> (x', y')); the characters of its four
# one-dimensional irreps by class
C4V_ELEMENTS = [
    ("E", lambda x, y: (x, y)),
    ("C4", lambda x, y: (-y, x)),
    ("C2", lambda x, y: (-x, -y)),
    ("C4", lambda x, y: (y, -x)),
    ("sv", lambda x, y: (-x, y)),
    ("sv", lambda x, y: (x, -y)),
    ("sd", lambda x, y: (y, x)),
    ("sd", lambda x, y: (-y, -x)),
]
C4V_CHARACTERS = {
    "A1": {"E": 1, "C2": 1, "C4": 1, "sv": 1, "sd": 1},
    "A2": {"E": 1, "C2": 1, "C4": 1, "sv": -1, "sd": -1},
    "B1": {"E": 1, "C2": 1, "C4": -1, "sv": 1, "sd": -1},
    "B2": {"E": 1, "C2": 1, "C4": -1, "sv": -1, "sd": 1},
}


def square_c4v_maps(L: int, momentum=(0, 0), irrep: str = "A1"):
    """Site maps and amplitudes of the symmorphic space group T x C4v of an L x L square torus (the
    translations times the point group about site 0, examples/spinhalfsquare_large.jl's
    tsymbed x psymbed), element t o p with amplitude exp(-2 pi i k.t / L) chi(p), identity first.
    k must be invariant under C4v (k = (0, 0) or (L/2, L/2)); irrep is one of A1, A2, B1, B2.
    Returns (maps [L^4 * 2][L^2] int32, amplitudes complex)."""
    k1, k2 = momentum
    for _, f in C4V_ELEMENTS:
        a, b = f(k1, k2)
        if (a - k1) % L or (b - k2) % L:
            raise ValueError(f"momentum {momentum} is not invariant under C4v")
    chi = C4V_CHARACTERS[irrep]
    n = L * L
    maps, amps = [], []
    for ty in range(L):
        for tx in range(L):
            ph = np.exp(-2j * np.pi * (k1 * tx + k2 * ty) / L)
            for cls, f in C4V_ELEMENTS:
                m = []
                for s in range(n):
                    x, y = s % L, s // L
                    px, py = f(x, y)
                    m.append((px + tx) % L + L * ((py + ty) % L))
                maps.append(m)
                amps.append(ph * chi[cls])
    return np.array(maps, dtype=np.int32), np.array(amps)


def square_c4v_symops(L: int, momentum=(0, 0), irrep: str = "A1"):
    """square_c4v_maps as [(SitePermutation, amplitude)] for symmetry_reduce."""
    from .representation import SitePermutation
    maps, amps = square_c4v_maps(L, momentum, irrep)
    return [(SitePermutation(m), complex(a)) for m, a in zip(maps, amps)]
