"""Operator layer: NullOperator, PureOperator, SumOperator, simplify, pauli_matrix, spin_half_system.

Mirrors src/Operator/*.jl and src/Toolkit/spin_half.jl of ExactDiagonalization.jl.  These host-side
objects only build the term table (bitmask, bitrow, bitcol, amplitude) that the GPU product consumes.
Site and local-state indices are 0-based.
"""
from __future__ import annotations

import math
from typing import List, Sequence

import numpy as np

from ._lib import ArgumentError
from .hilbert import HilbertSpace, Site, State, basespace

RTOL = math.sqrt(np.finfo(np.float64).eps)   # Base.rtoldefault(Float64)


class AbstractOperator:
    def __add__(self, other):
        return SumOperator(_terms(self) + _terms(other))

    def __radd__(self, other):
        if isinstance(other, (int, float, complex)) and other == 0:
            return self
        return NotImplemented

    def __sub__(self, other):
        return self + (-1) * other

    def __neg__(self):
        return (-1) * self

    def __rmul__(self, c):
        if isinstance(c, (int, float, complex, np.number)):
            return _scale(self, complex(c))
        return NotImplemented

    def __mul__(self, other):
        if isinstance(other, (int, float, complex, np.number)):
            return _scale(self, complex(other))
        return _product(self, other)

    def __truediv__(self, c):
        return _scale(self, 1.0 / complex(c))


class NullOperator(AbstractOperator):
    """null_operator.jl:9-47."""

    def __eq__(self, other):
        return isinstance(other, NullOperator)

    def __hash__(self):
        return 0

    @property
    def terms(self):
        return []

    def __repr__(self):
        return "NullOperator()"


class PureOperator(AbstractOperator):
    """alpha * prod_i (identity or |r_i><c_i|) -- pure_operator.jl:25-52."""

    def __init__(self, bitmask: int, bitrow: int, bitcol: int, amplitude):
        bitmask, bitrow, bitcol = int(bitmask), int(bitrow), int(bitcol)
        if (~bitmask) & bitrow:
            raise ArgumentError("every bit of bitrow not in bitmask should be set to zero")
        if (~bitmask) & bitcol:
            raise ArgumentError("every bit of bitcol not in bitmask should be set to zero")
        self.bitmask, self.bitrow, self.bitcol = bitmask, bitrow, bitcol
        self.amplitude = complex(amplitude)

    def key(self):
        return (self.bitmask, self.bitrow, self.bitcol, self.amplitude.real, self.amplitude.imag)

    def __eq__(self, other):
        return isinstance(other, PureOperator) and self.key() == other.key()

    def __hash__(self):
        return hash(self.key())

    def __lt__(self, other):   # isless, pure_operator.jl:78-90
        return self.key() < other.key()

    @property
    def terms(self):
        return [self]

    def adjoint(self):
        return PureOperator(self.bitmask, self.bitcol, self.bitrow, self.amplitude.conjugate())

    def transpose(self):
        return PureOperator(self.bitmask, self.bitcol, self.bitrow, self.amplitude)

    def __repr__(self):
        return f"PureOperator({self.bitmask:#b}, {self.bitrow:#b}, {self.bitcol:#b}, {self.amplitude})"


class SumOperator(AbstractOperator):
    """Sum of pure operators -- sum_operator.jl:13-23."""

    def __init__(self, terms: Sequence[PureOperator]):
        self.terms: List[PureOperator] = list(terms)

    def __eq__(self, other):
        return isinstance(other, SumOperator) and self.terms == other.terms

    def __hash__(self):
        return hash(tuple(self.terms))

    def adjoint(self):
        return SumOperator([t.adjoint() for t in self.terms])

    def transpose(self):
        return SumOperator([t.transpose() for t in self.terms])

    def __repr__(self):
        return f"SumOperator({len(self.terms)} terms)"


def _terms(op) -> List[PureOperator]:
    if isinstance(op, (int, float, complex)) and op == 0:
        return []
    return list(op.terms)


def _scale(op, c):
    if isinstance(op, NullOperator):
        return op
    if isinstance(op, PureOperator):
        return PureOperator(op.bitmask, op.bitrow, op.bitcol, c * op.amplitude)
    return SumOperator([_scale(t, c) for t in op.terms])


def _pure_product(l: PureOperator, r: PureOperator):
    """pure_operator.jl:136-154."""
    inter = l.bitmask & r.bitmask
    if (l.bitcol & inter) != (r.bitrow & inter):
        return None
    only_l = l.bitmask & ~r.bitmask
    only_r = ~l.bitmask & r.bitmask
    return PureOperator(l.bitmask | r.bitmask, l.bitrow | (r.bitrow & only_r), r.bitcol | (l.bitcol & only_l),
                        l.amplitude * r.amplitude)


def _product(lhs, rhs):
    """Products of pure/sum operators (sum_operator.jl:59-76); NullOperator terms are dropped."""
    if isinstance(lhs, NullOperator) or isinstance(rhs, NullOperator):
        return NullOperator()
    if isinstance(lhs, PureOperator) and isinstance(rhs, PureOperator):
        p = _pure_product(lhs, rhs)
        return NullOperator() if p is None else p
    out = []
    for a in _terms(lhs):
        for b in _terms(rhs):
            p = _pure_product(a, b)
            if p is not None:
                out.append(p)
    return SumOperator(out)


def simplify(op, tol: float = RTOL):
    """simplify -- operator_simplify.jl:9-81: drop ~0 terms, sort by (mask, row, col, re, im), merge
    equal projectors, drop merged ~0 terms; one term becomes a PureOperator, none a NullOperator."""
    if isinstance(op, NullOperator):
        return op
    if isinstance(op, PureOperator):
        return NullOperator() if abs(op.amplitude) <= tol else op
    terms = [t for t in op.terms if not (abs(t.amplitude) <= tol)]
    if not terms:
        return NullOperator()
    terms.sort(key=PureOperator.key)
    out = []
    bm, br, bc, am = terms[0].bitmask, terms[0].bitrow, terms[0].bitcol, terms[0].amplitude
    for t in terms[1:]:
        if (t.bitmask, t.bitrow, t.bitcol) == (bm, br, bc):
            am += t.amplitude
        else:
            if not (abs(am) <= tol):
                out.append(PureOperator(bm, br, bc, am))
            bm, br, bc, am = t.bitmask, t.bitrow, t.bitcol, t.amplitude
    if not (abs(am) <= tol):
        out.append(PureOperator(bm, br, bc, am))
    if not out:
        return NullOperator()
    if len(out) == 1:
        return out[0]
    return SumOperator(out)


def pure_operator(hs, isite: int, istate_row: int, istate_col: int, amplitude=1):
    """pure_operator(hs, isite, row, col, amp) -- pure_operator.jl:184-201 (all indices 0-based)."""
    hs = basespace(hs)
    site = hs.sites[isite]
    if not (0 <= istate_row < site.dimension and 0 <= istate_col < site.dimension):
        raise IndexError("local state index out of range")
    bm = hs.get_bitmask(isite)
    return PureOperator(bm, istate_row << hs.bitoffsets[isite], istate_col << hs.bitoffsets[isite], amplitude)


def pauli_matrix(hs, isite: int, j: str):
    """pauli_matrix(hs, isite, :x|:y|:z|:+|:-) -- spin_half.jl:28-42 (0-based isite; state 0 = Up)."""
    P = lambda r, c, a: pure_operator(hs, isite, r, c, a)
    if j == "x":
        return P(0, 1, 1) + P(1, 0, 1)
    if j == "y":
        return P(0, 1, -1j) + P(1, 0, 1j)
    if j == "z":
        return P(0, 0, 1) + P(1, 1, -1)
    if j == "+":
        return P(0, 1, 1)
    if j == "-":
        return P(1, 0, 1)
    raise ArgumentError(f"pauli matrix of type {j} not supported")


def spin_half_system(n_sites: int, nbits_type: int = 64):
    """spin_half_system(n) -- spin_half.jl:9-19: returns (hilbert_space, pauli) with pauli(i, j)."""
    if n_sites > nbits_type:
        raise ArgumentError(f"spin half system of {n_sites} sites cannot be expressed using UInt{nbits_type}")
    site = Site([State("Up", 1), State("Dn", -1)])
    hs = HilbertSpace([site for _ in range(n_sites)])
    return hs, (lambda i, j: pauli_matrix(hs, i, j))


def term_arrays(op):
    """(masks, rows, cols, amps) numpy arrays of an operator's terms, in term order."""
    terms = _terms(op) if not isinstance(op, NullOperator) else []
    masks = np.array([t.bitmask for t in terms], dtype=np.uint64)
    rows = np.array([t.bitrow for t in terms], dtype=np.uint64)
    cols = np.array([t.bitcol for t in terms], dtype=np.uint64)
    amps = np.array([t.amplitude for t in terms], dtype=np.complex128)
    return masks, rows, cols, amps
