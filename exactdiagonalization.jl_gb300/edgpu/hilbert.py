"""Hilbert-space layer: State, Site, HilbertSpace, HilbertSpaceSector.

Mirrors src/HilbertSpace/{site,hilbert_space,hilbert_space_sector}.jl of ExactDiagonalization.jl.
Python indices are 0-based: site i, local state s (stored as code s in the basis word); the
reference's 1-based (isite, state index) become (i - 1, s - 1).
"""
from __future__ import annotations

import math
from typing import Iterable, List, Sequence, Tuple


def _as_qn(q) -> Tuple[int, ...]:
    if isinstance(q, tuple):
        return tuple(int(v) for v in q)
    if isinstance(q, (list,)):
        return tuple(int(v) for v in q)
    return (int(q),)


class State:
    """State(name, quantum_number) -- site.jl:29-41.  An integer quantum number becomes a 1-tuple."""

    def __init__(self, name: str, quantum_number=()):
        self.name = name
        self.quantum_number = _as_qn(quantum_number)

    def __eq__(self, other):
        return isinstance(other, State) and self.name == other.name and self.quantum_number == other.quantum_number

    def __hash__(self):
        return hash((self.name, self.quantum_number))

    def __repr__(self):
        return f"State({self.name!r}, {self.quantum_number})"


class Site:
    """Site(states) -- site.jl:69-72."""

    def __init__(self, states: Sequence[State]):
        self.states = list(states)
        if not self.states:
            raise ValueError("a site needs at least one state")
        qlens = {len(s.quantum_number) for s in self.states}
        if len(qlens) != 1:
            raise ValueError("all states of a site must have quantum numbers of the same length")

    def __eq__(self, other):
        return isinstance(other, Site) and self.states == other.states

    def __hash__(self):
        return hash(tuple(self.states))

    @property
    def dimension(self) -> int:
        return len(self.states)

    @property
    def qlen(self) -> int:
        return len(self.states[0].quantum_number)


def bitwidth(x) -> int:
    """bitwidth(site) = ceil(log2(#states)) (site.jl:93); bitwidth(hs) = total bits (hilbert_space.jl:96)."""
    if isinstance(x, Site):
        return int(math.ceil(math.log2(x.dimension))) if x.dimension > 1 else 0
    return basespace(x).bitoffsets[-1]


def dimension(x) -> int:
    if isinstance(x, Site):
        return x.dimension
    return x.dimension


class HilbertSpace:
    """HilbertSpace(sites) with bitwidths and bitoffsets = [0, cumsum(bitwidths)...] -- hilbert_space.jl:25-41."""

    def __init__(self, sites: Sequence[Site]):
        self.sites = list(sites)
        self.bitwidths = [bitwidth(s) for s in self.sites]
        self.bitoffsets = [0]
        for w in self.bitwidths:
            self.bitoffsets.append(self.bitoffsets[-1] + w)

    def __eq__(self, other):
        return isinstance(other, HilbertSpace) and self.sites == other.sites

    def __hash__(self):
        return hash(tuple(self.sites))

    @property
    def n_sites(self) -> int:
        return len(self.sites)

    @property
    def qlen(self) -> int:
        return self.sites[0].qlen if self.sites else 0

    def get_bitmask(self, isite: int | None = None) -> int:
        """get_bitmask(hs, isite) / get_bitmask(hs) -- hilbert_space.jl:107-113 (0-based isite)."""
        if isite is None:
            return (1 << self.bitoffsets[-1]) - 1
        return ((1 << self.bitoffsets[isite + 1]) - 1) ^ ((1 << self.bitoffsets[isite]) - 1)

    def quantum_number_sectors(self) -> List[Tuple[int, ...]]:
        """hilbert_space.jl:119-129."""
        qns = {tuple([0] * self.qlen)}
        for site in self.sites:
            qns = {tuple(a + b for a, b in zip(q, s.quantum_number)) for s in site.states for q in qns}
        return sorted(qns)

    def get_quantum_number(self, bitrep: int) -> Tuple[int, ...]:
        """hilbert_space.jl:135-143."""
        acc = [0] * self.qlen
        for i, site in enumerate(self.sites):
            code = (bitrep >> self.bitoffsets[i]) & ((1 << self.bitwidths[i]) - 1)
            for k, v in enumerate(site.states[code].quantum_number):
                acc[k] += v
        return tuple(acc)

    def compress(self, indices: Sequence[int]) -> int:
        """compress(hs, CartesianIndex) with 0-based local indices -- hilbert_space.jl:199-215."""
        if len(indices) != self.n_sites:
            raise ValueError("length of indexarray should be the number of sites")
        out = 0
        for i, s in enumerate(indices):
            if not (0 <= s < self.sites[i].dimension):
                raise IndexError(f"local state {s} out of range for site {i}")
            out |= int(s) << self.bitoffsets[i]
        return out

    def extract(self, bitrep: int) -> Tuple[int, ...]:
        """extract(hs, binrep) with 0-based local indices -- hilbert_space.jl:172-184."""
        out = []
        for i, site in enumerate(self.sites):
            code = (bitrep >> self.bitoffsets[i]) & ((1 << self.bitwidths[i]) - 1)
            if code >= site.dimension:
                raise IndexError(f"code {code} invalid for site {i}")
            out.append(code)
        return tuple(out)


class HilbertSpaceSector:
    """HilbertSpaceSector(parent, allowed) -- hilbert_space_sector.jl:20-63.

    allowed: None (all sectors), an int (the tuple (int,)), a QN tuple, or a collection of either.
    The allowed set is intersected with the parent's reachable sectors, as in the reference."""

    def __init__(self, parent: HilbertSpace, allowed=None):
        self.parent = parent
        sectors = set(parent.quantum_number_sectors())
        if allowed is None:
            allowed_set = sectors
        elif isinstance(allowed, (int, tuple)):
            allowed_set = {_as_qn(allowed)}
        else:
            allowed_set = {_as_qn(a) for a in allowed}
        self.allowed_quantum_numbers = allowed_set & sectors

    def __eq__(self, other):
        return (isinstance(other, HilbertSpaceSector) and self.parent == other.parent
                and self.allowed_quantum_numbers == other.allowed_quantum_numbers)

    def __hash__(self):
        return hash((self.parent, frozenset(self.allowed_quantum_numbers)))

    def quantum_number_sectors(self):
        return self.parent.quantum_number_sectors()

    def get_bitmask(self, isite=None):
        return self.parent.get_bitmask(isite)

    @property
    def sites(self):
        return self.parent.sites

    @property
    def bitwidths(self):
        return self.parent.bitwidths

    @property
    def bitoffsets(self):
        return self.parent.bitoffsets


def basespace(x) -> HilbertSpace:
    """basespace(hs) / basespace(hss) -- hilbert_space.jl:78, hilbert_space_sector.jl:104."""
    if isinstance(x, HilbertSpace):
        return x
    if isinstance(x, HilbertSpaceSector):
        return basespace(x.parent)
    return basespace(x.hilbert_space)


def quantum_number_sectors(x) -> List[Tuple[int, ...]]:
    return basespace(x).quantum_number_sectors()
