"""oracle -- CPU restatement of ExactDiagonalization.jl's Hamiltonian-application path.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg may import this module, and only as the checker / the CPU baseline.
The product library (libedgpu.so and the `edgpu` package) never imports it.

It restates, function by function, the reference (kyungminlee/ExactDiagonalization.jl
v0.14.3) with its own data structures: the QN dynamic programme for the sector basis,
FrozenSortedArrayIndex lookups, the operator algebra that builds the term table
(pure_operator * pure_operator, simplify), the visited-flag orbit sweep of
symmetry_reduce with parent-sized mapping tables, and the row/column iterators of
(Reduced)OperatorRepresentation.  The heavy loops live in ed_oracle.c (ctypes).

Parity is pinned against the golden vectors of the reference's own tests
(tests/golden/reference_tests.json, transcribed from test/*.jl); see
tests/test_oracle_golden.py.
"""
from __future__ import annotations

import ctypes
import math
import os
from typing import Dict, List, Sequence, Tuple

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        i64p = ctypes.POINTER(ctypes.c_int64)
        i32p = ctypes.POINTER(ctypes.c_int32)
        dp = ctypes.POINTER(ctypes.c_double)
        L.or_lookup.restype = ctypes.c_int64
        L.or_lookup.argtypes = [u64p, ctypes.c_int64, ctypes.c_uint64]
        L.or_lookup_many.restype = None
        L.or_lookup_many.argtypes = [u64p, ctypes.c_int64, u64p, ctypes.c_int64, i64p]
        L.or_symmetry_apply.restype = ctypes.c_uint64
        L.or_symmetry_apply.argtypes = [ctypes.c_int, i32p, i32p, i32p, ctypes.c_uint64, ctypes.c_uint64]
        L.or_symmetry_reduce.restype = ctypes.c_int64
        L.or_symmetry_reduce.argtypes = [u64p, ctypes.c_int64, ctypes.c_int, i32p, i32p, ctypes.c_int, i32p,
                                         u64p, dp, ctypes.c_double, u64p, i64p, dp]
        for name in ("or_apply_rows", "or_apply_cols"):
            f = getattr(L, name)
            f.restype = None
            f.argtypes = [u64p, ctypes.c_int64, u64p, ctypes.c_int64, i64p, dp, ctypes.c_int, u64p, u64p, u64p,
                          dp, dp, dp, ctypes.c_int, ctypes.c_int]
        L.or_apply_rows_range.restype = None
        L.or_apply_rows_range.argtypes = [u64p, ctypes.c_int64, u64p, ctypes.c_int64, i64p, dp, ctypes.c_int, u64p,
                                          u64p, u64p, dp, dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                                          ctypes.c_int64, i64p]
        L.or_unreduce.restype = None
        L.or_unreduce.argtypes = [i64p, dp, ctypes.c_int64, dp, dp]
        L.or_reduce_vector.restype = None
        L.or_reduce_vector.argtypes = [i64p, dp, ctypes.c_int64, dp, dp, ctypes.c_int64]
        L.or_popcount_basis.restype = ctypes.c_int64
        L.or_popcount_basis.argtypes = [ctypes.c_int, ctypes.c_int, u64p, ctypes.c_int64]
        L.or_num_threads.restype = ctypes.c_int
        L.or_num_threads.argtypes = []
        L.or_orbit_info.restype = None
        L.or_orbit_info.argtypes = [ctypes.c_int, i32p, i32p, ctypes.c_int, i32p, u64p, dp, ctypes.c_double, u64p,
                                    ctypes.c_int64, u64p, i32p, i32p, dp]
        L.or_sampled_rows_torus.restype = None
        L.or_sampled_rows_torus.argtypes = [ctypes.c_int, ctypes.c_int, u64p, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                            i32p, i32p, ctypes.c_int, i32p, dp, ctypes.c_double, ctypes.c_int, u64p,
                                            u64p, u64p, dp, dp, i64p, ctypes.c_int64, dp, i32p, i64p]
        L.or_torus_reps.restype = ctypes.c_int64
        L.or_torus_reps.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, i32p, ctypes.c_int, ctypes.c_int, u64p]
        L.or_sampled_rows.restype = None
        L.or_sampled_rows.argtypes = [u64p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, i32p, i32p, ctypes.c_int, i32p,
                                      u64p, dp, ctypes.c_double, ctypes.c_int, u64p, u64p, u64p, dp, dp, i64p,
                                      ctypes.c_int64, dp, i32p, i64p]
        _lib = L
    return _lib


def _p(a, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def num_threads() -> int:
    return int(lib().or_num_threads())


# ---------------------------------------------------------------------------------------------
# Hilbert space layout and sector basis
# ---------------------------------------------------------------------------------------------

def bitwidth_of(n_states: int) -> int:
    """bitwidth(site) = Int(ceil(log2(#states))) -- site.jl:93."""
    return int(math.ceil(math.log2(n_states))) if n_states > 1 else 0


def bit_layout(site_qns: Sequence[Sequence[Tuple[int, ...]]]):
    """bitwidths and bitoffsets = [0, cumsum(bitwidths)...] -- hilbert_space.jl:25-41."""
    bw = [bitwidth_of(len(s)) for s in site_qns]
    off = [0]
    for w in bw:
        off.append(off[-1] + w)
    return bw, off


def _tadd(a, b):
    return tuple(x + y for x, y in zip(a, b))


def _tsub(a, b):
    return tuple(x - y for x, y in zip(a, b))


def quantum_number_sectors(site_qns) -> List[Tuple[int, ...]]:
    """hilbert_space.jl:119-129."""
    qlen = len(site_qns[0][0])
    qns = {tuple([0] * qlen)}
    for site in site_qns:
        qns = {_tadd(q, s) for s in site for q in qns}
    return sorted(qns)


class ArgumentError(ValueError):
    pass


def hs_get_basis_list(site_qns, allowed=None, nbits_type: int = 64) -> np.ndarray:
    """Sector basis, ascending uint64.

    allowed=None is hs_get_basis_list(::HilbertSpace) (hilbert_space_representation.jl:109-119);
    otherwise the QN dynamic programme of hs_get_basis_list(::HilbertSpaceSector) (:127-206):
    forward-possible and backward-requested QN sets, site-by-site appends
    s | (code << bitoffset[i]), and a final merge of the per-QN lists.
    """
    bw, off = bit_layout(site_qns)
    if nbits_type <= off[-1]:
        raise ArgumentError(f"type too small to represent the hilbert space (need {off[-1]} bits)")
    n = len(site_qns)
    qlen = len(site_qns[0][0])
    zero = tuple([0] * qlen)
    if allowed is None:
        allowed = quantum_number_sectors(site_qns)
    allowed = set(tuple(a) for a in allowed)
    if not (allowed & set(quantum_number_sectors(site_qns))):
        return np.zeros(0, dtype=np.uint64)
    possible = [[zero]]
    for i in range(n):
        possible.append(sorted({_tadd(qa, qi) for qi in site_qns[i] for qa in possible[i]}))
    requested = [None] * (n + 1)
    requested[n] = sorted(allowed)
    for i in range(n - 1, -1, -1):
        requested[i] = sorted({_tsub(qa, qi) for qi in site_qns[i] for qa in requested[i + 1]})
    schedule = [sorted(set(r) & set(p)) for r, p in zip(requested, possible)]
    cur: Dict[tuple, np.ndarray] = {zero: np.zeros(1, dtype=np.uint64)}
    for i in range(n):
        new: Dict[tuple, np.ndarray] = {}
        for q in schedule[i + 1]:
            parts = []
            for i_state, q_curr in enumerate(site_qns[i]):
                q_prev = _tsub(q, q_curr)
                if q_prev in cur:
                    parts.append(cur[q_prev] | np.uint64(i_state << off[i]))
            new[q] = np.concatenate(parts) if parts else np.zeros(0, dtype=np.uint64)
        cur = new
    out = np.concatenate(list(cur.values())) if cur else np.zeros(0, dtype=np.uint64)
    out = np.sort(out, kind="stable")        # merge_vec of disjoint sorted lists (util.jl:62-86)
    return out


def spin_half_sites(n: int):
    """spin_half_system(n): Site([Up(+1), Dn(-1)]) on every site -- spin_half.jl:9-19."""
    return [[(1,), (-1,)] for _ in range(n)]


def popcount_basis(n: int, k: int) -> np.ndarray:
    """All n-bit words with k set bits, ascending (the 2Sz = n-2k sector of spin_half_system(n))."""
    cnt = math.comb(n, k)
    out = np.empty(cnt, dtype=np.uint64)
    got = lib().or_popcount_basis(n, k, _p(out, ctypes.c_uint64), cnt)
    assert got == cnt
    return out


def check_frozen_sorted(keys: np.ndarray):
    """FrozenSortedArrayIndex constructor checks -- frozensortedarray.jl:14-22."""
    keys = np.asarray(keys)
    if keys.size > 1:
        if np.any(keys[1:] < keys[:-1]):
            raise ArgumentError("vals must be sorted")
        if np.any(keys[1:] == keys[:-1]):
            raise ArgumentError("vals contains duplicates")


def lookup(keys: np.ndarray, q: np.ndarray) -> np.ndarray:
    """get(FrozenSortedArrayIndex, key, -1) for many keys (0-based) -- frozensortedarray.jl:29-48."""
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    q = np.ascontiguousarray(q, dtype=np.uint64)
    out = np.empty(q.size, dtype=np.int64)
    lib().or_lookup_many(_p(keys, ctypes.c_uint64), keys.size, _p(q, ctypes.c_uint64), q.size,
                         _p(out, ctypes.c_int64))
    return out


# ---------------------------------------------------------------------------------------------
# Operator algebra -> term table (mask, row, col, amplitude)
# ---------------------------------------------------------------------------------------------

RTOL = math.sqrt(np.finfo(np.float64).eps)   # Base.rtoldefault(Float64)


def pure_operator(off, isite, istate_row, istate_col, amp):
    """pure_operator(hs, isite, row, col, amp) with 0-based isite and 1-based state indices
    -- pure_operator.jl:184-201."""
    mask = ((1 << off[isite + 1]) - 1) ^ ((1 << off[isite]) - 1)
    return [(mask, (istate_row - 1) << off[isite], (istate_col - 1) << off[isite], complex(amp))]


def op_mul(lhs, rhs):
    """Product of sums of pure operators -- pure_operator.jl:136-154, sum_operator.jl:72-76."""
    out = []
    for (lm, lr, lc, la) in lhs:
        for (rm, rr, rc, ra) in rhs:
            inter = lm & rm
            if (lc & inter) != (rr & inter):
                continue
            only_l = lm & ~rm
            only_r = ~lm & rm
            out.append((lm | rm, lr | (rr & only_r), rc | (lc & only_l), la * ra))
    return out


def op_scale(c, op):
    return [(m, r, cc, c * a) for (m, r, cc, a) in op]


def pauli_matrix(off, isite, j):
    """pauli_matrix -- spin_half.jl:28-42 (0-based isite)."""
    P = lambda r, c, a: pure_operator(off, isite, r, c, a)
    if j == "x":
        return P(1, 2, 1) + P(2, 1, 1)
    if j == "y":
        return P(1, 2, -1j) + P(2, 1, 1j)
    if j == "z":
        return P(1, 1, 1) + P(2, 2, -1)
    if j == "+":
        return P(1, 2, 1)
    if j == "-":
        return P(2, 1, 1)
    raise ArgumentError(f"pauli matrix of type {j} not supported")


def simplify(op, tol: float = RTOL):
    """simplify(::SumOperator) -- operator_simplify.jl:32-81: drop ~0 terms, sort by
    (mask,row,col,re,im), merge equal projectors, drop merged ~0 terms."""
    terms = [t for t in op if not (abs(t[3]) <= tol)]
    if not terms:
        return []
    terms.sort(key=lambda t: (t[0], t[1], t[2], t[3].real, t[3].imag))
    out = []
    bm, br, bc, am = terms[0]
    for (m, r, c, a) in terms[1:]:
        if m == bm and r == br and c == bc:
            am += a
        else:
            if not (abs(am) <= tol):
                out.append((bm, br, bc, am))
            bm, br, bc, am = m, r, c, a
    if not (abs(am) <= tol):
        out.append((bm, br, bc, am))
    return out


def heisenberg_terms(n_sites, bonds, jxy, jz):
    """H = sum_b (Jxy_b/4 (sx sx + sy sy) + Jz_b/4 sz sz), built with pauli_matrix and simplify
    (bonds are 0-based site pairs; jxy, jz per bond)."""
    _, off = bit_layout(spin_half_sites(n_sites))
    op = []
    for (i, j), a, b in zip(bonds, jxy, jz):
        op += op_scale(a / 4.0, op_mul(pauli_matrix(off, i, "x"), pauli_matrix(off, j, "x")))
        op += op_scale(a / 4.0, op_mul(pauli_matrix(off, i, "y"), pauli_matrix(off, j, "y")))
        op += op_scale(b / 4.0, op_mul(pauli_matrix(off, i, "z"), pauli_matrix(off, j, "z")))
    return simplify(op)


def term_arrays(terms):
    masks = np.array([t[0] for t in terms], dtype=np.uint64)
    rows = np.array([t[1] for t in terms], dtype=np.uint64)
    cols = np.array([t[2] for t in terms], dtype=np.uint64)
    amps = np.array([t[3] for t in terms], dtype=np.complex128)
    return masks, rows, cols, amps


# ---------------------------------------------------------------------------------------------
# Symmetry
# ---------------------------------------------------------------------------------------------

def translation_symops(shape, momentum):
    """Translation group of an L1 x L2 torus (site (x, y) -> index x + L1*y, 0-based) with
    amplitudes chi(T(a,b)) = exp(-2 pi i (m1 a / L1 + m2 b / L2)), element g = a + L1*b,
    g = 0 the identity.  This is the convention the reference's tests pin for LatticeTools'
    IrrepComponent: symmetry_unreduce of the L=7 one-particle state at momentum index 2 gives
    cis(+2 pi i x / 7)/sqrt(7) (test_symmetry_reduce.jl:164-212).

    Returns (maps[G, n] int32 with site i -> maps[g, i], amplitudes[G] complex128)."""
    L1, L2 = shape
    m1, m2 = momentum
    n = L1 * L2
    maps = np.empty((n, n), dtype=np.int32)
    amps = np.empty(n, dtype=np.complex128)
    for b in range(L2):
        for a in range(L1):
            g = a + L1 * b
            for y in range(L2):
                for x in range(L1):
                    maps[g, x + L1 * y] = (x + a) % L1 + L1 * ((y + b) % L2)
            amps[g] = np.exp(-2j * np.pi * (m1 * a / L1 + m2 * b / L2))
    return maps, amps


def symmetry_apply(bw, off, site_map, b, flip=0):
    bw = np.asarray(bw, dtype=np.int32)
    off = np.asarray(off, dtype=np.int32)
    site_map = np.asarray(site_map, dtype=np.int32)
    return int(lib().or_symmetry_apply(len(bw), _p(bw, ctypes.c_int32), _p(off, ctypes.c_int32),
                                       _p(site_map, ctypes.c_int32), flip, b))


class ReducedTables:
    """ReducedHilbertSpaceRepresentation fields -- reduced_hilbert_space_representation.jl:13-22."""

    def __init__(self, parent, basis_list, basis_mapping_index, basis_mapping_amplitude):
        self.parent = parent
        self.basis_list = basis_list
        self.basis_mapping_index = basis_mapping_index
        self.basis_mapping_amplitude = basis_mapping_amplitude

    @property
    def dim(self):
        return int(self.basis_list.size)


def symmetry_reduce(parent: np.ndarray, bw, off, maps, amps, flips=None, tol: float = RTOL) -> ReducedTables:
    """symmetry_reduce_serial(hsr, symops_and_amplitudes; tol) -- symmetry_reduce_generic.jl:22-106."""
    amps = np.asarray(amps, dtype=np.complex128)
    if not np.all(np.abs(np.abs(amps) - 1.0) <= RTOL):
        raise ArgumentError("all amplitudes need to have norm 1")
    parent = np.ascontiguousarray(parent, dtype=np.uint64)
    maps = np.ascontiguousarray(maps, dtype=np.int32)
    G, n = maps.shape
    bw = np.asarray(bw, dtype=np.int32)
    off = np.asarray(off, dtype=np.int32)
    fl = None if flips is None else np.ascontiguousarray(flips, dtype=np.uint64)
    a = np.ascontiguousarray(amps).view(np.float64)
    reps = np.empty(max(parent.size, 1), dtype=np.uint64)
    mi = np.empty(max(parent.size, 1), dtype=np.int64)
    ma = np.empty(max(parent.size, 1), dtype=np.complex128)
    nr = lib().or_symmetry_reduce(_p(parent, ctypes.c_uint64), parent.size, n, _p(bw, ctypes.c_int32),
                                  _p(off, ctypes.c_int32), G, _p(maps, ctypes.c_int32), _p(fl, ctypes.c_uint64),
                                  _p(a, ctypes.c_double), tol, _p(reps, ctypes.c_uint64),
                                  _p(mi, ctypes.c_int64), _p(ma.view(np.float64), ctypes.c_double))
    return ReducedTables(parent, reps[:nr].copy(), mi[:parent.size].copy(), ma[:parent.size].copy())


def _apply(fname, basis, parent, red, terms, x, out, accumulate, nthreads):
    masks, rows, cols, amps = term_arrays(terms) if not isinstance(terms, tuple) else terms
    amps = np.ascontiguousarray(amps, dtype=np.complex128)
    x = np.ascontiguousarray(x, dtype=np.complex128)
    if out is None:
        out = np.zeros(basis.size, dtype=np.complex128)
    mi = None if red is None else red.basis_mapping_index
    ma = None if red is None else red.basis_mapping_amplitude.view(np.float64)
    getattr(lib(), fname)(_p(basis, ctypes.c_uint64), basis.size, _p(parent, ctypes.c_uint64), parent.size,
                          _p(mi, ctypes.c_int64), _p(ma, ctypes.c_double), len(masks),
                          _p(masks, ctypes.c_uint64), _p(rows, ctypes.c_uint64), _p(cols, ctypes.c_uint64),
                          _p(amps.view(np.float64), ctypes.c_double), _p(x.view(np.float64), ctypes.c_double),
                          _p(out.view(np.float64), ctypes.c_double), int(accumulate), int(nthreads))
    return out


def apply_rows(space, terms, x, out=None, accumulate=False, nthreads=0):
    """mul!/apply!(out, opr, state) -- abstract_operator_representation.jl:110-118, 296-316, 358-378.
    `space` is a parent basis array (OperatorRepresentation) or ReducedTables
    (ReducedOperatorRepresentation)."""
    if isinstance(space, ReducedTables):
        return _apply("or_apply_rows", space.basis_list, space.parent, space, terms, x, out, accumulate, nthreads)
    return _apply("or_apply_rows", space, space, None, terms, x, out, accumulate, nthreads)


class RowSampler:
    """Bounded samples of mul! for the CPU baseline: rows [r0, r1) of opr * x with all host threads.
    The off-diagonal element count of each row block is returned for the byte model."""

    def __init__(self, space, terms, x, nthreads=0):
        if isinstance(space, ReducedTables):
            self.basis, self.parent, self.red = space.basis_list, space.parent, space
        else:
            self.basis, self.parent, self.red = space, space, None
        self.masks, self.rows, self.cols, amps = term_arrays(terms) if not isinstance(terms, tuple) else terms
        self.amps = np.ascontiguousarray(amps, dtype=np.complex128)
        self.x = np.ascontiguousarray(x, dtype=np.complex128)
        self.y = np.zeros(self.basis.size, dtype=np.complex128)
        self.nthreads = int(nthreads)

    def run(self, r0, r1, count=False):
        nnz = np.zeros(1, dtype=np.int64)
        mi = None if self.red is None else self.red.basis_mapping_index
        ma = None if self.red is None else self.red.basis_mapping_amplitude.view(np.float64)
        lib().or_apply_rows_range(_p(self.basis, ctypes.c_uint64), self.basis.size, _p(self.parent, ctypes.c_uint64),
                                  self.parent.size, _p(mi, ctypes.c_int64), _p(ma, ctypes.c_double), len(self.masks),
                                  _p(self.masks, ctypes.c_uint64), _p(self.rows, ctypes.c_uint64),
                                  _p(self.cols, ctypes.c_uint64), _p(self.amps.view(np.float64), ctypes.c_double),
                                  _p(self.x.view(np.float64), ctypes.c_double),
                                  _p(self.y.view(np.float64), ctypes.c_double), 0, self.nthreads, int(r0), int(r1),
                                  _p(nnz, ctypes.c_int64) if count else None)
        return int(nnz[0])


class OrbitTables:
    """The reference's mapping tables evaluated orbit by orbit, without parent-sized arrays.

    symmetry_reduce_generic.jl:22-106 fills basis_mapping_index / basis_mapping_amplitude for every
    parent state; where those tables do not fit in host memory (the 6x6 torus: ~290 GB), the entries a
    row needs are computed here for one orbit at a time with the same semantics (orbit minimum as
    representative, stabiliser amplitudes ~1 within tol, the last group element reaching a member
    gives its phase, 1/sqrt(#distinct members)).  The parent must be one popcount sector of 1-bit sites
    (a spin-1/2 2Sz sector).  `basis_list` is the sorted representative table under test; every
    representative a sampled row reaches is looked up in it (a missing one is reported)."""

    def __init__(self, n_sites, parent_popcount, maps, amps, basis_list, flips=None, tol: float = RTOL, torus=None):
        self.n = int(n_sites)
        self.k = int(parent_popcount)
        self.bw = np.ones(self.n, dtype=np.int32)
        self.off = np.arange(self.n, dtype=np.int32)
        self.maps = np.ascontiguousarray(maps, dtype=np.int32)
        self.G = self.maps.shape[0]
        self.amps = np.ascontiguousarray(np.asarray(amps, dtype=np.complex128))
        self.flips = None if flips is None else np.ascontiguousarray(flips, dtype=np.uint64)
        self.tol = float(tol)
        self.basis_list = np.ascontiguousarray(basis_list, dtype=np.uint64)
        # torus=(L1, L2): the group is the torus translation group in translation_symops's order;
        # rows() then applies its elements by word rotations (same results, faster), for timing
        self.torus = torus

    def orbit_info(self, states):
        """(representative, kept (bool), #distinct members, mapping amplitude) of every state."""
        states = np.ascontiguousarray(states, dtype=np.uint64)
        m = states.size
        rep = np.empty(m, dtype=np.uint64)
        comp = np.empty(m, dtype=np.int32)
        nd = np.empty(m, dtype=np.int32)
        am = np.empty(m, dtype=np.complex128)
        lib().or_orbit_info(self.n, _p(self.bw, ctypes.c_int32), _p(self.off, ctypes.c_int32), self.G,
                            _p(self.maps, ctypes.c_int32), _p(self.flips, ctypes.c_uint64),
                            _p(self.amps.view(np.float64), ctypes.c_double), self.tol, _p(states, ctypes.c_uint64), m,
                            _p(rep, ctypes.c_uint64), _p(comp, ctypes.c_int32), _p(nd, ctypes.c_int32),
                            _p(am.view(np.float64), ctypes.c_double))
        return rep, comp == 1, nd, am

    def rows(self, terms, x, sample):
        """Rows `sample` of mul!(out, represent(rhsr, op), x) (reduced_operator_representation.jl:57-85)
        as (values, status, nnz_off): status 0 ok, 1 not a representative, 2 orbit not kept, 3 a
        column's representative missing from basis_list."""
        masks, rows, cols, amps = term_arrays(terms) if not isinstance(terms, tuple) else terms
        masks = np.ascontiguousarray(masks, dtype=np.uint64)
        rows = np.ascontiguousarray(rows, dtype=np.uint64)
        cols = np.ascontiguousarray(cols, dtype=np.uint64)
        amps = np.ascontiguousarray(amps, dtype=np.complex128)
        x = np.ascontiguousarray(x, dtype=np.complex128)
        if x.size != self.basis_list.size:
            raise ValueError("x must have one entry per representative")
        sample = np.ascontiguousarray(sample, dtype=np.int64)
        m = sample.size
        out = np.empty(m, dtype=np.complex128)
        st = np.empty(m, dtype=np.int32)
        nnz = np.empty(m, dtype=np.int64)
        common = (_p(self.basis_list, ctypes.c_uint64), self.basis_list.size, self.k, self.n,
                  _p(self.bw, ctypes.c_int32), _p(self.off, ctypes.c_int32), self.G, _p(self.maps, ctypes.c_int32))
        tail = (_p(self.amps.view(np.float64), ctypes.c_double), self.tol, len(masks),
                _p(masks, ctypes.c_uint64), _p(rows, ctypes.c_uint64), _p(cols, ctypes.c_uint64),
                _p(amps.view(np.float64), ctypes.c_double), _p(x.view(np.float64), ctypes.c_double),
                _p(sample, ctypes.c_int64), m, _p(out.view(np.float64), ctypes.c_double),
                _p(st, ctypes.c_int32), _p(nnz, ctypes.c_int64))
        if self.torus is not None and self.flips is None:
            lib().or_sampled_rows_torus(int(self.torus[0]), int(self.torus[1]), *common, *tail)
        else:
            lib().or_sampled_rows(*common, _p(self.flips, ctypes.c_uint64), *tail)
        return out, st, nnz


def torus_representatives(shape, n_up, momentum=(0, 0)) -> np.ndarray:
    """Sorted representatives of the momentum sector of the n_up sector of an L1 x L2 torus of
    spin-1/2 sites, enumerated on the host without a parent basis: the states that are the minimum
    of their translation orbit and whose stabiliser has trivial character -- the set the reference's
    ascending visited-flag sweep keeps (symmetry_reduce_generic.jl:50-72).  Character convention of
    translation_symops."""
    L1, L2 = shape
    G = L1 * L2
    m1, m2 = momentum
    num = np.array([(m1 * (g % L1) * L2 + m2 * (g // L1) * L1) % G for g in range(G)], dtype=np.int32)
    nch = max(64, 16 * num_threads())
    n = lib().or_torus_reps(L1, L2, n_up, _p(num, ctypes.c_int32), G, nch, None)
    if n < 0:
        raise ArgumentError("unsupported torus")
    out = np.empty(max(n, 1), dtype=np.uint64)
    lib().or_torus_reps(L1, L2, n_up, _p(num, ctypes.c_int32), G, nch, _p(out, ctypes.c_uint64))
    return out[:n]


def _cycle_lengths(site_map):
    n = len(site_map)
    seen = [False] * n
    out = []
    for i in range(n):
        if seen[i]:
            continue
        ln, j = 0, i
        while not seen[j]:
            seen[j] = True
            j = int(site_map[j])
            ln += 1
        out.append(ln)
    return out


def sector_dimension(maps, char_num, char_den, n_up):
    """Dimension of the symmetry sector of the n_up-particle (popcount) sector of 1-bit sites, by
    Burnside's lemma: (1/|G|) sum_g conj(chi(g)) #{states with n_up ones fixed by g}, with
    chi(g) = exp(2 pi i char_num[g] / char_den).  A state is fixed by a site permutation when it is
    constant on every cycle, so the count is the number of cycle subsets holding n_up sites.  It equals
    the number of representatives whose stabiliser has character 1 (the reduced dimension), since each
    orbit contributes one to the isotypic component exactly when the character is trivial on its
    stabiliser.  Exact integer counts per character residue; the final sum is rounded."""
    maps = np.asarray(maps)
    G = maps.shape[0]
    per_res = {}
    for g in range(G):
        ways = [0] * (n_up + 1)
        ways[0] = 1
        for ln in _cycle_lengths(maps[g]):
            for t in range(n_up, ln - 1, -1):
                ways[t] += ways[t - ln]
        r = int(char_num[g]) % int(char_den)
        per_res[r] = per_res.get(r, 0) + ways[n_up]
    total = sum(cnt * complex(math.cos(2 * math.pi * r / char_den), -math.sin(2 * math.pi * r / char_den))
                for r, cnt in per_res.items())
    val = total / G
    out = int(round(val.real))
    if abs(val.real - out) > 1e-3 or abs(val.imag) > 1e-3:
        raise ValueError(f"non-integer sector dimension {val}")
    return out


def apply_cols(space, terms, x, out=None, accumulate=False, nthreads=0):
    """apply!(out, state, opr): out += transpose(state) * opr -- :327-347, 389-409."""
    if isinstance(space, ReducedTables):
        return _apply("or_apply_cols", space.basis_list, space.parent, space, terms, x, out, accumulate, nthreads)
    return _apply("or_apply_cols", space, space, None, terms, x, out, accumulate, nthreads)


def unreduce(red: ReducedTables, small: np.ndarray) -> np.ndarray:
    """symmetry_unreduce -- symmetry_reduce.jl:208-225."""
    small = np.ascontiguousarray(small, dtype=np.complex128)
    large = np.empty(red.parent.size, dtype=np.complex128)
    lib().or_unreduce(_p(red.basis_mapping_index, ctypes.c_int64),
                      _p(red.basis_mapping_amplitude.view(np.float64), ctypes.c_double), red.parent.size,
                      _p(small.view(np.float64), ctypes.c_double), _p(large.view(np.float64), ctypes.c_double))
    return large


def reduce_vector(red: ReducedTables, large: np.ndarray) -> np.ndarray:
    """symmetry_reduce(rhsr, large_vector) -- symmetry_reduce.jl:38-56."""
    large = np.ascontiguousarray(large, dtype=np.complex128)
    small = np.empty(red.dim, dtype=np.complex128)
    lib().or_reduce_vector(_p(red.basis_mapping_index, ctypes.c_int64),
                           _p(red.basis_mapping_amplitude.view(np.float64), ctypes.c_double), red.parent.size,
                           _p(large.view(np.float64), ctypes.c_double), _p(small.view(np.float64), ctypes.c_double),
                           red.dim)
    return small


def dense_matrix(space, terms) -> np.ndarray:
    """Matrix(opr) assembled column by column from the row iterator applied to unit vectors."""
    n = space.dim if isinstance(space, ReducedTables) else space.size
    M = np.zeros((n, n), dtype=np.complex128)
    e = np.zeros(n, dtype=np.complex128)
    for j in range(n):
        e[:] = 0
        e[j] = 1
        M[:, j] = apply_rows(space, terms, e)
    return M


# ---------------------------------------------------------------------------------------------
# Seeded inputs and the FP64 eigen oracle
# ---------------------------------------------------------------------------------------------

_GAMMA = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed: int, count: int, start: int = 0) -> np.ndarray:
    """Outputs start..start+count-1 of SplitMix64 seeded with `seed` (counter form)."""
    with np.errstate(over="ignore"):
        k = np.arange(start + 1, start + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def complex_gaussian(n: int, seed: int) -> np.ndarray:
    """Seeded complex Gaussian vector, (g1 + i g2)/sqrt(2) per entry by Box-Muller, normalised."""
    z = splitmix64(seed, 2 * n)
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    u1 = 1.0 - u[0::2]
    u2 = u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    v = (r * np.cos(2 * np.pi * u2) + 1j * r * np.sin(2 * np.pi * u2)) / math.sqrt(2.0)
    return v / np.linalg.norm(v)


def lanczos_e0(matvec, n: int, steps: int, seed: int = 1, reorth: bool = True):
    """Plain FP64 Lanczos with optional full reorthogonalisation; returns (E0, alphas, betas)."""
    v = complex_gaussian(n, seed)
    V = [v] if reorth else None
    alphas, betas = [], []
    v_prev = np.zeros(n, dtype=np.complex128)
    beta = 0.0
    for j in range(steps):
        w = matvec(v) - beta * v_prev
        a = np.vdot(v, w).real
        w = w - a * v
        if reorth:
            for u in V:
                w = w - np.vdot(u, w) * u
        alphas.append(a)
        beta = np.linalg.norm(w)
        if beta < 1e-13 or j == steps - 1:
            break
        betas.append(beta)
        v_prev, v = v, w / beta
        if reorth:
            V.append(v)
    from scipy.linalg import eigh_tridiagonal
    ev = eigh_tridiagonal(np.array(alphas), np.array(betas[:len(alphas) - 1]), eigvals_only=True)
    return float(ev[0]), alphas, betas
