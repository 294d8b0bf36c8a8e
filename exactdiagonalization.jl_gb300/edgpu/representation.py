"""Representation and symmetry layers over libedgpu.so.

Mirrors, for Python callers, the reference's API on this path:
  represent(hs) / represent(HilbertSpaceSector(...)) / represent(hs, basis_list)
        -> HilbertSpaceRepresentation            (hilbert_space_representation.jl:215-256)
  symmetry_reduce(hsr, symops_and_amplitudes)    (symmetry_reduce_generic.jl:7-106)
        -> ReducedHilbertSpaceRepresentation
  represent(hsr_or_rhsr, op)                     (operator_representation.jl:34-36,
        -> OperatorRepresentation                 reduced_operator_representation.jl:40-42)
  mul_(out, opr, state)   == LinearAlgebra.mul!  (abstract_operator_representation.jl:110-118)
  apply_(out, opr, state) == apply!  (adds)      (:260-267)
  apply_(out, state, opr) == apply!  transpose   (:278-285)
  opr @ state, state @ opr                       (operator_representation.jl:122-139)
Indices are 0-based; -1 marks "absent" as in the reference.  Vectors are numpy arrays (host buffers:
copied to the GPU and back inside the call) or torch CUDA tensors (device buffers, run on torch's
current stream).  All arithmetic runs in the CUDA kernels; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes
import math
from fractions import Fraction
from functools import reduce as _reduce
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import (ArgumentError, BoundsError, DimensionMismatch, FP64, MIXED, PAIR_UNIFORM, check, lib, ptr)
from .hilbert import HilbertSpace, HilbertSpaceSector, basespace
from .operators import NullOperator, RTOL, simplify, term_arrays

RTOL_F64 = float(np.sqrt(np.finfo(np.float64).eps))   # Base.rtoldefault(Float64)

_PREC = {"fp64": FP64, "float64": FP64, "complex128": FP64, FP64: FP64,
         "mixed": MIXED, "fp32": MIXED, "complex64": MIXED, MIXED: MIXED}


def _prec(p) -> int:
    try:
        return _PREC[p]
    except KeyError:
        raise ArgumentError(f"unknown precision {p!r}; use 'fp64' or 'mixed'")


def _is_torch(a) -> bool:
    return type(a).__module__.split(".")[0] == "torch"


def _torch_stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


# ------------------------------------------------------------------------------------------------
# spaces
# ------------------------------------------------------------------------------------------------

class _SpaceHandle:
    def __init__(self, handle):
        self._h = handle

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.edgpu_space_destroy(h)
            self._h = None


class HilbertSpaceRepresentation:
    """HilbertSpaceRepresentation(hilbert_space, basis_list, basis_lookup) with the sorted basis held on
    the GPU (hilbert_space_representation.jl:16-74)."""

    def __init__(self, hilbert_space, handle, lazy=False):
        self.hilbert_space = basespace(hilbert_space)
        self._space = _SpaceHandle(handle)
        self.lazy = lazy
        d = ctypes.c_int64()
        check(lib().edgpu_space_dim(handle, ctypes.byref(d)))
        self._dim = int(d.value)
        self._basis = None

    @property
    def handle(self):
        return self._space._h

    @property
    def dimension(self) -> int:
        return self._dim

    def __len__(self):
        return self._dim

    @property
    def basis_list(self) -> np.ndarray:
        if self._basis is None:
            out = np.empty(self._dim, dtype=np.uint64)
            check(lib().edgpu_space_get_basis(self.handle, ptr(out, ctypes.c_uint64), self._dim))
            self._basis = out
        return self._basis

    def lookup(self, keys) -> np.ndarray:
        """get(basis_lookup, key, -1) for each key, on the GPU (frozensortedarray.jl:45-48)."""
        keys = np.ascontiguousarray(np.atleast_1d(keys), dtype=np.uint64)
        out = np.empty(keys.size, dtype=np.int64)
        check(lib().edgpu_space_lookup(self.handle, ptr(keys, ctypes.c_uint64), keys.size,
                                       ptr(out, ctypes.c_int64)))
        return out

    def basis_lookup(self, key) -> int:
        """basis_lookup[key]: KeyError when absent (frozensortedarray.jl:34-38)."""
        i = int(self.lookup([key])[0])
        if i < 0:
            raise KeyError(f"key {key} not found")
        return i

    def __eq__(self, other):
        return (isinstance(other, HilbertSpaceRepresentation) and self.hilbert_space == other.hilbert_space
                and np.array_equal(self.basis_list, other.basis_list))

    def __hash__(self):
        return id(self)


def _space_arrays(hs: HilbertSpace):
    dims = np.array([s.dimension for s in hs.sites], dtype=np.int32)
    qlen = hs.qlen
    qn = np.array([v for s in hs.sites for st in s.states for v in st.quantum_number], dtype=np.int64)
    return dims, qlen, qn


def represent(x, arg=None, *, lazy: bool = False):
    """represent(...) dispatch, as in the reference:
      represent(hs) / represent(hss)            sector basis enumerated on the GPU
      represent(hs, basis_list)                 caller-given basis (sorted; duplicates rejected)
      represent(hsr_or_rhsr, operator)          OperatorRepresentation
    lazy=True keeps only the sector definition (for symmetry_reduce of very large sectors)."""
    if isinstance(x, (HilbertSpaceRepresentation, ReducedHilbertSpaceRepresentation)):
        return OperatorRepresentation(x, arg)
    if arg is not None and not isinstance(arg, (HilbertSpace, HilbertSpaceSector)):
        return _represent_basis(x, np.asarray(arg))
    if isinstance(x, HilbertSpaceSector):
        hs = basespace(x)
        allowed = sorted(x.allowed_quantum_numbers)
        n_allowed = len(allowed)
    elif isinstance(x, HilbertSpace):
        hs = x
        allowed = []
        n_allowed = -1
    else:
        raise ArgumentError(f"cannot represent {type(x).__name__}")
    dims, qlen, qn = _space_arrays(hs)
    al = np.array([v for q in allowed for v in q], dtype=np.int64)
    h = ctypes.c_void_p()
    check(lib().edgpu_space_create(hs.n_sites, ptr(dims, ctypes.c_int32), qlen,
                                   ptr(qn, ctypes.c_int64) if qn.size else None, n_allowed,
                                   ptr(al, ctypes.c_int64) if al.size else None,
                                   _lib.SPACE_LAZY if lazy else 0, ctypes.byref(h)))
    return HilbertSpaceRepresentation(hs, h, lazy=lazy)


def _represent_basis(x, basis_list: np.ndarray):
    hs = basespace(x)
    b = np.ascontiguousarray(basis_list, dtype=np.uint64)
    dims = np.array([s.dimension for s in hs.sites], dtype=np.int32)
    h = ctypes.c_void_p()
    check(lib().edgpu_space_from_basis(hs.n_sites, ptr(dims, ctypes.c_int32), ptr(b, ctypes.c_uint64), b.size,
                                       ctypes.byref(h)))
    return HilbertSpaceRepresentation(hs, h)


represent_array = represent


def dimension(x) -> int:
    return x.dimension


# ------------------------------------------------------------------------------------------------
# symmetry
# ------------------------------------------------------------------------------------------------

class SitePermutation:
    """SitePermutation: the field of site i moves to site map[i] (0-based) -- symmetry_apply.jl:82-92."""

    def __init__(self, site_map: Sequence[int]):
        self.map = [int(v) for v in site_map]
        if sorted(self.map) != list(range(len(self.map))):
            raise ArgumentError("not a permutation")

    def __mul__(self, other):
        return DirectProductOperation([self, other])

    def __eq__(self, other):
        return isinstance(other, SitePermutation) and self.map == other.map

    def __hash__(self):
        return hash(tuple(self.map))


class GlobalBitFlip:
    """GlobalBitFlip(value): XOR with the full mask when value -- bitflipsymmetry.jl:8-35."""

    def __init__(self, value: bool = False):
        self.value = bool(value)

    def __mul__(self, other):
        if isinstance(other, GlobalBitFlip):
            return GlobalBitFlip(self.value ^ other.value)
        return DirectProductOperation([self, other])

    def __eq__(self, other):
        return isinstance(other, GlobalBitFlip) and self.value == other.value

    def __hash__(self):
        return hash(self.value)


class DirectProductOperation:
    """(A B C)(psi) = A(B(C(psi))) -- symmetry_apply.jl:65-77."""

    def __init__(self, operations):
        self.operations = list(operations)

    def __mul__(self, other):
        return DirectProductOperation(self.operations + [other])


def _as_map_flip(hs: HilbertSpace, op):
    """Bit action of a symmetry operation as (site map, XOR mask): g.q = P(q) ^ f."""
    n = hs.n_sites
    if isinstance(op, SitePermutation):
        if len(op.map) != n:
            raise ArgumentError("permutation size does not match the number of sites")
        return list(op.map), 0
    if isinstance(op, GlobalBitFlip):
        return list(range(n)), (hs.get_bitmask() if op.value else 0)
    if isinstance(op, DirectProductOperation):
        m, f = list(range(n)), 0
        for sub in reversed(op.operations):          # apply right to left
            sm, sf = _as_map_flip(hs, sub)
            # sub.(P q ^ f) = Psub P q ^ Psub f ^ fsub
            f = _permute_bits(hs, sm, f) ^ sf
            m = [sm[m[i]] for i in range(n)]
        return m, f
    raise ArgumentError(f"unsupported symmetry operation {type(op).__name__}")


def _permute_bits(hs: HilbertSpace, site_map, b: int) -> int:
    out = 0
    for i in range(hs.n_sites):
        w = hs.bitwidths[i]
        out |= ((b >> hs.bitoffsets[i]) & ((1 << w) - 1)) << hs.bitoffsets[site_map[i]]
    return out


def symmetry_apply(hs, op, bitrep: int):
    """symmetry_apply(hs, op, bitrep) -> (bitrep', sign) -- symmetry_apply.jl:65-92, bitflipsymmetry.jl:23-35."""
    hs = basespace(hs)
    m, f = _as_map_flip(hs, op)
    return _permute_bits(hs, m, int(bitrep)) ^ f, 1


def _roots_of_unity(amps, tol):
    """Amplitudes -> (numerators, common denominator) with amp = exp(2 pi i num / den)."""
    dens, fracs = [], []
    for a in amps:
        a = complex(a)
        if not abs(abs(a) - 1.0) <= tol:
            raise ArgumentError("all amplitudes need to have norm 1")
        theta = (math.atan2(a.imag, a.real) / (2 * math.pi)) % 1.0
        fr = Fraction(theta).limit_denominator(4096)
        if abs(complex(math.cos(2 * math.pi * fr), math.sin(2 * math.pi * fr)) - a) > max(tol, 1e-12):
            raise ArgumentError("amplitudes must be roots of unity (characters of a finite group)")
        fr = fr % 1
        fracs.append(fr)
        dens.append(fr.denominator)
    den = _reduce(lambda x, y: x * y // math.gcd(x, y), dens, 1)
    if den > 4096:
        raise ArgumentError("character denominator too large")
    return [int(f * den) % den for f in fracs], den


class ReducedHilbertSpaceRepresentation:
    """ReducedHilbertSpaceRepresentation (reduced_hilbert_space_representation.jl:13-22).

    The sorted representatives live on the GPU; basis_mapping_index / basis_mapping_amplitude
    (parent-sized, the reference's fields) are materialised on request only."""

    def __init__(self, parent: HilbertSpaceRepresentation, handle, symops):
        self.parent = parent
        self._space = _SpaceHandle(handle)
        self.symops = symops
        d = ctypes.c_int64()
        check(lib().edgpu_space_dim(handle, ctypes.byref(d)))
        self._dim = int(d.value)
        self._basis = None
        self._mapping = None

    @property
    def handle(self):
        return self._space._h

    @property
    def hilbert_space(self):
        return self.parent.hilbert_space

    @property
    def dimension(self) -> int:
        return self._dim

    def build_map(self, max_bytes: Optional[int] = None) -> bool:
        """Build the compact parent-state map (the counterpart of the reference's parent-sized
        basis_mapping_index / basis_mapping_amplitude tables, 4 or 8 bytes per parent state) when the
        parent is one fixed-popcount sector and the map needs at most max_bytes (default: a quarter of
        the free device memory).  Products then look targets up instead of canonicalising them.
        Returns whether the map was built."""
        if max_bytes is None:
            import torch
            free, _ = torch.cuda.mem_get_info()
            max_bytes = free // 4
        built = ctypes.c_int32()
        check(lib().edgpu_space_build_map(self.handle, int(max_bytes), ctypes.byref(built)))
        return bool(built.value)

    def free_map(self) -> None:
        check(lib().edgpu_space_free_map(self.handle))

    @property
    def map_info(self) -> Tuple[int, int]:
        """(parent states covered, bytes per entry); (0, 0) without a map."""
        n = ctypes.c_int64()
        b = ctypes.c_int32()
        check(lib().edgpu_space_map_info(self.handle, ctypes.byref(n), ctypes.byref(b)))
        return int(n.value), int(b.value)

    def __len__(self):
        return self._dim

    @property
    def basis_list(self) -> np.ndarray:
        if self._basis is None:
            out = np.empty(self._dim, dtype=np.uint64)
            check(lib().edgpu_space_get_basis(self.handle, ptr(out, ctypes.c_uint64), self._dim))
            self._basis = out
        return self._basis

    def _get_mapping(self):
        if self._mapping is None:
            n = self.parent.dimension
            idx = np.empty(n, dtype=np.int64)
            amp = np.empty(n, dtype=np.complex128)
            check(lib().edgpu_reduce_mapping(self.handle, ptr(idx, ctypes.c_int64),
                                             ptr(amp.view(np.float64), ctypes.c_double), n))
            self._mapping = (idx, amp)
        return self._mapping

    @property
    def basis_mapping_index(self) -> np.ndarray:
        return self._get_mapping()[0]

    @property
    def basis_mapping_amplitude(self) -> np.ndarray:
        return self._get_mapping()[1]

    def orbit_sizes(self) -> np.ndarray:
        out = np.empty(self._dim, dtype=np.int32)
        check(lib().edgpu_space_orbit_sizes(self.handle, ptr(out, ctypes.c_int32), self._dim))
        return out

    def lookup(self, keys) -> np.ndarray:
        keys = np.ascontiguousarray(np.atleast_1d(keys), dtype=np.uint64)
        out = np.empty(keys.size, dtype=np.int64)
        check(lib().edgpu_space_lookup(self.handle, ptr(keys, ctypes.c_uint64), keys.size,
                                       ptr(out, ctypes.c_int64)))
        return out


def symmetry_reduce(x, arg, tol: float = RTOL):
    """symmetry_reduce(hsr, symops_and_amplitudes; tol) -> ReducedHilbertSpaceRepresentation
    (symmetry_reduce_generic.jl:7-106); symmetry_reduce(rhsr, large_vector) -> small vector
    (symmetry_reduce.jl:29-35).  The first element must be the identity."""
    if isinstance(x, ReducedHilbertSpaceRepresentation):
        return _reduce_vector(x, arg)
    if not isinstance(x, HilbertSpaceRepresentation):
        raise ArgumentError("symmetry_reduce needs a HilbertSpaceRepresentation")
    hs = x.hilbert_space
    symops = list(arg)
    if not symops:
        raise ArgumentError("empty symmetry group")
    maps, flips = [], []
    for op, _ in symops:
        m, f = _as_map_flip(hs, op)
        maps.append(m)
        flips.append(f)
    num, den = _roots_of_unity([a for _, a in symops], tol)
    maps_a = np.ascontiguousarray(np.array(maps, dtype=np.int32).reshape(-1))
    flips_a = np.array(flips, dtype=np.uint64)
    num_a = np.array(num, dtype=np.int32)
    h = ctypes.c_void_p()
    check(lib().edgpu_reduce(x.handle, len(symops), ptr(maps_a, ctypes.c_int32), ptr(flips_a, ctypes.c_uint64),
                             ptr(num_a, ctypes.c_int32), den, ctypes.byref(h)))
    return ReducedHilbertSpaceRepresentation(x, h, symops)


symmetry_reduce_serial = symmetry_reduce
symmetry_reduce_parallel = symmetry_reduce


def _parent_dim(rhsr) -> int:
    n = ctypes.c_int64()
    check(lib().edgpu_space_parent_dim(rhsr.handle, ctypes.byref(n)))
    return int(n.value)


def _device_vector_map(rhsr, v, unreduce: bool):
    """symmetry_unreduce / symmetry_reduce on the device (edgpu_symmetry_unreduce_device /
    edgpu_symmetry_reduce_device): CUDA tensors in and out (complex128: FP64, complex64: mixed); host
    arrays go through a complex128 device round trip."""
    import torch
    n, npar = rhsr.dimension, _parent_dim(rhsr)
    n_in, n_out = (n, npar) if unreduce else (npar, n)
    if len(v) != n_in:
        what = "reduced" if unreduce else "larger"
        raise DimensionMismatch(f"Dimension of the input vector should match the {what} representation")
    host = not _is_torch(v)
    t = torch.from_numpy(np.ascontiguousarray(v, dtype=np.complex128)).cuda() if host else v
    if not (t.is_cuda and t.is_contiguous() and t.dtype in (torch.complex128, torch.complex64)):
        raise ArgumentError("the vector must be a contiguous complex CUDA tensor")
    prec = FP64 if t.dtype == torch.complex128 else MIXED
    out = torch.empty(n_out, dtype=t.dtype, device=t.device)
    fn = lib().edgpu_symmetry_unreduce_device if unreduce else lib().edgpu_symmetry_reduce_device
    check(fn(rhsr.handle, prec, ctypes.c_void_p(t.data_ptr()), n_in, ctypes.c_void_p(out.data_ptr()), n_out,
             _torch_stream()))
    return out.cpu().numpy() if host else out


def _reduce_vector(rhsr: ReducedHilbertSpaceRepresentation, large):
    return _device_vector_map(rhsr, large, False)


def search_stats(space) -> dict:
    """Shape of a representation's search directory (buckets, shift, keys inline per bucket, window
    halvings, fraction of rows answered by a bucket summary)."""
    nb, sh, k, st, fr = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_double()
    check(lib().edgpu_space_search_stats(space.handle, ctypes.byref(nb), ctypes.byref(sh), ctypes.byref(k),
                                         ctypes.byref(st), ctypes.byref(fr)))
    return {"buckets": int(nb.value), "shift": int(sh.value), "inline_per_bucket": int(k.value),
            "window_steps": int(st.value), "inline_fraction": float(fr.value)}


def symmetry_unreduce(rhsr: ReducedHilbertSpaceRepresentation, small):
    """symmetry_unreduce(rhsr, small_vector) -- symmetry_reduce.jl:208-225: the parent-space vector
    large[i] = ampl(p_i) small[rep(p_i)], computed on the device without parent-sized tables.  CUDA
    tensors stay on the device; host arrays come back as complex128 numpy arrays."""
    return _device_vector_map(rhsr, small, True)


def translation_symops(shape, momentum=(0, 0)) -> List[Tuple[SitePermutation, complex]]:
    """Translation group of an L1 x L2 torus (sites x + L1*y, 0-based) at momentum (m1, m2):
    element T(a,b) (site (x,y) -> (x+a, y+b)) with amplitude exp(-2 pi i (m1 a/L1 + m2 b/L2)),
    listed with the identity first.  This is the convention the reference's tests pin for
    LatticeTools' IrrepComponent (test_symmetry_reduce.jl:164-212: the L=7 one-particle state at
    momentum index 2 unreduces to cis(+2 pi i x/7)/sqrt(7))."""
    if isinstance(shape, int):
        shape = (shape, 1)
    if isinstance(momentum, int):
        momentum = (momentum, 0)
    L1, L2 = shape
    m1, m2 = momentum
    out = []
    for b in range(L2):
        for a in range(L1):
            site_map = [(x + a) % L1 + L1 * ((y + b) % L2) for y in range(L2) for x in range(L1)]
            amp = complex(np.exp(-2j * np.pi * (m1 * a / L1 + m2 * b / L2)))
            out.append((SitePermutation(site_map), amp))
    return out


# ------------------------------------------------------------------------------------------------
# operator representation and the product
# ------------------------------------------------------------------------------------------------

class OperatorRepresentation:
    """OperatorRepresentation / ReducedOperatorRepresentation of a SumOperator on the GPU
    (operator_representation.jl:13-26, reduced_operator_representation.jl:15-30).

    couplings: optional (coupling_ids per term, values) -- the operator is then
    sum_t values[ids[t]] * amps[t] * P_t and coupling_grad() gives dL/dJ."""

    def __init__(self, space, operator, coupling_ids=None, couplings=None):
        self.space = space
        self.operator = operator
        masks, rows, cols, amps = term_arrays(operator)   # the operator's terms as given (no simplify)
        self._terms = (masks, rows, cols, amps)
        self.n_couplings = 1
        cid = None
        cvals = None
        if coupling_ids is not None:
            cid = np.ascontiguousarray(coupling_ids, dtype=np.int32)
            cvals = np.ascontiguousarray(couplings, dtype=np.float64)
            if cid.size != masks.size:
                raise DimensionMismatch("one coupling id per term is required")
            self.n_couplings = int(cvals.size)
        a = np.ascontiguousarray(amps).view(np.float64)
        h = ctypes.c_void_p()
        check(lib().edgpu_op_create(space.handle, int(masks.size), ptr(masks, ctypes.c_uint64),
                                    ptr(rows, ctypes.c_uint64), ptr(cols, ctypes.c_uint64),
                                    ptr(a, ctypes.c_double), ptr(cid, ctypes.c_int32),
                                    self.n_couplings, ptr(cvals, ctypes.c_double), ctypes.byref(h)))
        self._h = h
        self._couplings = np.ones(1) if cvals is None else cvals.copy()

    @classmethod
    def from_terms(cls, space, masks, rows, cols, amps, coupling_ids=None, couplings=None):
        """Operator given directly as a term table (no simplify)."""
        self = cls.__new__(cls)
        self.space = space
        self.operator = None
        masks = np.ascontiguousarray(masks, dtype=np.uint64)
        rows = np.ascontiguousarray(rows, dtype=np.uint64)
        cols = np.ascontiguousarray(cols, dtype=np.uint64)
        amps = np.ascontiguousarray(amps, dtype=np.complex128)
        self._terms = (masks, rows, cols, amps)
        self.n_couplings = 1
        cid = cvals = None
        if coupling_ids is not None:
            cid = np.ascontiguousarray(coupling_ids, dtype=np.int32)
            cvals = np.ascontiguousarray(couplings, dtype=np.float64)
            self.n_couplings = int(cvals.size)
        h = ctypes.c_void_p()
        check(lib().edgpu_op_create(space.handle, int(masks.size), ptr(masks, ctypes.c_uint64),
                                    ptr(rows, ctypes.c_uint64), ptr(cols, ctypes.c_uint64),
                                    ptr(amps.view(np.float64), ctypes.c_double), ptr(cid, ctypes.c_int32),
                                    self.n_couplings, ptr(cvals, ctypes.c_double), ctypes.byref(h)))
        self._h = h
        self._couplings = np.ones(1) if cvals is None else cvals.copy()
        return self

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.edgpu_op_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    @property
    def hilbert_space_representation(self):
        return self.space

    @property
    def terms(self):
        return self._terms

    @property
    def dimension(self) -> int:
        return self.space.dimension

    @property
    def shape(self):
        return (self.space.dimension, self.space.dimension)

    def set_couplings(self, values):
        """New coupling values J_c (same count); the operator's tables are rewritten in place."""
        v = np.ascontiguousarray(values, dtype=np.float64)
        check(lib().edgpu_op_set_couplings(self._h, ptr(v, ctypes.c_double), int(v.size)))
        self._couplings = v.copy()

    @property
    def couplings(self) -> np.ndarray:
        """The current coupling values (a copy)."""
        return self._couplings.copy()

    def autotune(self, precision="mixed"):
        r = ctypes.c_int32()
        ms = ctypes.c_double()
        check(lib().edgpu_op_autotune(self._h, _prec(precision), ctypes.byref(r), ctypes.byref(ms)))
        return int(r.value), float(ms.value)

    def count_nnz(self):
        """(off-diagonal targets generated, of which land on a row of the representation)."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        check(lib().edgpu_op_count_nnz(self._h, ctypes.byref(a), ctypes.byref(b)))
        return int(a.value), int(b.value)

    def set_tiling(self, precision, rows_per_tile):
        check(lib().edgpu_op_set_tiling(self._h, _prec(precision), int(rows_per_tile)))

    def set_pair_schedule(self, enable, targets_per_step: int = 2, uniform: bool = False):
        """Use (default) or bypass the pair-flip schedule of the product for operators whose
        off-diagonal terms all flip two spin-1/2 sites; bypassed, every row tests every term.
        targets_per_step: 2, 4 (with a parent-state map or a target table) or 8 (with a target
        table).  uniform: warp-uniform pair steps of the target-table product (4 or 8 targets per
        step; same results)."""
        code = (int(targets_per_step) | (PAIR_UNIFORM if uniform else 0)) if enable else 0
        check(lib().edgpu_op_set_pair_schedule(self._h, code))

    def schedule(self, precision="mixed"):
        """(rows_per_tile as in set_tiling, pair flips) used by the product: pair flips = 0 when
        every row tests every term, else the targets per lane and step of the pair-flip schedule
        (with PAIR_UNIFORM added for warp-uniform steps)."""
        a, b = ctypes.c_int32(), ctypes.c_int32()
        check(lib().edgpu_op_get_schedule(self._h, _prec(precision), ctypes.byref(a), ctypes.byref(b), None))
        return int(a.value), int(b.value)

    def uses_target_table(self, precision="mixed") -> bool:
        t = ctypes.c_int32()
        check(lib().edgpu_op_get_schedule(self._h, _prec(precision), None, None, ctypes.byref(t)))
        return bool(t.value)

    def build_targets(self, max_bytes: Optional[int] = None) -> bool:
        """Build the target table of the pair-flip schedule (the entry of every (row, target) of the
        product, 4 or 8 bytes each) when the terms allow the schedule and the table needs at most
        max_bytes (default: a quarter of the free device memory).  Returns whether it was built."""
        if max_bytes is None:
            import torch
            free, _ = torch.cuda.mem_get_info()
            max_bytes = free // 4
        built = ctypes.c_int32()
        check(lib().edgpu_op_build_targets(self._h, int(max_bytes), ctypes.byref(built)))
        return bool(built.value)

    def grad_kernel(self, precision="mixed") -> str:
        """The kernel coupling_grad runs: "pair-flip table", "pair-flip map", "term scan" or "queued"."""
        k = ctypes.c_int32()
        check(lib().edgpu_op_grad_kernel(self._h, _prec(precision), ctypes.byref(k)))
        return {2: "pair-flip table", 1: "pair-flip map", 0: "term scan", -1: "queued"}[k.value]

    def table_prefetch(self, precision="mixed", steps: Optional[int] = None) -> int:
        """x prefetch distance (in steps) of the target-table product; sets it when steps is given.
        Returns the setting."""
        cur = ctypes.c_int32()
        check(lib().edgpu_op_table_prefetch(self._h, _prec(precision), -1 if steps is None else int(steps),
                                            ctypes.byref(cur)))
        return int(cur.value)

    def build_adjoint_targets(self, max_bytes: Optional[int] = None) -> bool:
        """Build the adjoint target table (needs the target table): for terms that do not commute with
        the symmetry group, mul_adjoint_ then gathers every column's contributions in a fixed order
        instead of scattering them with atomics.  Returns whether it was built."""
        if max_bytes is None:
            import torch
            free, _ = torch.cuda.mem_get_info()
            max_bytes = free // 2
        built = ctypes.c_int32()
        check(lib().edgpu_op_build_adjoint_targets(self._h, int(max_bytes), ctypes.byref(built)))
        return bool(built.value)

    def free_adjoint_targets(self) -> None:
        check(lib().edgpu_op_free_adjoint_targets(self._h))

    def free_targets(self) -> None:
        check(lib().edgpu_op_free_targets(self._h))

    @property
    def targets_info(self) -> Tuple[int, int]:
        """(entries, bytes per entry) of the target table; (0, 0) without one."""
        n, b = ctypes.c_int64(), ctypes.c_int32()
        check(lib().edgpu_op_targets_info(self._h, ctypes.byref(n), ctypes.byref(b)))
        return int(n.value), int(b.value)

    def build_slabs(self, slab_bytes: int = 54 << 20, max_bytes: Optional[int] = None) -> bool:
        """Build the column-slab table from the target table (which must exist): the product then runs
        one pass per slab of slab_bytes of complex64 x, each gathering only from its slab (mixed
        precision).  max_bytes defaults to a quarter of the free device memory.  Returns whether it
        was built."""
        if max_bytes is None:
            import torch
            free, _ = torch.cuda.mem_get_info()
            max_bytes = free // 4
        built = ctypes.c_int32()
        check(lib().edgpu_op_build_slabs(self._h, int(slab_bytes), int(max_bytes), ctypes.byref(built)))
        return bool(built.value)

    def free_slabs(self) -> None:
        check(lib().edgpu_op_free_slabs(self._h))

    @property
    def slabs_info(self) -> Tuple[int, int, int]:
        """(passes, columns per slab, entries) of the slab table; zeros without one."""
        a, b, c = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64()
        check(lib().edgpu_op_slabs_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return int(a.value), int(b.value), int(c.value)

    def slab_use(self, precision="mixed", use=None) -> int:
        """Whether products read the slab table: 0 (no), or 1 + v for the variant v; sets it when use is
        given (False/True or 0 to 6).  v = 0 to 3: one lane per row (bit 0: cache hints, bit 1: eight
        entries per lane and step), bit-identical; v = 4, 5: two, four lanes per row (their sums are
        added in another fixed order, so they differ from v = 0 to 3 by rounding)."""
        cur = ctypes.c_int32()
        check(lib().edgpu_op_slab_use(self._h, _prec(precision), -1 if use is None else int(use),
                                      ctypes.byref(cur)))
        return int(cur.value)

    def slab_scaling(self, mode=None) -> bool:
        """Layout of the next slab table (mode 0: scaled on sectors of 2^22 rows or more where that saves
        passes or the coefficients are complex, 1: never, 2: always); returns whether the current table
        is scaled (the orbit-size ratio applied to x and to the result rows instead of each entry's
        coefficient)."""
        cur = ctypes.c_int32()
        check(lib().edgpu_op_slab_scaling(self._h, -1 if mode is None else int(mode), ctypes.byref(cur)))
        return bool(cur.value)

    def pair_classes(self):
        """(bond classes, rotation components) of the pair-flip schedule; (0, 0) when it does not apply."""
        a, b = ctypes.c_int32(), ctypes.c_int32()
        check(lib().edgpu_op_pair_classes(self._h, ctypes.byref(a), ctypes.byref(b)))
        return int(a.value), int(b.value)

    def __matmul__(self, state):
        """opr * state: allocates out and calls apply! (operator_representation.jl:122-129)."""
        if _is_torch(state):
            import torch
            out = torch.zeros_like(state)
        else:
            out = np.zeros(self.dimension, dtype=np.complex128)
        return apply_(out, self, state)

    def __rmatmul__(self, state):
        """state * opr: transpose product (operator_representation.jl:132-139)."""
        out = np.zeros(self.dimension, dtype=np.complex128)
        return apply_(out, state, self)

    # -- algebra on representations (abstract_operator_representation.jl:55-107): the operators are
    # combined and simplified on the host, then represented again on the same space ---------------
    def _operator(self):
        if self.operator is None:
            raise ArgumentError("this representation was built from a raw term table; it has no operator")
        return self.operator

    def _same_space(self, other):
        if other.space is not self.space:
            raise ArgumentError("The two OperatorRepresentation's do not have the same HilbertSpaceRepresentation")

    def __add__(self, other):
        if not isinstance(other, OperatorRepresentation):
            return NotImplemented
        self._same_space(other)
        return represent(self.space, simplify(self._operator() + other._operator()))

    def __sub__(self, other):
        if not isinstance(other, OperatorRepresentation):
            return NotImplemented
        self._same_space(other)
        return represent(self.space, simplify(self._operator() - other._operator()))

    def __mul__(self, other):
        if isinstance(other, OperatorRepresentation):
            self._same_space(other)
            return represent(self.space, simplify(self._operator() * other._operator()))
        if isinstance(other, (int, float, complex, np.number)):
            return represent(self.space, simplify(self._operator() * other))
        return NotImplemented

    def __rmul__(self, other):
        if isinstance(other, (int, float, complex, np.number)):
            return represent(self.space, simplify(other * self._operator()))
        return NotImplemented

    def __truediv__(self, other):
        return represent(self.space, simplify(self._operator() / other))

    def __neg__(self):
        return represent(self.space, -self._operator())

    def __pos__(self):
        return represent(self.space, self._operator())

    def simplify(self):
        return represent(self.space, simplify(self._operator()))

    def ishermitian(self) -> bool:
        """ishermitian(opr) (abstract_operator_representation.jl:105-107): of the operator."""
        op = simplify(self._operator())
        if isinstance(op, NullOperator):
            return True
        return isinstance(simplify(op - op.adjoint()), NullOperator)

    @property
    def is_invariant(self) -> bool:
        """Whether the terms commute with every element of the space's symmetry group (then the
        reference's reduced row and column iterators are transposes of each other)."""
        v = ctypes.c_int32()
        check(lib().edgpu_op_is_invariant(self._h, ctypes.byref(v)))
        return bool(v.value)

    # -- sparse assembly (sparse(opr), Matrix(opr), get_row, get_column, getindex) ---------------
    def sparse(self, tol: float = RTOL_F64):
        """sparse(opr) (abstract_operator_representation.jl:135-198) assembled on the GPU in FP64: the
        matrix of the column iterators (as the reference builds it, column by column), entries of
        equal position summed, |value| < tol dropped; a scipy.sparse CSC matrix."""
        return self._assemble(tol, True).T.tocsc()

    def sparse_rows(self, tol: float = RTOL_F64):
        """The matrix of the row iterators, the one mul! applies (CSR).  It equals sparse() for operators
        that commute with the symmetry group."""
        return self._assemble(tol, False)

    def _assemble(self, tol: float, transpose: bool):
        import scipy.sparse as sps
        n = self.dimension
        nnz = ctypes.c_int64()
        check(lib().edgpu_op_sparse(self._h, int(transpose), float(tol), ctypes.byref(nnz), None, None, None))
        rp = np.zeros(n + 1, dtype=np.int64)
        ci = np.zeros(max(nnz.value, 1), dtype=np.int64)
        va = np.zeros(max(nnz.value, 1), dtype=np.complex128)
        check(lib().edgpu_op_sparse(self._h, int(transpose), float(tol), ctypes.byref(nnz), ptr(rp, ctypes.c_int64),
                                    ptr(ci, ctypes.c_int64), ptr(va.view(np.float64), ctypes.c_double)))
        return sps.csr_matrix((va[:nnz.value], ci[:nnz.value], rp), shape=(n, n))

    def todense(self) -> np.ndarray:
        """Matrix(opr) (abstract_operator_representation.jl:121-131): column iterators, nothing dropped."""
        return self.sparse(tol=0.0).toarray()

    def _line(self, i: int, transpose: bool, tol: float):
        n = self.dimension
        if not 0 <= i < n:
            raise BoundsError(f"index {i} out of range for dimension {n}")
        cnt = ctypes.c_int64()
        check(lib().edgpu_op_get_row(self._h, int(transpose), int(i), float(tol), 0, ctypes.byref(cnt), None, None))
        k = cnt.value
        ci = np.zeros(max(k, 1), dtype=np.int64)
        va = np.zeros(max(k, 1), dtype=np.complex128)
        check(lib().edgpu_op_get_row(self._h, int(transpose), int(i), float(tol), k, ctypes.byref(cnt),
                                     ptr(ci, ctypes.c_int64), ptr(va.view(np.float64), ctypes.c_double)))
        return ci[:k], va[:k]

    def get_row(self, i: int, tol: float = RTOL_F64):
        """get_row(opr, irow) (abstract_operator_representation.jl:201-213): (column indices, values)."""
        return self._line(i, False, tol)

    def get_column(self, j: int, tol: float = RTOL_F64):
        """get_column(opr, icol) (abstract_operator_representation.jl:216-228): (row indices, values)."""
        return self._line(j, True, tol)

    def get_element(self, i: int, j: int) -> complex:
        """opr[i, j] (get_element, reduced_operator_representation.jl:119-138): the sum of column j's
        iterator entries in row i (zero when absent)."""
        if not 0 <= i < self.dimension:
            raise BoundsError(f"index {i} out of range for dimension {self.dimension}")
        rows, vals = self._line(j, True, 0.0)
        hit = np.nonzero(rows == i)[0]
        return complex(vals[hit[0]]) if hit.size else 0j

    def __getitem__(self, key):
        """opr[i, :], opr[:, j], opr[:, :] and opr[i, j] (abstract_operator_representation.jl:231-250)."""
        import scipy.sparse as sps
        i, j = key
        full = slice(None)
        n = self.dimension
        if isinstance(i, slice) and i == full and isinstance(j, slice) and j == full:
            return self.sparse()
        if isinstance(j, slice) and j == full:
            cols, vals = self.get_row(int(i))
            return sps.csr_matrix((vals, cols, [0, cols.size]), shape=(1, n))
        if isinstance(i, slice) and i == full:
            rows, vals = self.get_column(int(j))
            return sps.csr_matrix((vals, rows, [0, rows.size]), shape=(1, n)).T
        return self.get_element(int(i), int(j))

    def lanczos(self, *args, **kwargs):
        from .lanczos import lanczos
        return lanczos(self, *args, **kwargs)


def _check_len(v, n, what):
    if len(v) != n:
        raise DimensionMismatch(f"{what} has length {len(v)} != dimension {n}")


def _host_c128(v, writable=False):
    a = np.asarray(v)
    if a.dtype != np.complex128 or not a.flags.c_contiguous:
        if writable:
            raise ArgumentError("out must be a contiguous complex128 array")
        a = np.ascontiguousarray(a, dtype=np.complex128)
    return a


def _product(out, opr, state, accumulate, precision, transpose=False):
    prec = _prec(precision)
    n = opr.dimension
    _check_len(out, n, "out")
    _check_len(state, n, "state")
    if _is_torch(out) or _is_torch(state):
        import torch
        if transpose:
            raise ArgumentError("the transpose product takes host vectors")
        want = torch.complex128 if prec == FP64 else torch.complex64
        for t, nm in ((out, "out"), (state, "state")):
            if not (_is_torch(t) and t.is_cuda and t.dtype == want and t.is_contiguous()):
                raise ArgumentError(f"{nm} must be a contiguous CUDA tensor of {want}")
        check(lib().edgpu_mul_device(opr.handle, prec, ctypes.c_void_p(state.data_ptr()),
                                     ctypes.c_void_p(out.data_ptr()), n, int(accumulate), _torch_stream()))
        return out
    x = _host_c128(state)
    y = _host_c128(out, writable=True)
    fn = lib().edgpu_mul_transpose if transpose else lib().edgpu_mul
    check(fn(opr.handle, prec, ptr(x.view(np.float64), ctypes.c_double), ptr(y.view(np.float64), ctypes.c_double),
             n, int(accumulate)))
    return out


def mul_(out, opr, state, precision="fp64"):
    """LinearAlgebra.mul!(out, opr, state): out = opr * state (abstract_operator_representation.jl:110-118)."""
    return _product(out, opr, state, False, precision)


def apply_(out, a, b, precision="fp64"):
    """apply!(out, opr, state): out += opr * state; apply!(out, state, opr): out += transpose(state) * opr
    (abstract_operator_representation.jl:260-285)."""
    if isinstance(a, OperatorRepresentation):
        return _product(out, a, b, True, precision)
    if isinstance(b, OperatorRepresentation):
        return _product(out, b, a, True, precision, transpose=True)
    raise ArgumentError("apply_ needs an OperatorRepresentation")


apply_serial_ = apply_
apply_parallel_ = apply_


def mul_adjoint_(out, opr, state, precision="fp64", accumulate=False):
    """out = opr^dagger * state on CUDA tensors (the adjoint product dL/dx = H^dagger gy)."""
    prec = _prec(precision)
    n = opr.dimension
    _check_len(out, n, "out")
    _check_len(state, n, "state")
    check(lib().edgpu_mul_adjoint_device(opr.handle, prec, ctypes.c_void_p(state.data_ptr()),
                                         ctypes.c_void_p(out.data_ptr()), n, int(accumulate), _torch_stream()))
    return out


def coupling_grad(opr, x, gy, precision="fp64", y=None) -> np.ndarray:
    """dL/dJ_c = Re <gy | H_c x> for every coupling (CUDA tensors); fills y = H x when given."""
    prec = _prec(precision)
    n = opr.dimension
    _check_len(x, n, "x")
    _check_len(gy, n, "gy")
    g = np.empty(opr.n_couplings, dtype=np.float64)
    check(lib().edgpu_coupling_grad_device(opr.handle, prec, ctypes.c_void_p(x.data_ptr()),
                                           ctypes.c_void_p(gy.data_ptr()),
                                           ctypes.c_void_p(y.data_ptr()) if y is not None else None, n,
                                           ptr(g, ctypes.c_double), _torch_stream()))
    return g


class Batch:
    """Several operator representations (every momentum sector of one Hamiltonian) applied in one
    persistent launch, optionally replayed from a captured CUDA graph.  The representations must
    share the operator terms, the basis layout and the symmetry group; each sector's result equals
    ``mul_`` on that sector with the same lanes per row."""

    def __init__(self, oprs: Sequence[OperatorRepresentation]):
        self.oprs = list(oprs)
        arr = (ctypes.c_void_p * len(self.oprs))(*[o.handle for o in self.oprs])
        h = ctypes.c_void_p()
        check(lib().edgpu_batch_create(len(self.oprs), arr, ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.edgpu_batch_destroy(h)
            self._h = None

    def set_tiling(self, precision, lanes_per_row: int):
        """Lanes per row of the batched launch: 0 (default, 1), 1, 2 or 4."""
        check(lib().edgpu_batch_set_tiling(self._h, _prec(precision), int(lanes_per_row)))

    def schedule(self, precision="mixed"):
        """(lanes per row, pair flips as in OperatorRepresentation.schedule) of the batched launch."""
        a, b = ctypes.c_int32(), ctypes.c_int32()
        check(lib().edgpu_batch_get_schedule(self._h, _prec(precision), ctypes.byref(a), ctypes.byref(b), None))
        return int(a.value), int(b.value)

    def uses_target_tables(self, precision="mixed") -> bool:
        t = ctypes.c_int32()
        check(lib().edgpu_batch_get_schedule(self._h, _prec(precision), None, None, ctypes.byref(t)))
        return bool(t.value)

    def set_launch(self, precision, streams: int):
        """0: all sectors in one persistent launch; 1: one product launch per sector on the call's
        stream; 2 or 3: per-sector launches spread over that many concurrent streams; 5 to 7: the
        same on 1 to 3 streams with each operator's own (autotuned) schedule."""
        check(lib().edgpu_batch_set_launch(self._h, _prec(precision), int(streams)))

    def launch(self, precision="mixed") -> int:
        """The launch mode (see set_launch)."""
        k = ctypes.c_int32()
        check(lib().edgpu_batch_get_launch(self._h, _prec(precision), ctypes.byref(k)))
        return int(k.value)

    def autotune(self, precision="mixed"):
        """Time 1, 2 and 4 lanes per row, with and without the pair-flip schedule, and per-sector
        launches on 1 to 3 streams, and keep the fastest; returns (lanes_per_row, ms)."""
        l = ctypes.c_int32()
        ms = ctypes.c_double()
        check(lib().edgpu_batch_autotune(self._h, _prec(precision), ctypes.byref(l), ctypes.byref(ms)))
        return l.value, ms.value

    def mul_(self, outs, states, precision="mixed", use_graph=True):
        prec = _prec(precision)
        if len(outs) != len(self.oprs) or len(states) != len(self.oprs):
            raise ArgumentError(f"expected {len(self.oprs)} vectors, got {len(states)} and {len(outs)}")
        for o, x, y in zip(self.oprs, states, outs):
            _check_len(x, o.dimension, "x")
            _check_len(y, o.dimension, "y")
        xs = (ctypes.c_void_p * len(states))(*[s.data_ptr() for s in states])
        ys = (ctypes.c_void_p * len(outs))(*[o.data_ptr() for o in outs])
        check(lib().edgpu_batch_mul_device(self._h, prec, xs, ys, int(use_graph), _torch_stream()))
        return outs


def random_state(n: int, seed: int, precision="fp64", device=True):
    """Seeded complex Gaussian vector ((g1 + i g2)/sqrt(2), SplitMix64 + Box-Muller, normalised)
    generated on the GPU into a new torch CUDA tensor."""
    import torch
    prec = _prec(precision)
    t = torch.empty(n, dtype=torch.complex128 if prec == FP64 else torch.complex64, device="cuda")
    check(lib().edgpu_random_vector_device(n, seed, prec, ctypes.c_void_p(t.data_ptr()), _torch_stream()))
    return t
