"""ctypes binding of libedgpu.so and the mapping of its status codes to the reference's exceptions.

The library is built in-tree (csrc/build.py) next to this file.  Loading it never touches the GPU;
any call that needs one fails with CudaError when no device is present.  There is no CPU fallback:
if the library is missing, importing the package raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# EDGPU_LIBRARY selects another build of the library (e.g. one with different tile constants).
LIB_PATH = os.environ.get("EDGPU_LIBRARY") or os.path.join(HERE, "libedgpu.so")

OK, ERR_ARG, ERR_DIM, ERR_BOUNDS, ERR_KEY, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_STATE = range(9)
FP64, MIXED = 0, 1
SPACE_LAZY = 1
PAIR_UNIFORM = 16   # EDGPU_PAIR_UNIFORM: warp-uniform pair steps of the target-table product


class ArgumentError(ValueError):
    """ArgumentError of the reference (bad masks, non-unit amplitudes, word type too small)."""


class DimensionMismatch(ValueError):
    """DimensionMismatch of the reference (vector lengths)."""


class BoundsError(IndexError):
    """BoundsError of the reference (row/column index out of range)."""


class CudaError(RuntimeError):
    """A CUDA runtime failure (including: no device)."""


class EdgpuTimeout(RuntimeError):
    """A bounded device-side wait ran out."""


_EXC = {ERR_ARG: ArgumentError, ERR_DIM: DimensionMismatch, ERR_BOUNDS: BoundsError, ERR_KEY: KeyError,
        ERR_OOM: MemoryError, ERR_CUDA: CudaError, ERR_TIMEOUT: EdgpuTimeout, ERR_STATE: RuntimeError}

_lib = None

i32, i64, u64, dbl = ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double
P = ctypes.POINTER
vp = ctypes.c_void_p

SIGNATURES = {
    "edgpu_last_error": (ctypes.c_char_p, []),
    "edgpu_version": (ctypes.c_char_p, []),
    "edgpu_device_count": (ctypes.c_int, [P(i32)]),
    "edgpu_space_create": (ctypes.c_int, [i32, P(i32), i32, P(i64), i32, P(i64), i32, P(vp)]),
    "edgpu_space_from_basis": (ctypes.c_int, [i32, P(i32), P(u64), i64, P(vp)]),
    "edgpu_space_dim": (ctypes.c_int, [vp, P(i64)]),
    "edgpu_space_nbits": (ctypes.c_int, [vp, P(i32)]),
    "edgpu_space_get_basis": (ctypes.c_int, [vp, P(u64), i64]),
    "edgpu_space_lookup": (ctypes.c_int, [vp, P(u64), i64, P(i64)]),
    "edgpu_space_destroy": (None, [vp]),
    "edgpu_space_search_stats": (ctypes.c_int, [vp, P(i64), P(i32), P(i32), P(i32), P(dbl)]),
    "edgpu_space_build_map": (ctypes.c_int, [vp, i64, P(i32)]),
    "edgpu_space_free_map": (ctypes.c_int, [vp]),
    "edgpu_space_map_info": (ctypes.c_int, [vp, P(i64), P(i32)]),
    "edgpu_reduce": (ctypes.c_int, [vp, i32, P(i32), P(u64), P(i32), i32, P(vp)]),
    "edgpu_reduce_mapping": (ctypes.c_int, [vp, P(i64), P(dbl), i64]),
    "edgpu_space_orbit_sizes": (ctypes.c_int, [vp, P(i32), i64]),
    "edgpu_space_parent_dim": (ctypes.c_int, [vp, P(i64)]),
    "edgpu_symmetry_unreduce_device": (ctypes.c_int, [vp, i32, vp, i64, vp, i64, vp]),
    "edgpu_symmetry_reduce_device": (ctypes.c_int, [vp, i32, vp, i64, vp, i64, vp]),
    "edgpu_op_create": (ctypes.c_int, [vp, i32, P(u64), P(u64), P(u64), P(dbl), P(i32), i32, P(dbl), P(vp)]),
    "edgpu_op_set_couplings": (ctypes.c_int, [vp, P(dbl), i32]),
    "edgpu_op_dim": (ctypes.c_int, [vp, P(i64)]),
    "edgpu_op_destroy": (None, [vp]),
    "edgpu_op_set_tiling": (ctypes.c_int, [vp, i32, i32]),
    "edgpu_op_autotune": (ctypes.c_int, [vp, i32, P(i32), P(dbl)]),
    "edgpu_op_set_pair_schedule": (ctypes.c_int, [vp, i32]),
    "edgpu_op_pair_classes": (ctypes.c_int, [vp, P(i32), P(i32)]),
    "edgpu_pair_classes_of_terms": (ctypes.c_int, [i32, i32, P(u64), P(u64), P(u64), P(dbl), i32, P(i32), P(i32),
                                                   P(u64), P(u64), P(dbl)]),
    "edgpu_op_get_schedule": (ctypes.c_int, [vp, i32, P(i32), P(i32), P(i32)]),
    "edgpu_op_build_targets": (ctypes.c_int, [vp, i64, P(i32)]),
    "edgpu_op_free_targets": (ctypes.c_int, [vp]),
    "edgpu_op_targets_info": (ctypes.c_int, [vp, P(i64), P(i32)]),
    "edgpu_op_build_slabs": (ctypes.c_int, [vp, i64, i64, P(i32)]),
    "edgpu_op_free_slabs": (ctypes.c_int, [vp]),
    "edgpu_op_slabs_info": (ctypes.c_int, [vp, P(i32), P(i64), P(i64)]),
    "edgpu_op_slab_use": (ctypes.c_int, [vp, i32, i32, P(i32)]),
    "edgpu_op_slab_scaling": (ctypes.c_int, [vp, i32, P(i32)]),
    "edgpu_op_build_adjoint_targets": (ctypes.c_int, [vp, i64, P(i32)]),
    "edgpu_op_table_prefetch": (ctypes.c_int, [vp, i32, i32, P(i32)]),
    "edgpu_op_grad_kernel": (ctypes.c_int, [vp, i32, P(i32)]),
    "edgpu_op_free_adjoint_targets": (ctypes.c_int, [vp]),
    "edgpu_batch_get_schedule": (ctypes.c_int, [vp, i32, P(i32), P(i32), P(i32)]),
    "edgpu_op_sparse": (ctypes.c_int, [vp, i32, dbl, P(i64), P(i64), P(i64), P(dbl)]),
    "edgpu_op_get_row": (ctypes.c_int, [vp, i32, i64, dbl, i64, P(i64), P(i64), P(dbl)]),
    "edgpu_op_is_invariant": (ctypes.c_int, [vp, P(i32)]),
    "edgpu_op_count_nnz": (ctypes.c_int, [vp, P(i64), P(i64)]),
    "edgpu_mul": (ctypes.c_int, [vp, i32, P(dbl), P(dbl), i64, i32]),
    "edgpu_mul_device": (ctypes.c_int, [vp, i32, vp, vp, i64, i32, vp]),
    "edgpu_mul_transpose": (ctypes.c_int, [vp, i32, P(dbl), P(dbl), i64, i32]),
    "edgpu_mul_adjoint_device": (ctypes.c_int, [vp, i32, vp, vp, i64, i32, vp]),
    "edgpu_coupling_grad_device": (ctypes.c_int, [vp, i32, vp, vp, vp, i64, P(dbl), vp]),
    "edgpu_coupling_grad_device_noalloc": (ctypes.c_int, [vp, i32, vp, vp, vp, i64, P(dbl), vp]),
    "edgpu_batch_create": (ctypes.c_int, [i32, P(vp), P(vp)]),
    "edgpu_batch_set_tiling": (ctypes.c_int, [vp, i32, i32]),
    "edgpu_batch_autotune": (ctypes.c_int, [vp, i32, P(i32), P(ctypes.c_double)]),
    "edgpu_batch_set_launch": (ctypes.c_int, [vp, i32, i32]),
    "edgpu_batch_get_launch": (ctypes.c_int, [vp, i32, P(i32)]),
    "edgpu_batch_mul_device": (ctypes.c_int, [vp, i32, P(vp), P(vp), i32, vp]),
    "edgpu_batch_destroy": (None, [vp]),
    "edgpu_lanczos": (ctypes.c_int, [vp, i32, i32, i32, u64, P(dbl), i32, dbl, P(dbl), P(dbl), P(dbl), P(i32),
                                     P(dbl)]),
    "edgpu_set_krylov_limit": (ctypes.c_int, [ctypes.c_int64]),
    "edgpu_random_vector_device": (ctypes.c_int, [i64, u64, i32, vp, vp]),
    "edgpu_sync": (ctypes.c_int, []),
    "edgpu_host_alloc": (ctypes.c_int, [i64, P(vp)]),
    "edgpu_host_free": (None, [vp]),
}


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libedgpu.so is not built ({LIB_PATH}); run "
                              "`python -c 'import __graft_entry__ as g; g.build()'` at the repository root")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int):
    if status != OK:
        msg = lib().edgpu_last_error().decode(errors="replace")
        raise _EXC.get(status, RuntimeError)(msg)


def device_count() -> int:
    n = i32(0)
    check(lib().edgpu_device_count(ctypes.byref(n)))
    return int(n.value)


def ptr(a, ctype):
    """ctypes pointer to a contiguous numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(P(ctype))
