"""Lanczos driver for the lowest eigenvalue, on the GPU (no counterpart in the reference, which uses
dense eigvals or an external Arpack.eigs that calls mul! repeatedly, docs/src/examples/spinhalf.md:26).

FP64 throughout for the scalars, dot products, norms, reorthogonalisation and the tridiagonal
eigensolve; `precision` selects the product (fp64, or mixed: complex64 vectors and FP32
accumulation).  tol > 0 stops a run once the lowest Ritz value moved by less than tol |E| over five
steps or (when no vector is wanted, from step 10 on) once the Kato-Temple estimate of its error from
the tridiagonal matrix, (beta s_last)^2 / (theta_2 - theta_1), is below tol max(1, |E|).  With
refine=True (mixed precision) the mixed-precision run goes on until that estimate is below tol / 4,
or for 6 steps after its lowest Ritz value settled to max(tol, 1e-9); then one FP64 product gives
the Rayleigh quotient E_RQ = <psi|H psi> of its Ritz vector psi and the residual r = H psi - E_RQ psi;
E_RQ is returned when the Kato-Temple estimate |r|^2 / (theta_2 - E_RQ) (theta_2: the second Ritz
value of the mixed run) is below tol max(1, |E_RQ|), else FP64 Lanczos restarts from psi until the
eigenvalue settles to tol or the estimate certifies it.  The Krylov basis is kept only
when reorthogonalisation or a Ritz vector needs it and it fits (see set_krylov_limit): in FP64 for an
FP64 run, as the complex64 product inputs for a mixed run (reorthogonalisation then uses those
complex64-rounded vectors with FP64 arithmetic); otherwise a Ritz vector is rebuilt by a second pass of
the recurrence.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np

from ._lib import check, lib, ptr
from .representation import OperatorRepresentation, _prec


@dataclass
class LanczosResult:
    e0: float
    alphas: np.ndarray
    betas: np.ndarray
    steps: int
    ground_state: Optional[np.ndarray] = None


def lanczos(opr: OperatorRepresentation, n_steps: int = 200, precision="fp64", reorth: bool = True, seed: int = 1,
            v0=None, refine: bool = False, tol: float = 1e-12, want_vector: bool = False) -> LanczosResult:
    prec = _prec(precision)
    e0 = ctypes.c_double()
    al = np.zeros(n_steps, dtype=np.float64)
    be = np.zeros(n_steps, dtype=np.float64)
    done = ctypes.c_int32()
    v = None if v0 is None else np.ascontiguousarray(v0, dtype=np.complex128)
    gs = np.empty(opr.dimension, dtype=np.complex128) if want_vector else None
    check(lib().edgpu_lanczos(opr.handle, prec, int(n_steps), int(bool(reorth)), int(seed),
                              ptr(v.view(np.float64), ctypes.c_double) if v is not None else None,
                              int(bool(refine)), float(tol), ctypes.byref(e0), ptr(al, ctypes.c_double),
                              ptr(be, ctypes.c_double), ctypes.byref(done),
                              ptr(gs.view(np.float64), ctypes.c_double) if gs is not None else None))
    return LanczosResult(float(e0.value), al, be, int(done.value), gs)


def set_krylov_limit(nbytes: int) -> None:
    """Largest Krylov basis (bytes) the Lanczos driver stores; 0 restores the default (half of the free
    device memory).  Below it, Ritz vectors are rebuilt by a second pass of the recurrence.  The
    complex64 basis of a refined mixed-precision run is also held to the device memory left after the
    run's other buffers, less 2 GiB."""
    check(lib().edgpu_set_krylov_limit(int(nbytes)))
