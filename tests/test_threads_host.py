"""Concurrent calls from several host threads, without a GPU.

Calls on distinct handles may run concurrently; each thread has its own error slot
(edgpu_last_error).  Here several threads drive the library's host-only entry point
(edgpu_pair_classes_of_terms, the bond-class builder of the pair-flip schedule) and failing calls
with thread-specific arguments at the same time; every thread must see its own results and its own
error messages, identical to a serial run.  ctypes releases the GIL during foreign calls, so the
calls really overlap."""
import ctypes
import threading

import numpy as np

import edgpu
from edgpu import _lib, lattice


def _classes(n):
    hs, _ = edgpu.spin_half_system(n)
    bonds = [(i, (i + 1) % n) for i in range(n)] + [(i, (i + 2) % n) for i in range(n)]
    H = lattice.xxz_hamiltonian(hs, bonds, [1.0] * n + [0.5] * n, [0.7] * n + [0.35] * n)
    m, r, c, a = edgpu.term_arrays(H)
    a = np.ascontiguousarray(a.astype(np.complex128)).view(np.float64)
    L = _lib.lib()
    ncls = ctypes.c_int32(0)
    cap = 32
    info = np.zeros(cap, dtype=np.int32)
    comps = np.zeros(cap * 4 * 3, dtype=np.uint64)
    flips = np.zeros(cap * n, dtype=np.uint64)
    amps = np.zeros(cap * n * 4 * 2, dtype=np.float64)
    st = L.edgpu_pair_classes_of_terms(n, len(m), _lib.ptr(m, ctypes.c_uint64), _lib.ptr(r, ctypes.c_uint64),
                                       _lib.ptr(c, ctypes.c_uint64), _lib.ptr(a, ctypes.c_double), cap,
                                       ctypes.byref(ncls), _lib.ptr(info, ctypes.c_int32),
                                       _lib.ptr(comps, ctypes.c_uint64), _lib.ptr(flips, ctypes.c_uint64),
                                       _lib.ptr(amps, ctypes.c_double))
    _lib.check(st)
    k = ncls.value
    return k, info[:k].copy(), comps[:k * 12].copy(), flips[:k * n].copy(), amps[:k * n * 8].copy()


def _failing_call(tag):
    """A call that fails argument validation with a message naming this thread's value."""
    L = _lib.lib()
    ncls = ctypes.c_int32(0)
    # n_bits = tag is out of range (> 64) -> ArgumentError with the value in the message, no device work
    st = L.edgpu_pair_classes_of_terms(tag, 0, None, None, None, None, 0, ctypes.byref(ncls), None, None, None, None)
    return st, L.edgpu_last_error().decode()


def test_concurrent_host_calls_match_serial():
    sizes = [8, 10, 12, 14, 16, 20, 24, 28]
    serial = {n: _classes(n) for n in sizes}
    serial_err = {t: _failing_call(t) for t in range(100, 108)}
    assert all(st == _lib.ERR_ARG for st, _ in serial_err.values())
    assert len({msg for _, msg in serial_err.values()}) == len(serial_err), "messages must name the argument"
    errors = []
    barrier = threading.Barrier(len(sizes))

    def worker(i, n):
        try:
            barrier.wait()
            for _ in range(20):
                got = _classes(n)
                ref = serial[n]
                assert got[0] == ref[0]
                for g, r in zip(got[1:], ref[1:]):
                    assert np.array_equal(g, r)
                t = 100 + i
                st, msg = _failing_call(t)
                assert (st, msg) == serial_err[t], (st, msg, serial_err[t])
        except Exception as e:   # noqa: BLE001  (reported below)
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(i, n)) for i, n in enumerate(sizes)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
