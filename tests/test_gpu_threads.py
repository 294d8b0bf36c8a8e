"""Concurrent products from several host threads on two operator handles (one of them through the
multi-pass slab product).

Calls on one handle are serialised by the handle's lock; distinct handles run concurrently, each on
its own stream (host-buffer calls) or on the caller's stream (device-buffer calls).  Four threads,
two per handle, issue host-buffer products (FP64 and mixed precision) and device-buffer products on
their own torch streams; every result must equal the serial result bit for bit (the products have a
fixed summation order)."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _operator(L, k):
    import edgpu
    from edgpu import lattice
    hs, _ = edgpu.spin_half_system(L)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0))
    rhsr = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, k))
    bonds = lattice.chain_bonds(L) + [(i, (i + 2) % L) for i in range(L)]
    H = lattice.xxz_hamiltonian(hs, bonds, [1.0] * L + [0.4] * L, [0.8] * L + [0.3] * L)
    return edgpu.represent(rhsr, H)


def test_two_handles_from_four_threads_equal_serial():
    import torch
    import edgpu
    from oracle import oracle as O
    ops = [_operator(20, 0), _operator(18, 5)]
    # the first operator runs the multi-pass slab product (small slabs: several launches per product)
    assert ops[0].build_targets(1 << 28) and ops[0].build_slabs(slab_bytes=1024 * 8, max_bytes=1 << 28)
    assert ops[0].slabs_info[0] >= 3
    xs = [O.complex_gaussian(o.dimension, 3 + i) for i, o in enumerate(ops)]
    ref = {}
    for i, o in enumerate(ops):
        for prec in ("fp64", "mixed"):
            y = np.zeros_like(xs[i])
            edgpu.mul_(y, o, xs[i], precision=prec)
            ref[(i, prec, "host")] = y
            dt = torch.complex128 if prec == "fp64" else torch.complex64
            xd = torch.from_numpy(xs[i]).to(dt).cuda()
            yd = torch.empty_like(xd)
            edgpu.mul_(yd, o, xd, precision=prec)
            torch.cuda.synchronize()
            ref[(i, prec, "dev")] = yd.cpu().numpy()
    errors = []
    barrier = threading.Barrier(4)

    def worker(t):
        try:
            i = t % 2
            o = ops[i]
            stream = torch.cuda.Stream()
            barrier.wait()
            for it in range(12):
                prec = "fp64" if (it + t) % 2 == 0 else "mixed"
                y = np.zeros_like(xs[i])
                edgpu.mul_(y, o, xs[i], precision=prec)
                assert np.array_equal(y, ref[(i, prec, "host")]), ("host", t, it, prec)
                dt = torch.complex128 if prec == "fp64" else torch.complex64
                with torch.cuda.stream(stream):
                    xd = torch.from_numpy(xs[i]).to(dt).to("cuda", non_blocking=False)
                    yd = torch.empty_like(xd)
                    edgpu.mul_(yd, o, xd, precision=prec)
                stream.synchronize()
                assert np.array_equal(yd.cpu().numpy(), ref[(i, prec, "dev")]), ("device", t, it, prec)
        except Exception as e:   # noqa: BLE001  (reported below)
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
