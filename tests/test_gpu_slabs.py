"""The column-slab table and its multi-pass mixed-precision product (edgpu_op_build_slabs).

Small slabs force several passes on sectors the oracle handles in seconds: the product must match the
oracle's reduced product within 1e-5 (mixed precision) and the one-pass target-table product within
1e-6, be reproducible bit for bit, accumulate (y += H x), write complex128 host buffers, follow new
coupling values, and cover real and complex coefficients (momentum 0 and k != 0), a torus and a
chain; the FP64 product through the same table must match the oracle within 1e-12.  Both table
layouts: coefficients with the orbit-size ratio, and the scaled layout (ratio applied to x and to the
result rows)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _chain(E, L, k, coupled):
    from edgpu import lattice
    hs, _ = E.spin_half_system(L)
    hsr = E.represent(E.HilbertSpaceSector(hs, 0))
    rh = E.symmetry_reduce(hsr, E.translation_symops(L, k))
    sites = O.spin_half_sites(L)
    parent = O.hs_get_basis_list(sites, [(0,)])
    bw, off = O.bit_layout(sites)
    maps, amps = O.translation_symops((L, 1), (k, 0))
    red = O.symmetry_reduce(parent, bw, off, maps, amps)
    if coupled:
        m, r, c, a, ids = lattice.heisenberg_coupled(hs, lattice.chain_bonds(L))
        J = 0.5 + np.random.default_rng(3).random(L)
        opr = E.OperatorRepresentation.from_terms(rh, m, r, c, a, coupling_ids=ids, couplings=J)
        terms = [(int(m[t]), int(r[t]), int(c[t]), complex(a[t]) * J[ids[t]]) for t in range(len(m))]
        return opr, red, terms, (m, r, c, a, ids, J)
    bonds = lattice.chain_bonds(L) + [(i, (i + 2) % L) for i in range(L)]
    jxy, jz = [1.0] * L + [0.4] * L, [0.8] * L + [0.3] * L
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    return E.represent(rh, H), red, O.heisenberg_terms(L, bonds, jxy, jz), None


def _products(E, opr, x):
    import torch
    xd = torch.from_numpy(x).to(torch.complex64).cuda()
    y = torch.empty_like(xd)
    E.mul_(y, opr, xd, precision="mixed")
    torch.cuda.synchronize()
    return xd, y


@pytest.mark.parametrize("scaling", [1, 2])
@pytest.mark.parametrize("L,k,coupled", [(20, 0, False), (18, 5, False), (20, 0, True)])
def test_slab_product_chain(L, k, coupled, scaling):
    """scaling 1: coefficients with the orbit-size ratio; 2: the scaled layout (x scaled slab by slab on
    the handle's second stream, rows in the last pass), whose coefficients sit in registers (k = 0,
    two couplings), in a copy per shared-memory bank group (k = 5, complex) or in one shared-memory
    copy (per-bond couplings)."""
    import torch
    import edgpu as E
    opr, red, terms, extra = _chain(E, L, k, coupled)
    N = opr.dimension
    assert opr.build_targets(1 << 30)
    x = O.complex_gaussian(N, 7)
    want = O.apply_rows(red, terms, x)
    xd, y_tab = _products(E, opr, x)
    # slabs of 1024 columns: several passes
    assert not opr.slab_scaling(scaling)
    assert opr.build_slabs(slab_bytes=1024 * 8, max_bytes=1 << 30)
    assert opr.slab_scaling() == (scaling == 2)
    passes, wc, entries = opr.slabs_info
    assert wc == 1024 and passes == (N + 1023) // 1024 and passes >= 3
    assert 0 < entries <= opr.targets_info[0]   # the targets with a representative
    assert opr.slab_use("mixed")
    y = torch.empty_like(xd)
    E.mul_(y, opr, xd, precision="mixed")
    y2 = torch.full_like(xd, float("nan"))
    E.mul_(y2, opr, xd, precision="mixed")
    torch.cuda.synchronize()
    assert torch.equal(y, y2)
    # the other variants (cache hints, eight entries per step): the same arithmetic in the same order
    for mode in (2, 3, 4):
        assert opr.slab_use("mixed", mode) == mode
        y2.fill_(float("nan"))
        E.mul_(y2, opr, xd, precision="mixed")
        torch.cuda.synchronize()
        assert torch.equal(y, y2), mode
    # two and four lanes per row: another fixed order of the sums, deterministic, equal within rounding
    for mode in (5, 6):
        assert opr.slab_use("mixed", mode) == mode
        y2.fill_(float("nan"))
        E.mul_(y2, opr, xd, precision="mixed")
        y2b = torch.full_like(xd, float("nan"))
        E.mul_(y2b, opr, xd, precision="mixed")
        torch.cuda.synchronize()
        assert torch.equal(y2, y2b), mode
        assert relerr(y2.cpu().numpy().astype(np.complex128), want) < 1e-5, mode
        yh5 = np.zeros(N, dtype=np.complex128)
        E.mul_(yh5, opr, x, precision="mixed")
        assert relerr(yh5, want) < 1e-5, mode
    assert opr.slab_use("mixed", 1) == 1
    yn = y.cpu().numpy().astype(np.complex128)
    assert relerr(yn, want) < 1e-5
    assert relerr(yn, y_tab.cpu().numpy().astype(np.complex128)) < 1e-6
    # y += H x
    y3 = y.clone()
    E.apply_(y3, opr, xd, precision="mixed")
    torch.cuda.synchronize()
    assert relerr(y3.cpu().numpy().astype(np.complex128), 2 * want) < 1e-5
    # complex128 host buffers (the last pass writes complex128)
    yh = np.zeros(N, dtype=np.complex128)
    E.mul_(yh, opr, x, precision="mixed")
    assert relerr(yh, want) < 1e-5
    yh2 = yh.copy()
    E.apply_(yh2, opr, x, precision="mixed")
    assert relerr(yh2, 2 * want) < 1e-5
    # FP64 products read it too: device vectors, pageable and pinned host buffers (the last pass
    # writes the pinned buffer), y += H x
    assert opr.slab_use("fp64")
    x64 = torch.from_numpy(x).cuda()
    yd64 = torch.empty_like(x64)
    E.mul_(yd64, opr, x64, precision="fp64")
    torch.cuda.synchronize()
    assert relerr(yd64.cpu().numpy(), want) < 1e-12
    for mode in (2, 3, 4):
        opr.slab_use("fp64", mode)
        yd64b = torch.full_like(x64, float("nan"))
        E.mul_(yd64b, opr, x64, precision="fp64")
        torch.cuda.synchronize()
        assert torch.equal(yd64, yd64b), mode
    for mode in (5, 6):
        opr.slab_use("fp64", mode)
        yd64b = torch.full_like(x64, float("nan"))
        E.mul_(yd64b, opr, x64, precision="fp64")
        torch.cuda.synchronize()
        assert relerr(yd64b.cpu().numpy(), want) < 1e-12, mode
    opr.slab_use("fp64", 1)
    yf = np.zeros(N, dtype=np.complex128)
    E.mul_(yf, opr, x, precision="fp64")
    assert relerr(yf, want) < 1e-12
    xp = torch.from_numpy(x).pin_memory()
    yp = torch.zeros(N, dtype=torch.complex128).pin_memory()
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-5)):
        yp.zero_()
        E.mul_(yp.numpy(), opr, xp.numpy(), precision=prec)
        assert relerr(yp.numpy(), want) < tol
        E.apply_(yp.numpy(), opr, xp.numpy(), precision=prec)
        assert relerr(yp.numpy(), 2 * want) < tol
    if coupled:
        m, r, c, a, ids, J = extra
        J2 = J[::-1] * 1.3
        opr.set_couplings(J2)
        terms2 = [(int(m[t]), int(r[t]), int(c[t]), complex(a[t]) * J2[ids[t]]) for t in range(len(m))]
        _, y4 = _products(E, opr, x)
        assert relerr(y4.cpu().numpy().astype(np.complex128), O.apply_rows(red, terms2, x)) < 1e-5
    # switched off: the one-pass product again, bit for bit
    assert not opr.slab_use("mixed", False)
    assert not opr.slab_use("fp64", False)
    if not coupled:
        _, y5 = _products(E, opr, x)
        assert torch.equal(y5, y_tab)
    # the autotuner times the slab product among the others
    opr.autotune("mixed")
    _, y6 = _products(E, opr, x)
    assert relerr(y6.cpu().numpy().astype(np.complex128), want if not coupled else
                  O.apply_rows(red, terms2, x)) < 1e-5
    opr.free_slabs()
    assert opr.slabs_info == (0, 0, 0)
    with pytest.raises(RuntimeError):
        opr.slab_use("mixed", True)


def test_slab_product_torus_j1j2():
    import torch
    import edgpu as E
    from edgpu import lattice
    shape = (6, 3)
    n = shape[0] * shape[1]
    hs, _ = E.spin_half_system(n)
    nn = lattice.torus_bonds(*shape, [(1, 0), (0, 1)])
    nnn = lattice.torus_bonds(*shape, [(1, 1), (1, -1)])
    jj = [1.0] * len(nn) + [0.5] * len(nnn)
    H = lattice.xxz_hamiltonian(hs, nn + nnn, jj, jj)
    terms = O.heisenberg_terms(n, nn + nnn, jj, jj)
    sites = O.spin_half_sites(n)
    parent = O.hs_get_basis_list(sites, [(0,)])
    bw, off = O.bit_layout(sites)
    for k in ((0, 0), (1, 1)):
        hsr = E.represent(E.HilbertSpaceSector(hs, 0))
        opr = E.represent(E.symmetry_reduce(hsr, E.translation_symops(shape, k)), H)
        maps, amps = O.translation_symops(shape, k)
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        N = opr.dimension
        assert opr.build_targets(1 << 30)
        opr.slab_scaling(2 if k == (1, 1) else 0)
        assert opr.build_slabs(slab_bytes=1024 * 8, max_bytes=1 << 30)
        assert opr.slabs_info[0] >= 3 and opr.slab_scaling() == (k == (1, 1))
        x = O.complex_gaussian(N, 9)
        want = O.apply_rows(red, terms, x)
        _, y = _products(E, opr, x)
        assert relerr(y.cpu().numpy().astype(np.complex128), want) < 1e-5
        y64 = np.zeros(N, dtype=np.complex128)
        E.mul_(y64, opr, x, precision="fp64")
        assert relerr(y64, want) < 1e-12


@pytest.mark.parametrize("k", [0, 3])
def test_slab_product_scaled_one_pass(k):
    """A scaled table of one pass (x scaled on the calling stream before the pass): device vectors,
    y += H x, pinned and pageable host buffers in both precisions, against the oracle."""
    import torch
    import edgpu as E
    opr, red, terms, _ = _chain(E, 16, k, False)
    N = opr.dimension
    assert opr.build_targets(1 << 30)
    opr.slab_scaling(2)
    assert opr.build_slabs(slab_bytes=1 << 20, max_bytes=1 << 30)
    assert opr.slab_scaling() and opr.slabs_info[0] == 1
    x = O.complex_gaussian(N, 4)
    want = O.apply_rows(red, terms, x)
    xd, y = _products(E, opr, x)
    assert relerr(y.cpu().numpy().astype(np.complex128), want) < 1e-5
    y2 = y.clone()
    E.apply_(y2, opr, xd, precision="mixed")
    torch.cuda.synchronize()
    assert relerr(y2.cpu().numpy().astype(np.complex128), 2 * want) < 1e-5
    x64 = torch.from_numpy(x).cuda()
    y64 = torch.empty_like(x64)
    E.mul_(y64, opr, x64, precision="fp64")
    torch.cuda.synchronize()
    assert relerr(y64.cpu().numpy(), want) < 1e-12
    E.apply_(y64, opr, x64, precision="fp64")
    torch.cuda.synchronize()
    assert relerr(y64.cpu().numpy(), 2 * want) < 1e-12
    xp = torch.from_numpy(x).pin_memory()
    yp = torch.zeros(N, dtype=torch.complex128).pin_memory()
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-5)):
        yp.zero_()
        E.mul_(yp.numpy(), opr, xp.numpy(), precision=prec)
        assert relerr(yp.numpy(), want) < tol
        yh = np.zeros(N, dtype=np.complex128)
        E.mul_(yh, opr, x, precision=prec)
        assert relerr(yh, want) < tol
    # the default policy keeps a sector this small unscaled
    opr.slab_scaling(0)
    assert opr.build_slabs(slab_bytes=1 << 20, max_bytes=1 << 30)
    assert not opr.slab_scaling()


@pytest.mark.parametrize("scaling", [1, 2])
def test_slab_row_blocks_host_buffers(monkeypatch, scaling):
    """Host-buffer products in row blocks (each block's last pass on a second stream beside the next
    block's passes): the same sums in the same order as one block, bit for bit, in both precisions and
    for y += H x."""
    import torch
    import edgpu as E
    opr, red, terms, _ = _chain(E, 20, 0, False)
    N = opr.dimension
    assert opr.build_targets(1 << 30)
    opr.slab_scaling(scaling)
    assert opr.build_slabs(slab_bytes=1024 * 8, max_bytes=1 << 30)
    assert opr.slabs_info[0] >= 3
    x = O.complex_gaussian(N, 8)
    want = O.apply_rows(red, terms, x)
    xp = torch.from_numpy(x).pin_memory()
    out = {}
    for blocks in ("1", "3", "7"):
        monkeypatch.setenv("EDGPU_SLAB_ROW_BLOCKS", blocks)
        for prec in ("mixed", "fp64"):
            yp = torch.zeros(N, dtype=torch.complex128).pin_memory()
            E.mul_(yp.numpy(), opr, xp.numpy(), precision=prec)
            E.apply_(yp.numpy(), opr, xp.numpy(), precision=prec)
            out[blocks, prec] = yp.numpy().copy()
    for prec, tol in (("mixed", 1e-5), ("fp64", 1e-12)):
        assert relerr(out["1", prec], 2 * want) < tol
        assert np.array_equal(out["3", prec], out["1", prec]), prec
        assert np.array_equal(out["7", prec], out["1", prec]), prec


def test_slab_build_refusals():
    import edgpu as E
    opr, _, _, _ = _chain(E, 12, 0, False)
    # no target table: nothing built
    assert not opr.build_slabs(slab_bytes=1 << 20)
    assert opr.build_targets(1 << 30)
    # a byte limit below the table's size: nothing kept
    assert not opr.build_slabs(slab_bytes=1 << 20, max_bytes=16)
    assert opr.slabs_info == (0, 0, 0)
    # slabs of at least 1024 columns: one pass for this small sector (the first pass is also the last)
    assert opr.build_slabs(slab_bytes=8, max_bytes=1 << 30)
    assert opr.slabs_info[0] == 1 and opr.slabs_info[1] == 1024
    import torch
    x = O.complex_gaussian(opr.dimension, 2)
    _, y = _products(E, opr, x)
    opr.slab_use("mixed", False)
    _, y0 = _products(E, opr, x)
    assert relerr(y.cpu().numpy().astype(np.complex128), y0.cpu().numpy().astype(np.complex128)) < 1e-6
