"""Pair-flip schedule of the product (edgpu_op_set_pair_schedule): for operators whose off-diagonal
terms all flip two spin-1/2 sites, rows find their matching terms from bond classes.  The product
equals the oracle's row iterator (reduced_operator_representation.jl:57-85) within the FP64 and mixed
tolerances, equals the term-scan schedule up to summation order, is deterministic, and is the same
with and without parent-state maps and in batched launches."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-5
ORDER_TOL = 1e-13   # pair-flip vs term-scan schedule in FP64: the same elements summed in another order


@pytest.fixture(scope="module")
def edgpu():
    import torch
    assert torch.cuda.is_available()
    import edgpu as E
    return E


def relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def run(E, opr, x, prec, sched, pair, tps=2, uniform=False):
    import torch
    dt = torch.complex128 if prec == "fp64" else torch.complex64
    xd = torch.from_numpy(x).to(dt).cuda()
    yd = torch.empty_like(xd)
    opr.set_tiling(prec, sched)
    opr.set_pair_schedule(pair, tps, uniform)
    E.mul_(yd, opr, xd, precision=prec)
    torch.cuda.synchronize()
    opr.set_tiling(prec, 0)
    opr.set_pair_schedule(True)
    return yd


def check_pairs(E, opr, space_oracle, terms, N, seed=3, schedules=(-1, -2, -4)):
    import torch
    x = O.complex_gaussian(N, seed)
    want = O.apply_rows(space_oracle, terms, x)
    for sched in schedules:
        scan = run(E, opr, x, "fp64", sched, False).cpu().numpy()
        y = run(E, opr, x, "fp64", sched, True)
        y2 = run(E, opr, x, "fp64", sched, True)
        assert torch.equal(y, y2), sched                       # deterministic
        y = y.cpu().numpy()
        assert relerr(scan, want) < FP64_TOL, sched
        assert relerr(y, want) < FP64_TOL, sched
        assert relerr(y, scan) < ORDER_TOL, sched
        y32 = run(E, opr, x, "mixed", sched, True).cpu().numpy().astype(np.complex128)
        assert relerr(y32, want) < MIXED_TOL, sched
    # apply! adds
    y = np.zeros(N, dtype=np.complex128)
    E.mul_(y, opr, x)
    E.apply_(y, opr, x)
    assert relerr(y, 2 * want) < FP64_TOL


def chain(E, L, sector=0):
    hs, _ = E.spin_half_system(L)
    hsr = E.represent(E.HilbertSpaceSector(hs, sector))
    sites = O.spin_half_sites(L)
    parent = O.hs_get_basis_list(sites, [(sector,)])
    bw, off = O.bit_layout(sites)
    return hs, hsr, parent, bw, off


def test_pair_classes(edgpu):
    from edgpu import lattice
    hs, hsr, _, _, _ = chain(edgpu, 24)
    opr = edgpu.represent(hsr, lattice.xxz_hamiltonian(hs, lattice.chain_bonds(24), 1.0, 1.0))
    assert opr.pair_classes() == (1, 1)     # one bond direction, one rotation
    bonds = lattice.chain_bonds(24) + [(i, (i + 2) % 24) for i in range(24)]
    opr2 = edgpu.represent(hsr, lattice.xxz_hamiltonian(hs, bonds, 1.0, 0.5))
    assert opr2.pair_classes() == (2, 2)
    hs24, _ = edgpu.spin_half_system(24)
    h24 = edgpu.represent(edgpu.HilbertSpaceSector(hs24, 0), lazy=True)
    r24 = edgpu.symmetry_reduce(h24, edgpu.translation_symops((6, 4), (0, 0)))
    b24 = lattice.torus_bonds(6, 4, lattice.SQUARE_NN + lattice.SQUARE_NNN)
    o24 = edgpu.represent(r24, lattice.xxz_hamiltonian(hs24, b24, 1.0, 1.0))
    assert o24.pair_classes() == (4, 5)     # four bond directions, five rotations
    # a term that is not a two-site flip (a transverse field): the term-scan schedule only
    hs12, hsr12, _, _, _ = chain(edgpu, 12)
    Hx = lattice.xxz_hamiltonian(hs12, lattice.chain_bonds(12), 1.0, 1.0) + 0.3 * edgpu.pauli_matrix(hs12, 0, "x")
    full12 = edgpu.represent(hs12)
    assert edgpu.represent(full12, Hx).pair_classes() == (0, 0)


@pytest.mark.parametrize("L", [10, 16])
def test_unreduced_chain(edgpu, L):
    from edgpu import lattice
    hs, hsr, parent, _, _ = chain(edgpu, L)
    bonds = lattice.chain_bonds(L) + [(i, (i + 3) % L) for i in range(L)]
    jxy = [1.0] * L + [0.4] * L
    jz = [0.7] * L + [0.2] * L
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    check_pairs(edgpu, edgpu.represent(hsr, H), parent, O.heisenberg_terms(L, bonds, jxy, jz), parent.size)


def test_reduced_chain_all_momenta_with_and_without_map(edgpu):
    import torch
    from edgpu import lattice
    L = 16
    hs, hsr, parent, bw, off = chain(edgpu, L)
    bonds = lattice.chain_bonds(L) + [(i, (i + 2) % L) for i in range(L)]
    rng = np.random.default_rng(8)
    jxy = 0.5 + rng.random(len(bonds))       # per-bond couplings: terms need not commute with translations
    jz = 0.5 + rng.random(len(bonds))
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    terms = O.heisenberg_terms(L, bonds, jxy, jz)
    for m in range(L):
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m))
        maps, amps = O.translation_symops((L, 1), (m, 0))
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        opr = edgpu.represent(rh, H)
        check_pairs(edgpu, opr, red, terms, rh.dimension, seed=m + 1, schedules=(-1, -2))
        x = O.complex_gaussian(rh.dimension, 40 + m)
        plain = {p: run(edgpu, opr, x, p, -1, True) for p in ("fp64", "mixed")}
        assert rh.build_map(1 << 28)
        for p in ("fp64", "mixed"):
            assert torch.equal(run(edgpu, opr, x, p, -1, True), plain[p]), (m, p)
        rh.free_map()


@pytest.mark.parametrize("shape,vectors,sector", [
    ((4, 4), "square", 0), ((6, 3), "triangular", 2), ((4, 5), "square", 0)])
def test_torus(edgpu, shape, vectors, sector):
    import torch
    from edgpu import lattice
    L1, L2 = shape
    n = L1 * L2
    hs, _ = edgpu.spin_half_system(n)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, sector), lazy=True)
    if vectors == "square":
        b1, b2 = lattice.torus_bonds(L1, L2, lattice.SQUARE_NN), lattice.torus_bonds(L1, L2, lattice.SQUARE_NNN)
    else:
        b1, b2 = lattice.torus_bonds(L1, L2, lattice.TRIANGULAR_NN), lattice.torus_bonds(L1, L2, lattice.TRIANGULAR_NNN)
    bonds = b1 + b2
    jxy = [1.0] * len(b1) + [0.5] * len(b2)
    jz = [0.8 * j for j in jxy]
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    terms = O.heisenberg_terms(n, bonds, jxy, jz)
    sites = O.spin_half_sites(n)
    parent = O.hs_get_basis_list(sites, [(sector,)])
    bw, off = O.bit_layout(sites)
    for k in [(0, 0), (1, 0), (L1 // 2, L2 - 1)]:
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(shape, k))
        maps, amps = O.translation_symops(shape, k)
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        opr = edgpu.represent(rh, H)
        assert opr.pair_classes()[0] > 0
        check_pairs(edgpu, opr, red, terms, rh.dimension, seed=k[0] + 5 * k[1])
        x = O.complex_gaussian(rh.dimension, 3)
        plain = run(edgpu, opr, x, "mixed", -2, True)
        assert rh.build_map(1 << 28)
        assert torch.equal(run(edgpu, opr, x, "mixed", -2, True), plain), k
        rh.free_map()


def test_complex_exchange_and_pair_terms(edgpu):
    """Complex exchange (a chirality term) and S+S+ / S-S- pair terms on parallel bits, in the full
    space (pair terms leave every fixed-magnetisation sector), reduced by translations."""
    L = 10
    hs, _ = edgpu.spin_half_system(L)
    full = edgpu.represent(hs)
    sites = O.spin_half_sites(L)
    parent = O.hs_get_basis_list(sites)
    bw, offs = O.bit_layout(sites)
    op_o = []
    for i in range(L):
        j = (i + 1) % L
        op_o += O.op_scale(0.6 + 0.35j, O.op_mul(O.pauli_matrix(offs, i, "+"), O.pauli_matrix(offs, j, "-")))
        op_o += O.op_scale(0.6 - 0.35j, O.op_mul(O.pauli_matrix(offs, i, "-"), O.pauli_matrix(offs, j, "+")))
        op_o += O.op_scale(0.25, O.op_mul(O.pauli_matrix(offs, i, "+"), O.pauli_matrix(offs, j, "+")))
        op_o += O.op_scale(0.25, O.op_mul(O.pauli_matrix(offs, i, "-"), O.pauli_matrix(offs, j, "-")))
        op_o += O.op_scale(0.3, O.op_mul(O.pauli_matrix(offs, i, "z"), O.pauli_matrix(offs, j, "z")))
    op_o = O.simplify(op_o)
    m_, r_, c_, a_ = O.term_arrays(op_o)
    opr_full = edgpu.OperatorRepresentation.from_terms(full, m_, r_, c_, a_)
    assert opr_full.pair_classes() == (1, 1)
    check_pairs(edgpu, opr_full, parent, op_o, parent.size)
    for m in (0, 3):
        rh = edgpu.symmetry_reduce(full, edgpu.translation_symops(L, m))
        maps, amps = O.translation_symops((L, 1), (m, 0))
        red = O.symmetry_reduce(parent, bw, offs, maps, amps)
        opr = edgpu.OperatorRepresentation.from_terms(rh, m_, r_, c_, a_)
        check_pairs(edgpu, opr, red, op_o, rh.dimension, seed=20 + m)


def test_generic_group_with_bitflip(edgpu):
    from edgpu import lattice
    L = 12
    hs, hsr, parent, bw, off = chain(edgpu, L)
    full = (1 << L) - 1
    bonds = lattice.chain_bonds(L)
    H = lattice.xxz_hamiltonian(hs, bonds, 1.0, 0.9)
    terms = O.heisenberg_terms(L, bonds, [1.0] * L, [0.9] * L)
    for m, par in ((0, 1), (4, -1)):
        ops, maps, flips, amps = [], [], [], []
        for t, a in edgpu.translation_symops(L, m):
            for f, chi in ((False, 1), (True, par)):
                ops.append((t * edgpu.GlobalBitFlip(f) if f else t, chi * a))
                maps.append(t.map)
                flips.append(full if f else 0)
                amps.append(chi * a)
        rh = edgpu.symmetry_reduce(hsr, ops)
        red = O.symmetry_reduce(parent, bw, off, np.array(maps, dtype=np.int32), np.array(amps),
                                flips=np.array(flips, dtype=np.uint64))
        check_pairs(edgpu, edgpu.represent(rh, H), red, terms, rh.dimension)


def test_batch_pair_schedule(edgpu):
    """All momentum sectors of a triangular 4x3 torus in one launch equal the per-sector products
    bit for bit (same lanes per row), with and without maps; both equal the oracle."""
    import torch
    from edgpu import lattice
    L1, L2 = 4, 3
    n = L1 * L2
    hs, _ = edgpu.spin_half_system(n)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0))
    bonds = lattice.torus_bonds(L1, L2, lattice.TRIANGULAR_NN) + lattice.torus_bonds(L1, L2, lattice.TRIANGULAR_NNN)
    H = lattice.xxz_hamiltonian(hs, bonds, 1.0, 0.8)
    terms = O.heisenberg_terms(n, bonds, [1.0] * len(bonds), [0.8] * len(bonds))
    sites = O.spin_half_sites(n)
    parent = O.hs_get_basis_list(sites, [(0,)])
    bw, off = O.bit_layout(sites)
    ks = [(a, b) for b in range(L2) for a in range(L1)]
    spaces = [edgpu.symmetry_reduce(hsr, edgpu.translation_symops((L1, L2), k)) for k in ks]
    oprs = [edgpu.represent(sp, H) for sp in spaces]
    assert all(o.pair_classes()[0] > 0 for o in oprs)
    for prec, dt in (("fp64", torch.complex128), ("mixed", torch.complex64)):
        xs = [edgpu.random_state(o.dimension, 60 + i, prec) for i, o in enumerate(oprs)]
        for lpr in (1, 2):
            ref = []
            for o, x in zip(oprs, xs):
                o.set_tiling(prec, -lpr)
                y = torch.empty_like(x)
                edgpu.mul_(y, o, x, precision=prec)
                ref.append(y)
                o.set_tiling(prec, 0)
            b = edgpu.Batch(oprs)
            b.set_tiling(prec, lpr)
            for mapped in (False, True):
                for sp in spaces:
                    if mapped:
                        assert sp.build_map(1 << 26)
                    else:
                        sp.free_map()
                for use_graph in (False, True):
                    ys = [torch.empty_like(x) for x in xs]
                    b.mul_(ys, xs, precision=prec, use_graph=use_graph)
                    torch.cuda.synchronize()
                    for y, r in zip(ys, ref):
                        assert torch.equal(y, r), (prec, lpr, mapped, use_graph)
            for sp in spaces:
                sp.free_map()
        tol = FP64_TOL if prec == "fp64" else MIXED_TOL
        for k, o, x, y in zip(ks, oprs, xs, ref):
            maps, amps = O.translation_symops((L1, L2), k)
            red = O.symmetry_reduce(parent, bw, off, maps, amps)
            want = O.apply_rows(red, terms, x.cpu().numpy().astype(np.complex128))
            assert relerr(y.cpu().numpy().astype(np.complex128), want) < tol, k


def test_autotune_picks_a_schedule(edgpu):
    """The autotuner times the row-per-lane schedules with and without pair flips and keeps one; the
    product then still equals the oracle, and switching the pair-flip schedule off is respected."""
    from edgpu import lattice
    L = 14
    hs, hsr, parent, bw, off = chain(edgpu, L)
    H = lattice.xxz_hamiltonian(hs, lattice.chain_bonds(L), 1.0, 0.7)
    terms = O.heisenberg_terms(L, lattice.chain_bonds(L), [1.0] * L, [0.7] * L)
    rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, 2))
    maps, amps = O.translation_symops((L, 1), (2, 0))
    red = O.symmetry_reduce(parent, bw, off, maps, amps)
    opr = edgpu.represent(rh, H)
    x = O.complex_gaussian(rh.dimension, 4)
    want = O.apply_rows(red, terms, x)
    for prec, tol in (("fp64", FP64_TOL), ("mixed", MIXED_TOL)):
        rows, _ = opr.autotune(prec)
        assert rows in (-1, -2, -4, 32, 16)
        r2, pair = opr.schedule(prec)
        assert r2 == rows and pair in (0, 2, 4) and (not pair or rows < 0)
        y = np.zeros_like(x)
        edgpu.mul_(y, opr, x, precision=prec)
        assert relerr(y, want) < tol
    opr.set_pair_schedule(False)
    opr.autotune("mixed")
    assert opr.schedule("mixed")[1] == 0
    b = edgpu.Batch([opr])
    lpr, _ = b.autotune("mixed")
    assert lpr in (1, 2, 4) and b.schedule("mixed") == (lpr, 0)


def products_lpr1(E, opr, x):
    """Pair-flip products at one lane per row in both precisions (2 targets per step)."""
    return {p: run(E, opr, x, p, -1, True) for p in ("fp64", "mixed")}


def test_target_table_chain_all_momenta(edgpu):
    """The target table holds the entry of every (row, target) in the product's order: the product
    that streams it equals the looked-up product bit for bit (built with and without a parent-state
    map, at every momentum, so with group elements in the entries) and the oracle."""
    import torch
    from edgpu import lattice
    L = 14
    hs, hsr, parent, bw, off = chain(edgpu, L)
    bonds = lattice.chain_bonds(L) + [(i, (i + 2) % L) for i in range(L)]
    jxy = [1.0] * L + [0.35] * L
    jz = [0.8] * L + [0.2] * L
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    terms = O.heisenberg_terms(L, bonds, jxy, jz)
    for m in range(L):
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m))
        maps, amps = O.translation_symops((L, 1), (m, 0))
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        opr = edgpu.represent(rh, H)
        x = O.complex_gaussian(rh.dimension, 70 + m)
        plain = products_lpr1(edgpu, opr, x)
        for with_map in (False, True):
            if with_map:
                assert rh.build_map(1 << 28)
            assert opr.build_targets(1 << 28)
            n, b = opr.targets_info
            nt, nnz = opr.count_nnz()
            assert n == nt and b in (4, 8)
            for prec in ("fp64", "mixed"):
                assert opr.uses_target_table(prec)
                for tps in (2, 4, 8):
                    y = run(edgpu, opr, x, prec, -1, True, tps)
                    assert torch.equal(y, plain[prec]), (m, with_map, prec, tps)
                for tps in (4, 8):
                    # warp-uniform pair steps: same visiting order per row, same bits
                    opr.set_pair_schedule(True, tps, True)
                    assert opr.schedule(prec)[1] == tps | edgpu.representation.PAIR_UNIFORM
                    y = run(edgpu, opr, x, prec, -1, True, tps, True)
                    assert torch.equal(y, plain[prec]), (m, with_map, prec, tps, "uniform")
            y = run(edgpu, opr, x, "fp64", -1, True).cpu().numpy()
            assert relerr(y, O.apply_rows(red, terms, x)) < FP64_TOL
            opr.free_targets()
            assert opr.targets_info == (0, 0)
            rh.free_map()


@pytest.mark.parametrize("shape,vectors", [((4, 4), "square"), ((6, 3), "triangular")])
def test_target_table_torus(edgpu, shape, vectors):
    import torch
    from edgpu import lattice
    L1, L2 = shape
    n = L1 * L2
    hs, _ = edgpu.spin_half_system(n)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0), lazy=True)
    nn, nnn = ((lattice.SQUARE_NN, lattice.SQUARE_NNN) if vectors == "square"
               else (lattice.TRIANGULAR_NN, lattice.TRIANGULAR_NNN))
    bonds = lattice.torus_bonds(L1, L2, nn) + lattice.torus_bonds(L1, L2, nnn)
    H = lattice.xxz_hamiltonian(hs, bonds, 1.0, 0.7)
    for k in [(0, 0), (1, 1), (L1 - 1, 0)]:
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(shape, k))
        opr = edgpu.represent(rh, H)
        x = O.complex_gaussian(rh.dimension, 11)
        plain = products_lpr1(edgpu, opr, x)
        assert opr.build_targets(1 << 28)
        for prec in ("fp64", "mixed"):
            assert torch.equal(run(edgpu, opr, x, prec, -1, True), plain[prec]), (k, prec)
            for tps in (4, 8):
                assert torch.equal(run(edgpu, opr, x, prec, -1, True, tps, True), plain[prec]), (k, prec, tps)
        opr.free_targets()


def test_target_table_pair_terms_full_space(edgpu):
    """Entries of targets outside the table (here none are) and parallel-bit terms in the full space."""
    import torch
    L = 10
    hs, _ = edgpu.spin_half_system(L)
    full = edgpu.represent(hs)
    _, offs = O.bit_layout(O.spin_half_sites(L))
    op_o = []
    for i in range(L):
        j = (i + 1) % L
        op_o += O.op_scale(0.6 + 0.35j, O.op_mul(O.pauli_matrix(offs, i, "+"), O.pauli_matrix(offs, j, "-")))
        op_o += O.op_scale(0.6 - 0.35j, O.op_mul(O.pauli_matrix(offs, i, "-"), O.pauli_matrix(offs, j, "+")))
        op_o += O.op_scale(0.25, O.op_mul(O.pauli_matrix(offs, i, "+"), O.pauli_matrix(offs, j, "+")))
        op_o += O.op_scale(0.25, O.op_mul(O.pauli_matrix(offs, i, "-"), O.pauli_matrix(offs, j, "-")))
    op_o = O.simplify(op_o)
    m_, r_, c_, a_ = O.term_arrays(op_o)
    for m in (0, 3):
        rh = edgpu.symmetry_reduce(full, edgpu.translation_symops(L, m))
        opr = edgpu.OperatorRepresentation.from_terms(rh, m_, r_, c_, a_)
        x = O.complex_gaussian(rh.dimension, 5)
        plain = products_lpr1(edgpu, opr, x)
        assert opr.build_targets(1 << 26)
        for prec in ("fp64", "mixed"):
            assert torch.equal(run(edgpu, opr, x, prec, -1, True), plain[prec])


def test_target_table_limit_and_term_scan(edgpu):
    """No table when it would exceed the byte limit or when the terms do not allow pair flips."""
    from edgpu import lattice
    hs, hsr, _, _, _ = chain(edgpu, 12)
    rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(12, 0))
    opr = edgpu.represent(rh, lattice.xxz_hamiltonian(hs, lattice.chain_bonds(12), 1.0, 1.0))
    assert not opr.build_targets(16)
    assert opr.targets_info == (0, 0)
    Hx = lattice.xxz_hamiltonian(hs, lattice.chain_bonds(12), 1.0, 1.0) + 0.3 * edgpu.pauli_matrix(hs, 0, "x")
    opx = edgpu.represent(edgpu.represent(hs), Hx)
    assert not opx.build_targets(1 << 26)


def test_target_table_batch(edgpu):
    """All momentum sectors of a triangular 4x3 torus in one launch through their target tables equal
    the per-sector products bit for bit."""
    import torch
    from edgpu import lattice
    L1, L2 = 4, 3
    n = L1 * L2
    hs, _ = edgpu.spin_half_system(n)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0))
    bonds = lattice.torus_bonds(L1, L2, lattice.TRIANGULAR_NN) + lattice.torus_bonds(L1, L2, lattice.TRIANGULAR_NNN)
    H = lattice.xxz_hamiltonian(hs, bonds, 1.0, 0.8)
    spaces = [edgpu.symmetry_reduce(hsr, edgpu.translation_symops((L1, L2), (a, b)))
              for b in range(L2) for a in range(L1)]
    oprs = [edgpu.represent(sp, H) for sp in spaces]
    for prec in ("fp64", "mixed"):
        xs = [edgpu.random_state(o.dimension, 80 + i, prec) for i, o in enumerate(oprs)]
        ref = []
        for o, x in zip(oprs, xs):
            o.set_tiling(prec, -1)
            y = torch.empty_like(x)
            edgpu.mul_(y, o, x, precision=prec)
            ref.append(y)
            o.set_tiling(prec, 0)
        for o in oprs:
            assert o.build_targets(1 << 26)
        b = edgpu.Batch(oprs)
        b.set_tiling(prec, 1)
        assert b.uses_target_tables(prec)
        for use_graph in (False, True):
            ys = [torch.empty_like(x) for x in xs]
            b.mul_(ys, xs, precision=prec, use_graph=use_graph)
            torch.cuda.synchronize()
            for y, r in zip(ys, ref):
                assert torch.equal(y, r), (prec, use_graph)
        lpr, _ = b.autotune(prec)
        ys = [torch.empty_like(x) for x in xs]
        b.mul_(ys, xs, precision=prec, use_graph=True)
        torch.cuda.synchronize()
        tol = FP64_TOL if prec == "fp64" else MIXED_TOL
        for y, r in zip(ys, ref):
            assert (torch.linalg.vector_norm(y - r) / torch.linalg.vector_norm(r)).item() < tol
        for o in oprs:
            o.free_targets()


def hermitian_checks(E, opr, N, prec_tol=1e-12):
    """<u|H v> = conj(<v|H u>), linearity and determinism of the FP64 product on seeded vectors."""
    import torch
    u = E.random_state(N, 1, "fp64")
    v = E.random_state(N, 2, "fp64")
    Hu, Hv = torch.empty_like(u), torch.empty_like(v)
    E.mul_(Hu, opr, u)
    E.mul_(Hv, opr, v)
    lhs = torch.vdot(u, Hv).item()
    rhs = torch.vdot(v, Hu).item().conjugate()
    assert abs(lhs - rhs) < prec_tol * max(1.0, abs(lhs))
    w = (0.3 - 0.2j) * u + 1.7 * v
    Hw = torch.empty_like(w)
    E.mul_(Hw, opr, w)
    ref = (0.3 - 0.2j) * Hu + 1.7 * Hv
    assert (torch.linalg.vector_norm(Hw - ref) / torch.linalg.vector_norm(Hw)).item() < prec_tol
    Hu2 = torch.empty_like(u)
    E.mul_(Hu2, opr, u)
    assert torch.equal(Hu, Hu2)
    return u, Hu


@pytest.mark.parametrize("workload", ["triangular6x5_k1", "chain28_k0"])
def test_full_size_target_table(edgpu, workload):
    """At the benchmark sizes (5,170,578 and 1,432,860 rows): the product through the target table is
    Hermitian, linear and deterministic in FP64, equals the looked-up product bit for bit, and the
    mixed product agrees with FP64 to single precision."""
    import torch
    import bench
    wl = bench.WORKLOADS[workload]
    space, opr, _ = bench.build_gpu_operator(wl)
    assert space.build_map(8 << 30)
    N = space.dimension
    opr.set_tiling("fp64", -1)
    opr.set_tiling("mixed", -1)
    u, Hu_map = hermitian_checks(edgpu, opr, N)
    assert opr.build_targets(8 << 30)
    n, _ = opr.targets_info
    assert n == opr.count_nnz()[0]
    assert opr.uses_target_table("fp64")
    _, Hu_tab = hermitian_checks(edgpu, opr, N)
    assert torch.equal(Hu_tab, Hu_map)
    opr.set_pair_schedule(True, 8, True)
    Hu_uni = torch.empty_like(Hu_tab)
    edgpu.mul_(Hu_uni, opr, u)
    assert torch.equal(Hu_uni, Hu_tab)
    opr.set_pair_schedule(True)
    u32, H32 = u.to(torch.complex64), torch.empty(N, dtype=torch.complex64, device="cuda")
    edgpu.mul_(H32, opr, u32, precision="mixed")
    assert (torch.linalg.vector_norm(H32.to(torch.complex128) - Hu_tab) /
            torch.linalg.vector_norm(Hu_tab)).item() < 1e-6
    opr.free_targets()
    space.free_map()
