"""Sparse assembly on the GPU (sparse(opr), Matrix(opr), get_row, get_column, getindex) against the
oracle's dense matrices and the reference's explicit L=4 reduced Hamiltonian."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_tests.json")))
TOL = 1e-12


@pytest.fixture(scope="module")
def edgpu():
    import torch
    assert torch.cuda.is_available()
    import edgpu as E
    return E


def chain(E, L, sector=0):
    hs, _ = E.spin_half_system(L)
    hsr = E.represent(E.HilbertSpaceSector(hs, sector))
    sites = O.spin_half_sites(L)
    parent = O.hs_get_basis_list(sites, [(sector,)])
    bw, off = O.bit_layout(sites)
    return hs, hsr, parent, bw, off


def column_matrix(space, terms):
    """The matrix of the reference's column iterators: row r is e_r^T H by the column iterator."""
    n = space.dim if isinstance(space, O.ReducedTables) else space.size
    M = np.zeros((n, n), dtype=np.complex128)
    e = np.zeros(n, dtype=np.complex128)
    for r in range(n):
        e[:] = 0
        e[r] = 1
        M[r, :] = O.apply_cols(space, terms, e)
    return M


def check_assembly(E, opr, space, terms):
    """sparse / Matrix / rows / columns / elements of opr against the oracle: sparse, Matrix, get_column
    and getindex follow the column iterators, get_row and mul! the row iterators (the two agree for
    operators that commute with the group)."""
    Mr = O.dense_matrix(space, terms)
    Mc = column_matrix(space, terms)
    tol = E.representation.RTOL_F64
    n = Mr.shape[0]
    S = opr.sparse()
    assert S.shape == (n, n)
    assert np.allclose(S.toarray(), Mc, atol=TOL, rtol=0)
    assert np.all(np.abs(S.data) >= tol)
    R = opr.sparse_rows()
    assert np.allclose(R.toarray(), Mr, atol=TOL, rtol=0)
    for r in range(n):                                   # sorted, unique columns per row
        cols = R.indices[R.indptr[r]:R.indptr[r + 1]]
        assert np.all(np.diff(cols) > 0)
    assert np.allclose(opr.todense(), Mc, atol=TOL, rtol=0)
    rng = np.random.default_rng(n)
    for i in rng.integers(0, n, size=min(n, 6)):
        cols, vals = opr.get_row(int(i))
        want = np.nonzero(np.abs(Mr[i]) >= tol)[0]
        assert cols.tolist() == want.tolist()
        assert np.allclose(vals, Mr[i, want], atol=TOL, rtol=0)
        rows, vals = opr.get_column(int(i))
        want = np.nonzero(np.abs(Mc[:, i]) >= tol)[0]
        assert rows.tolist() == want.tolist()
        assert np.allclose(vals, Mc[want, i], atol=TOL, rtol=0)
        j = int(rng.integers(0, n))
        assert abs(opr[int(i), j] - Mc[i, j]) < TOL
        assert np.allclose(opr[int(i), :].toarray().ravel(), np.where(np.abs(Mr[i]) >= tol, Mr[i], 0))
        assert np.allclose(opr[:, int(i)].toarray().ravel(), np.where(np.abs(Mc[:, i]) >= tol, Mc[:, i], 0))
    with pytest.raises(E.BoundsError):
        opr.get_row(n)


def test_sparse_unreduced_and_reduced_chains(edgpu):
    L = 10
    hs, hsr, parent, bw, off = chain(edgpu, L)
    bonds = [(i, (i + 1) % L) for i in range(L)] + [(i, (i + 2) % L) for i in range(L)]
    rng = np.random.default_rng(3)
    jxy = list(rng.uniform(0.5, 1.5, len(bonds)))
    jz = list(rng.uniform(-1, 1, len(bonds)))
    from edgpu import lattice
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    terms = O.heisenberg_terms(L, bonds, jxy, jz)
    check_assembly(edgpu, edgpu.represent(hsr, H), parent, terms)
    for m in (0, 1, 5):
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m))
        maps, amps = O.translation_symops((L, 1), (m, 0))
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        check_assembly(edgpu, edgpu.represent(rh, H), red, terms)


@pytest.mark.parametrize("shape,sector", [((3, 3), 1), ((4, 4), 0)])
def test_sparse_torus(edgpu, shape, sector):
    from edgpu import lattice
    L1, L2 = shape
    n = L1 * L2
    hs, hsr, parent, bw, off = chain(edgpu, n, sector)
    bonds = lattice.torus_bonds(L1, L2, lattice.SQUARE_NN) + lattice.torus_bonds(L1, L2, lattice.SQUARE_NNN)
    jxy = [1.0] * (2 * n) + [0.5] * (2 * n)
    jz = list(jxy)
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    terms = O.heisenberg_terms(n, bonds, jxy, jz)
    for k in [(0, 0), (1, 0), (L1 - 1, 1)]:
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(shape, k))
        maps, amps = O.translation_symops(shape, k)
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        check_assembly(edgpu, edgpu.represent(rh, H), red, terms)


def test_sparse_complex_non_hermitian(edgpu):
    L = 8
    hs, hsr, parent, bw, off = chain(edgpu, L)
    _, offs = O.bit_layout(O.spin_half_sites(L))
    op_o = []
    for i in range(L):
        j = (i + 1) % L
        op_o += O.op_scale(0.7 + 0.3j, O.op_mul(O.pauli_matrix(offs, i, "+"), O.pauli_matrix(offs, j, "-")))
        op_o += O.op_scale(0.2, O.op_mul(O.pauli_matrix(offs, i, "z"), O.pauli_matrix(offs, j, "z")))
    m_, r_, c_, a_ = O.term_arrays(op_o)
    for m in (0, 3):
        rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m))
        maps, amps = O.translation_symops((L, 1), (m, 0))
        red = O.symmetry_reduce(parent, bw, off, maps, amps)
        opr = edgpu.OperatorRepresentation.from_terms(rh, m_, r_, c_, a_)
        check_assembly(edgpu, opr, red, op_o)


def test_sparse_golden_reduced_hamiltonian_L4(edgpu):
    g = GOLD["reduced_H_L4"]
    hs, hsr, parent, bw, off = chain(edgpu, 4)
    j1 = sum((edgpu.pauli_matrix(hs, i, s) * edgpu.pauli_matrix(hs, (i + 1) % 4, s)
              for i in range(4) for s in "xyz"), edgpu.NullOperator())
    full = edgpu.represent(hsr, j1).todense()
    psis = [np.array(p) / np.linalg.norm(p) for p in g["psis"]]
    H = np.array([[psis[i] @ (full @ psis[j]) for j in range(2)] for i in range(2)])
    rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(4, 0))
    assert np.allclose(edgpu.represent(rh, j1)[:, :].toarray(), H, atol=1e-14)


def test_sparse_drops_cancelled_entries(edgpu):
    # two terms with opposite amplitudes on the same flip cancel: the entry is dropped by the tolerance
    hs, hsr, parent, _, _ = chain(edgpu, 4)
    a = edgpu.pauli_matrix(hs, 0, "+") * edgpu.pauli_matrix(hs, 1, "-")
    m_, r_, c_, a_ = [], [], [], []
    for t in a.terms:
        for sgn in (1.0, -1.0 + 1e-13):
            m_.append(t.bitmask); r_.append(t.bitrow); c_.append(t.bitcol); a_.append(sgn * t.amplitude)
    opr = edgpu.OperatorRepresentation.from_terms(hsr, np.array(m_, np.uint64), np.array(r_, np.uint64),
                                                  np.array(c_, np.uint64), np.array(a_))
    assert opr.sparse().nnz == 0
    assert opr.sparse(tol=0.0).nnz > 0


def test_adjoint_is_adjoint_of_the_product_matrix(edgpu):
    """dL/dx = H^dagger gy for the matrix mul! applies: through the adjoint term table when the terms
    commute with the group, by scatter otherwise (random per-bond couplings in a momentum sector)."""
    import torch
    from edgpu import lattice
    L = 10
    hs, hsr, parent, bw, off = chain(edgpu, L)
    bonds = lattice.chain_bonds(L)
    rng = np.random.default_rng(11)
    for jxy, jz in (([1.0] * L, [0.8] * L), (list(0.5 + rng.random(L)), list(0.5 + rng.random(L)))):
        H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
        terms = O.heisenberg_terms(L, bonds, jxy, jz)
        for m in (0, 3):
            rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m))
            maps, amps = O.translation_symops((L, 1), (m, 0))
            red = O.symmetry_reduce(parent, bw, off, maps, amps)
            opr = edgpu.represent(rh, H)
            assert opr.is_invariant == (jxy[0] == jxy[1])
            Mr = O.dense_matrix(red, terms)
            x = O.complex_gaussian(rh.dimension, 5 + m)
            want = Mr.conj().T @ x
            for prec, tol, dt in (("fp64", TOL, torch.complex128), ("mixed", 1e-5, torch.complex64)):
                xd = torch.from_numpy(x).to(dt).cuda()
                yd = torch.full_like(xd, 7.0)
                edgpu.mul_adjoint_(yd, opr, xd, precision=prec)
                torch.cuda.synchronize()
                got = yd.cpu().numpy().astype(np.complex128)
                assert np.linalg.norm(got - want) < tol * np.linalg.norm(want), (prec, m)


def test_representation_algebra(edgpu):
    from edgpu import lattice
    L = 8
    hs, hsr, parent, bw, off = chain(edgpu, L)
    rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, 2))
    A = edgpu.represent(rh, lattice.xxz_hamiltonian(hs, lattice.chain_bonds(L), 1.0, 0.5))
    B = edgpu.represent(rh, lattice.xxz_hamiltonian(hs, [(i, (i + 2) % L) for i in range(L)], 0.3, 0.7))
    x = O.complex_gaussian(rh.dimension, 4)
    ax, bx = A @ x, B @ x
    assert np.allclose((A + B) @ x, ax + bx, atol=TOL)
    assert np.allclose((A - B) @ x, ax - bx, atol=TOL)
    assert np.allclose((2.5 * A) @ x, 2.5 * ax, atol=TOL)
    assert np.allclose((A * 2.5) @ x, 2.5 * ax, atol=TOL)
    assert np.allclose((A / 4) @ x, ax / 4, atol=TOL)
    assert np.allclose((-A) @ x, -ax, atol=TOL)
    assert np.allclose(A.simplify() @ x, ax, atol=TOL)
    assert A.ishermitian()
    C = edgpu.represent(rh, edgpu.pauli_matrix(hs, 0, "+") * edgpu.pauli_matrix(hs, 1, "-"))
    assert not C.ishermitian()
    other = edgpu.represent(edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, 3)),
                            lattice.xxz_hamiltonian(hs, lattice.chain_bonds(L), 1.0, 0.5))
    with pytest.raises(edgpu.ArgumentError):
        A + other


def test_host_buffer_product_graph_replay(edgpu):
    """Pinned host buffers take the graph-replayed path: new contents in the same buffers give the same
    results as pageable buffers, for both precisions, mul! and apply!."""
    import torch
    from edgpu import lattice
    L = 12
    hs, hsr, parent, bw, off = chain(edgpu, L)
    rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, 1))
    opr = edgpu.represent(rh, lattice.xxz_hamiltonian(hs, lattice.chain_bonds(L), 1.0, 0.6))
    n = rh.dimension
    xp = torch.empty(n, dtype=torch.complex128, pin_memory=True)
    yp = torch.empty(n, dtype=torch.complex128, pin_memory=True)
    for prec in ("fp64", "mixed"):
        for seed in (1, 2, 3):
            x = O.complex_gaussian(n, seed)
            xp.numpy()[:] = x
            y_ref = np.zeros(n, complex)
            edgpu.mul_(y_ref, opr, x.copy(), precision=prec)
            edgpu.mul_(yp.numpy(), opr, xp.numpy(), precision=prec)
            assert np.array_equal(yp.numpy(), y_ref)
            edgpu.apply_(yp.numpy(), opr, xp.numpy(), precision=prec)
            assert np.allclose(yp.numpy(), 2 * y_ref, atol=1e-12 if prec == "fp64" else 1e-5)
