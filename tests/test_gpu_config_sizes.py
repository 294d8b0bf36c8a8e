"""GPU parity at the benchmark configurations' full sizes.

Every workload is built exactly as the benchmark builds it (bench.hamiltonian_spec, parent-state map,
target table, autotuned schedule), and checked against the oracle:

* chain L=16 unreduced (12,870 rows) and chain L=24 k=0 (112,720 rows): every row of the product
  against the oracle's table-based restatement of the reference's mul!
  (reduced_operator_representation.jl:57-85), representatives and indices bit-exact against its
  symmetry_reduce (symmetry_reduce_generic.jl:22-106), and the lowest eigenvalue against ARPACK on the
  oracle's product within 1e-10 relative;
* chain L=28 k=0 with per-bond couplings (1,432,860 rows): forward product against the oracle,
  dL/dJ_b for all 28 bonds against Re<gy|H_b x> from the oracle, the adjoint against <gy|H x> for
  random directions, central finite differences (h = 1e-6); Hellmann-Feynman at the ground state of
  the same Hamiltonian in its unreduced 2Sz=0 sector (the random couplings break the translations);
* the triangular 6x5 k=(1,0) sector (5,170,578 rows, complex characters) and the 6x6 J1-J2 k=(0,0)
  sector (252,091,362 rows), whose parent-sized tables do not fit in host memory: the representative
  table against Burnside's count, sortedness and orbit minimality of sampled rows, completeness for
  sampled parent states, and sampled rows of the product against the oracle's orbit-by-orbit
  evaluation of the same row formula (oracle.OrbitTables), through the target table and through the
  column-slab table; the 6x6 ground-state energy against the
  published 36-site value.

Tolerances: FP64 products 1e-12 relative (to the largest |y| entry of the compared set), mixed
precision 1e-5; eigenvalues 1e-10 relative (the FP64 target for E0), mixed E0 within 1e-9 of FP64."""
import math
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


@pytest.fixture(scope="module")
def E():
    import torch
    assert torch.cuda.is_available()
    import edgpu
    return edgpu


def _bench():
    import bench
    return bench


def _prepare(opr, space, reduced=True):
    """The benchmark's set-up: parent-state map, target table, autotuned schedule (FP64 and mixed)."""
    import torch
    if reduced:
        space.build_map()
    free, _ = torch.cuda.mem_get_info()
    opr.build_targets(int(0.8 * free))
    if reduced and space.map_info[0] > 0:
        space.free_map()
    opr.autotune("mixed")
    opr.autotune("fp64")


def _products(E, opr, x):
    """FP64 and mixed-precision products of the host vector x (device buffers)."""
    import torch
    xd = torch.from_numpy(x).cuda()
    y64 = torch.empty_like(xd)
    E.mul_(y64, opr, xd, precision="fp64")
    x32 = xd.to(torch.complex64)
    y32 = torch.empty_like(x32)
    E.mul_(y32, opr, x32, precision="mixed")
    torch.cuda.synchronize()
    out = y64.cpu().numpy(), y32.cpu().numpy().astype(np.complex128)
    del xd, y64, x32, y32
    return out


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b))))


def _oracle_chain(L, k, n_up=None):
    n_up = L // 2 if n_up is None else n_up
    parent = O.popcount_basis(L, n_up)
    sites = O.spin_half_sites(L)
    bw, off = O.bit_layout(sites)
    maps, amps = O.translation_symops((L, 1), (k, 0))
    return O.symmetry_reduce(parent, bw, off, maps, amps)


def _arpack_e0(red_or_parent, terms, n):
    from scipy.sparse.linalg import LinearOperator, eigsh

    def mv(v):
        return O.apply_rows(red_or_parent, terms, np.ascontiguousarray(v.ravel(), dtype=np.complex128))

    A = LinearOperator((n, n), matvec=mv, dtype=np.complex128)
    return float(eigsh(A, k=1, which="SA", tol=1e-14, v0=O.complex_gaussian(n, 9).real + 0j)[0][0])


# ---- chain L=16 (unreduced) and chain L=24 k=0 ----------------------------------------------------

@pytest.mark.parametrize("workload", ["chain16_full", "chain24_k0"])
def test_chain_workload_full_parity(E, workload):
    bench = _bench()
    wl = bench.WORKLOADS[workload]
    space, opr, _ = bench.build_gpu_operator(wl)
    n, bonds, jxy, jz, _, k = bench.hamiltonian_spec(wl)
    terms = O.heisenberg_terms(n, bonds, jxy, jz)
    if wl["kind"] == "chain_full":
        ref_space = O.popcount_basis(n, n // 2)
        assert np.array_equal(space.basis_list, ref_space)
    else:
        ref_space = _oracle_chain(n, k[0])
        assert np.array_equal(space.basis_list, ref_space.basis_list)
        # orbit sizes, and the reference-format mapping tables of the same reduction over a
        # materialised parent (the benchmark's space keeps its parent lazy)
        rep_p = O.lookup(ref_space.parent, ref_space.basis_list)
        sizes = np.rint(1.0 / np.abs(ref_space.basis_mapping_amplitude[rep_p]) ** 2).astype(np.int64)
        assert np.array_equal(space.orbit_sizes(), sizes)
        hs, _ = E.spin_half_system(n)
        full = E.symmetry_reduce(E.represent(E.HilbertSpaceSector(hs, 0)), E.translation_symops(n, k[0]))
        assert np.array_equal(full.basis_mapping_index, ref_space.basis_mapping_index)
        assert np.max(np.abs(full.basis_mapping_amplitude - ref_space.basis_mapping_amplitude)) < 1e-13
        del full
    _prepare(opr, space, reduced=wl["kind"] != "chain_full")
    N = space.dimension
    x = O.complex_gaussian(N, wl["seed"])
    y_ref = O.apply_rows(ref_space, terms, x)
    y64, y32 = _products(E, opr, x)
    assert _rel(y64, y_ref) < 1e-12
    assert _rel(y32, y_ref) < 1e-5
    # lowest eigenvalue: the benchmark's Lanczos (FP64, and mixed closed in FP64) against ARPACK on the
    # oracle's product
    e_ref = _arpack_e0(ref_space, terms, N)
    r64 = E.lanczos(opr, wl["lanczos_steps"], precision="fp64", reorth=wl["reorth"], seed=wl["seed"], tol=1e-12)
    assert abs(r64.e0 - e_ref) < 1e-10 * abs(e_ref)
    rmx = E.lanczos(opr, wl["lanczos_steps"], precision="mixed", reorth=wl["reorth"], seed=wl["seed"], refine=True,
                    tol=1e-10)
    assert abs(rmx.e0 - e_ref) < 1e-10 * abs(e_ref)


# ---- chain L=28 k=0, per-bond couplings: forward, gradients, adjoint -------------------------------

def test_chain28_random_bond_gradients_full_size(E):
    import torch
    from edgpu import lattice
    bench = _bench()
    wl = bench.WORKLOADS["chain28_grad"]
    L = wl["L"]
    hs, _ = E.spin_half_system(L)
    hsr = E.represent(E.HilbertSpaceSector(hs, 0), lazy=True)
    space = E.symmetry_reduce(hsr, E.translation_symops(L, wl["k"]))
    J = 0.5 + np.random.default_rng(wl["seed"]).random(L)
    m, r, c, a, ids = lattice.heisenberg_coupled(hs, lattice.chain_bonds(L))
    opr = E.OperatorRepresentation.from_terms(space, m, r, c, a, coupling_ids=ids, couplings=J)
    assert not opr.is_invariant
    red = _oracle_chain(L, wl["k"])
    assert np.array_equal(space.basis_list, red.basis_list)
    N = space.dimension
    assert N == 1432860
    _prepare(opr, space)
    x = O.complex_gaussian(N, wl["x_seed"])
    gy = O.complex_gaussian(N, wl["gy_seed"])
    terms = [(int(m[t]), int(r[t]), int(c[t]), complex(a[t]) * J[ids[t]]) for t in range(len(m))]
    y_ref = O.apply_rows(red, terms, x)
    y64, y32 = _products(E, opr, x)
    assert _rel(y64, y_ref) < 1e-12
    assert _rel(y32, y_ref) < 1e-5
    xd, gyd = torch.from_numpy(x).cuda(), torch.from_numpy(gy).cuda()
    yd = torch.empty_like(xd)
    assert opr.grad_kernel("fp64") == "pair-flip table" and opr.grad_kernel("mixed") == "pair-flip table"
    g = E.coupling_grad(opr, xd, gyd, precision="fp64", y=yd)
    torch.cuda.synchronize()
    assert _rel(yd.cpu().numpy(), y_ref) < 1e-12
    gm = E.coupling_grad(opr, xd.to(torch.complex64), gyd.to(torch.complex64), precision="mixed")
    for b in range(L):
        tb = [(int(m[t]), int(r[t]), int(c[t]), complex(a[t])) for t in range(len(m)) if ids[t] == b]
        want = np.vdot(gy, O.apply_rows(red, tb, x)).real
        assert abs(g[b] - want) < 1e-11 * max(1.0, abs(want)), (b, g[b], want)
        assert abs(gm[b] - want) < 1e-4 * max(1.0, abs(want)), (b, gm[b], want)
    # the coupling gradient is reproducible bit for bit (per-thread accumulators, fixed block sums)
    g2 = E.coupling_grad(opr, xd, gyd, precision="fp64")
    assert np.array_equal(g, g2)
    # the adjoint: <H^dagger gy, v> = <gy, H v> for random directions v (oracle products), by the
    # scatter and by the adjoint target table (a gather in a fixed order, reproducible bit for bit)
    gx = torch.empty_like(xd)
    E.mul_adjoint_(gx, opr, gyd, precision="fp64")
    assert opr.build_adjoint_targets()
    gxt = torch.empty_like(xd)
    E.mul_adjoint_(gxt, opr, gyd, precision="fp64")
    gxt2 = torch.empty_like(xd)
    E.mul_adjoint_(gxt2, opr, gyd, precision="fp64")
    torch.cuda.synchronize()
    assert torch.equal(gxt, gxt2)
    assert _rel(gxt.cpu().numpy(), gx.cpu().numpy()) < 1e-12
    gxm = torch.empty(N, dtype=torch.complex64, device="cuda")
    E.mul_adjoint_(gxm, opr, gyd.to(torch.complex64), precision="mixed")
    torch.cuda.synchronize()
    assert _rel(gxm.cpu().numpy().astype(np.complex128), gxt.cpu().numpy()) < 1e-5
    for gxn in (gx.cpu().numpy(), gxt.cpu().numpy()):
        for seed in (11, 12, 13):
            v = O.complex_gaussian(N, seed)
            lhs = np.vdot(gxn, v)
            rhs = np.vdot(gy, O.apply_rows(red, terms, v))
            assert abs(lhs - rhs) < 1e-11 * max(1.0, abs(rhs))

    # central finite differences of L(J) = Re<gy|H(J) x> (h = 1e-6, FP64 products)
    def loss(Jv):
        opr.set_couplings(Jv)
        E.mul_(yd, opr, xd, precision="fp64")
        torch.cuda.synchronize()
        return np.vdot(gy, yd.cpu().numpy()).real

    h = 1e-6
    for b in (0, 9, 27):
        Jp, Jm = J.copy(), J.copy()
        Jp[b] += h
        Jm[b] -= h
        assert abs((loss(Jp) - loss(Jm)) / (2 * h) - g[b]) < 1e-6 * max(1.0, abs(g[b]))
    opr.set_couplings(J)
    # Hellmann-Feynman at the ground state: dE0/dJ_b = <psi|H_b|psi> (the coupling gradient with x =
    # gy = psi) against central differences of E0.  The random couplings break the translations, so
    # the momentum sector is not invariant and the reference's row formula gives a non-Hermitian
    # matrix there; the ground state of this Hamiltonian is checked in its unreduced 2Sz = 0 sector
    # (40,116,600 states), where H is Hermitian.
    del opr, space
    import gc
    gc.collect()
    torch.cuda.empty_cache()
    full = E.represent(E.HilbertSpaceSector(hs, 0))
    assert full.dimension == 40116600
    opf = E.OperatorRepresentation.from_terms(full, m, r, c, a, coupling_ids=ids, couplings=J)
    free, _ = torch.cuda.mem_get_info()
    opf.build_targets(int(0.5 * free))
    E.set_krylov_limit(0)

    def e0(Jv, want_vector=False):
        opf.set_couplings(Jv)
        return E.lanczos(opf, 400, precision="fp64", reorth=False, seed=3, tol=1e-13, want_vector=want_vector)

    rv = e0(J, True)
    psi = torch.from_numpy(rv.ground_state).cuda()
    ghf = E.coupling_grad(opf, psi, psi, precision="fp64")
    assert abs(float(np.dot(ghf, J)) - rv.e0) < 1e-9 * abs(rv.e0)   # H is linear in J (Euler)
    h = 1e-5
    for b in (0, 13):
        Jp, Jm = J.copy(), J.copy()
        Jp[b] += h
        Jm[b] -= h
        fd = (e0(Jp).e0 - e0(Jm).e0) / (2 * h)
        assert abs(fd - ghf[b]) < 2e-5, (b, fd, ghf[b])


# ---- 6x5 triangular k=(1,0) and 6x6 J1-J2 k=(0,0): sampled rows ------------------------------------

def _torus_sampled(E, workload, momentum, n_rows_sample, seed, slab_mb=None):
    import torch
    from edgpu import lattice
    bench = _bench()
    wl = dict(bench.WORKLOADS[workload])
    n, bonds, jxy, jz, shape, _ = bench.hamiltonian_spec(wl)
    hs, _ = E.spin_half_system(n)
    hsr = E.represent(E.HilbertSpaceSector(hs, 0), lazy=True)
    space = E.symmetry_reduce(hsr, E.translation_symops(shape, momentum))
    H = lattice.xxz_hamiltonian(hs, bonds, jxy, jz)
    opr = E.represent(space, H)
    N = space.dimension
    maps, amps = O.translation_symops(shape, momentum)
    G = maps.shape[0]
    L1, L2 = shape
    num = np.array([(momentum[0] * (g % L1) * L2 + momentum[1] * (g // L1) * L1) % G for g in range(G)])
    assert np.allclose(np.exp(-2j * np.pi * num / G), amps)
    assert N == O.sector_dimension(maps, num, G, n // 2)
    basis = space.basis_list
    assert basis.size == N and np.all(basis[1:] > basis[:-1])
    # bit-exact against the oracle's enumeration of the same representatives on the host
    assert np.array_equal(basis, O.torus_representatives(shape, n // 2, momentum))
    ot = O.OrbitTables(n, n // 2, maps, amps, basis)
    rng = np.random.default_rng(seed)
    sample = np.unique(np.concatenate([rng.integers(0, N, n_rows_sample), np.arange(64), np.arange(N - 64, N)]))
    rep, kept, nd, _ = ot.orbit_info(basis[sample])
    assert np.array_equal(rep, basis[sample]) and kept.all()
    assert np.array_equal(nd, space.orbit_sizes()[sample])
    # completeness: random parent states whose orbit is kept have their representative in the table
    parent_states = np.array([int(sum(1 << int(b) for b in rng.choice(n, n // 2, replace=False)))
                              for _ in range(20000)], dtype=np.uint64)
    prep, pkept, _, _ = ot.orbit_info(parent_states)
    found = O.lookup(basis, prep)
    assert np.all((found >= 0) == pkept)
    _prepare(opr, space)
    x = O.complex_gaussian(N, wl["seed"])
    y64, y32 = _products(E, opr, x)
    terms = O.heisenberg_terms(n, bonds, jxy, jz)
    vals, st, nnz = ot.rows(terms, x, sample)
    assert (st == 0).all()
    assert _rel(y64[sample], vals) < 1e-12
    assert _rel(y32[sample], vals) < 1e-5
    if slab_mb is not None:
        # the column-slab product (several passes) in both precisions: the sampled rows against the
        # oracle, the whole vectors against the one-pass target-table product; then the target table
        # is freed (the products read the slab table from here on)
        free, _ = torch.cuda.mem_get_info()
        assert opr.build_slabs(slab_bytes=int(slab_mb * (1 << 20)), max_bytes=int(0.8 * free))
        assert opr.slabs_info[0] >= 3
        y64s, y32s = _products(E, opr, x)
        assert _rel(y64s[sample], vals) < 1e-12
        assert _rel(y32s[sample], vals) < 1e-5
        assert _rel(y64s, y64) < 1e-12
        assert _rel(y32s, y32) < 1e-6
        del y64s, y32s
        opr.free_targets()
    del y64, y32
    return opr, N, x


def test_triangular6x5_k10_sector_sampled_rows(E):
    # complex characters; slabs of 16 MB of x: 3 passes
    _torus_sampled(E, "triangular6x5_k1", (1, 0), 20000, 31, slab_mb=16)


def test_square6x6_k0_sector_sampled_rows_and_e0(E):
    """Config 5.  The ground-state energy per site of the 36-site J1-J2 model at J2/J1 = 0.5 (in units of
    J1, H = sum J S_i.S_j) is -0.50381 in H. J. Schulz, T. A. L. Ziman and D. Poilblanc, J. Phys. I
    France 6, 675 (1996) (Table of 6x6 energies); the k=(0,0), 2Sz=0 sector holds that ground state."""
    opr, N, _ = _torus_sampled(E, "square6x6_k0", (0, 0), 10000, 37, slab_mb=112)
    assert N == 252091362
    bench = _bench()
    wl = bench.WORKLOADS["square6x6_k0"]
    import torch
    torch.cuda.empty_cache()
    r64 = E.lanczos(opr, wl["lanczos_steps"], precision="fp64", reorth=False, seed=wl["seed"], tol=1e-11)
    assert abs(r64.e0 / 36 - (-0.50381)) < 5e-6, r64.e0 / 36
    rmx = E.lanczos(opr, wl["lanczos_steps"], precision="mixed", reorth=False, seed=wl["seed"], refine=True,
                    tol=1e-10)
    assert abs(rmx.e0 - r64.e0) < 1e-9 * abs(r64.e0), (rmx.e0, r64.e0)
