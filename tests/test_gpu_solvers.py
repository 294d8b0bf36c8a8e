"""Lanczos, coupling gradients, batched sectors and size-independent properties at full size (GPU)."""
import math

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def edgpu():
    import torch
    assert torch.cuda.is_available()
    import edgpu as E
    return E


def chain_op(E, L, m=0, jxy=1.0, jz=1.0):
    from edgpu import lattice
    hs, _ = E.spin_half_system(L)
    hsr = E.represent(E.HilbertSpaceSector(hs, 0), lazy=True)
    rh = E.symmetry_reduce(hsr, E.translation_symops(L, m))
    H = lattice.xxz_hamiltonian(hs, lattice.chain_bonds(L), jxy, jz)
    return hs, rh, E.represent(rh, H)


def test_lanczos_e0_matches_dense(edgpu):
    L = 16
    sites = O.spin_half_sites(L)
    parent = O.hs_get_basis_list(sites, [(0,)])
    bw, off = O.bit_layout(sites)
    maps, amps = O.translation_symops((L, 1), (0, 0))
    red = O.symmetry_reduce(parent, bw, off, maps, amps)
    terms = O.heisenberg_terms(L, [(i, (i + 1) % L) for i in range(L)], [1.0] * L, [1.0] * L)
    e_dense = np.linalg.eigvalsh(O.dense_matrix(red, terms))[0]
    _, rh, opr = chain_op(edgpu, L)
    r64 = edgpu.lanczos(opr, 120, precision="fp64", reorth=True, seed=1)
    assert abs(r64.e0 - e_dense) < 1e-10 * abs(e_dense)
    rmx = edgpu.lanczos(opr, 120, precision="mixed", reorth=True, seed=1, refine=True, tol=1e-12)
    assert abs(rmx.e0 - e_dense) < 1e-10 * abs(e_dense)
    rnr = edgpu.lanczos(opr, 120, precision="fp64", reorth=False, seed=1)
    assert abs(rnr.e0 - e_dense) < 1e-10 * abs(e_dense)
    # mixed run closed by the FP64 Rayleigh quotient of its Ritz vector (accepted at 1e-10), and a
    # tolerance no estimate can meet, which falls back to FP64 Lanczos from that vector
    rrq = edgpu.lanczos(opr, 120, precision="mixed", reorth=False, seed=1, refine=True, tol=1e-10)
    assert abs(rrq.e0 - e_dense) < 1e-10 * abs(e_dense)
    rfb = edgpu.lanczos(opr, 120, precision="mixed", reorth=False, seed=1, refine=True, tol=1e-17)
    assert abs(rfb.e0 - e_dense) < 1e-10 * abs(e_dense)
    assert rfb.steps > rrq.steps
    rgs = edgpu.lanczos(opr, 120, precision="mixed", reorth=False, seed=1, refine=True, tol=1e-10,
                        want_vector=True)
    g = rgs.ground_state
    assert abs(np.linalg.norm(g) - 1.0) < 1e-12
    assert abs(np.vdot(g, opr @ g).real - e_dense) < 1e-9 * abs(e_dense)
    rv = edgpu.lanczos(opr, 120, precision="fp64", reorth=True, seed=1, want_vector=True)
    psi = rv.ground_state
    hpsi = opr @ psi
    assert abs(np.vdot(psi, hpsi).real - e_dense) < 1e-9 * abs(e_dense)
    assert np.linalg.norm(hpsi - e_dense * psi) < 1e-6


def test_lanczos_without_stored_basis(edgpu):
    """Ritz vectors rebuilt by a second pass of the recurrence (Krylov basis not stored) equal the
    stored-basis ones; mixed precision polished in FP64 reaches the FP64 eigenvalue."""
    _, rh, opr = chain_op(edgpu, 20)
    ref = edgpu.lanczos(opr, 90, precision="fp64", reorth=False, seed=3, want_vector=True)
    ref_mx = edgpu.lanczos(opr, 90, precision="mixed", reorth=False, seed=3, want_vector=True)
    try:
        edgpu.set_krylov_limit(1)          # nothing fits: rolling vectors, two-pass Ritz vectors
        lean = edgpu.lanczos(opr, 90, precision="fp64", reorth=False, seed=3, want_vector=True)
        lean_mx = edgpu.lanczos(opr, 90, precision="mixed", reorth=False, seed=3, want_vector=True)
        pol = edgpu.lanczos(opr, 90, precision="mixed", reorth=False, seed=3, refine=True, tol=1e-12)
        with pytest.raises(MemoryError):
            edgpu.lanczos(opr, 90, precision="fp64", reorth=True, seed=3)
    finally:
        edgpu.set_krylov_limit(0)
    assert lean.e0 == ref.e0 and lean.steps == ref.steps
    assert np.array_equal(lean.alphas, ref.alphas)
    assert np.linalg.norm(lean.ground_state - ref.ground_state) < 1e-10
    assert lean_mx.e0 == ref_mx.e0
    assert np.linalg.norm(lean_mx.ground_state - ref_mx.ground_state) < 1e-10
    assert abs(pol.e0 - ref.e0) < 1e-11 * abs(ref.e0)


def test_lanczos_chain24_k0_known_energy(edgpu):
    # E0 of the L=24 Heisenberg chain (J=1, S=1/2 spins, H = sum S.S) in the k=0 sector
    _, rh, opr = chain_op(edgpu, 24)
    assert rh.dimension == 112720
    r = edgpu.lanczos(opr, 200, precision="fp64", reorth=True, seed=2)
    rm = edgpu.lanczos(opr, 200, precision="mixed", reorth=True, seed=2, refine=True, tol=1e-12)
    assert abs(rm.e0 - r.e0) < 1e-9 * abs(r.e0)
    # per-site energy close to the Bethe-ansatz value 1/4 - ln 2 for a finite ring
    assert -0.46 < r.e0 / 24 < -0.44


def coupled_chain(E, L, J):
    from edgpu import lattice
    hs, _ = E.spin_half_system(L)
    hsr = E.represent(E.HilbertSpaceSector(hs, 0))
    rh = E.symmetry_reduce(hsr, E.translation_symops(L, 0)) if False else hsr
    m, r, c, a, ids = lattice.heisenberg_coupled(hs, lattice.chain_bonds(L))
    opr = E.OperatorRepresentation.from_terms(rh, m, r, c, a, coupling_ids=ids, couplings=J)
    return hs, rh, opr, (m, r, c, a, ids)


def test_coupling_gradient_fd_and_oracle(edgpu):
    import torch
    L = 12
    rng = np.random.default_rng(4)
    J = 0.5 + rng.random(L)
    hs, sp, opr, (m, r, c, a, ids) = coupled_chain(edgpu, L, J)
    N = sp.dimension
    x = O.complex_gaussian(N, 5)
    gy = O.complex_gaussian(N, 6)
    xd, gyd = torch.from_numpy(x).cuda(), torch.from_numpy(gy).cuda()
    yd = torch.empty_like(xd)
    g = edgpu.coupling_grad(opr, xd, gyd, precision="fp64", y=yd)
    # y = H x
    parent = sp.basis_list
    terms_full = [(int(m[t]), int(r[t]), int(c[t]), complex(a[t]) * J[ids[t]]) for t in range(len(m))]
    assert np.allclose(yd.cpu().numpy(), O.apply_rows(parent, terms_full, x), atol=1e-12)
    # oracle: Re <gy | H_b x> with H_b the unit-coupling bond operator
    for b in range(L):
        tb = [(int(m[t]), int(r[t]), int(c[t]), complex(a[t])) for t in range(len(m)) if ids[t] == b]
        want = np.vdot(gy, O.apply_rows(parent, tb, x)).real
        assert abs(g[b] - want) < 1e-12 * max(1.0, abs(want))
    # central finite differences of L(J) = Re <gy | H(J) x>, h = 1e-6
    yv = torch.empty_like(xd)
    for b in (0, 5, 11):
        vals = []
        for s in (1, -1):
            Jp = J.copy()
            Jp[b] += s * 1e-6
            opr.set_couplings(Jp)
            edgpu.mul_(yv, opr, xd, precision="fp64")
            vals.append(np.vdot(gy, yv.cpu().numpy()).real)
        opr.set_couplings(J)
        fd = (vals[0] - vals[1]) / 2e-6
        assert abs(fd - g[b]) < 1e-6 * max(1.0, abs(g[b]))
    # dL/dx = H^dagger gy
    gx = torch.empty_like(xd)
    edgpu.mul_adjoint_(gx, opr, gyd, precision="fp64")
    assert np.allclose(gx.cpu().numpy(), np.conj(O.apply_cols(parent, terms_full, np.conj(gy))), atol=1e-12)
    # mixed precision gradient
    g32 = edgpu.coupling_grad(opr, xd.to(torch.complex64), gyd.to(torch.complex64), precision="mixed")
    assert np.allclose(g32, g, atol=1e-5)


def test_hellmann_feynman(edgpu):
    # at the ground state, dE0/dJ_b = <psi|H_b|psi> = coupling_grad(x=psi, gy=psi)
    import torch
    L = 10
    rng = np.random.default_rng(8)
    J = 0.5 + rng.random(L)
    hs, sp, opr, _ = coupled_chain(edgpu, L, J)
    r = edgpu.lanczos(opr, 150, precision="fp64", reorth=True, want_vector=True)
    psi = torch.from_numpy(r.ground_state).cuda()
    g = edgpu.coupling_grad(opr, psi, psi, precision="fp64")
    assert abs(np.dot(g, J) - r.e0) < 1e-9 * abs(r.e0)       # Euler: E0 = sum_b J_b dE0/dJ_b
    for b in (0, 3):
        es = []
        for s in (1, -1):
            Jp = J.copy()
            Jp[b] += s * 1e-5
            opr.set_couplings(Jp)
            es.append(edgpu.lanczos(opr, 150, precision="fp64", reorth=True).e0)
        opr.set_couplings(J)
        assert abs((es[0] - es[1]) / 2e-5 - g[b]) < 1e-6


def test_batched_sectors_equal_individual(edgpu):
    import torch
    from edgpu import lattice
    L = 16
    hs, _ = edgpu.spin_half_system(L)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0), lazy=True)
    H = lattice.xxz_hamiltonian(hs, lattice.chain_bonds(L), 1.0, 0.8)
    oprs = [edgpu.represent(edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m)), H) for m in range(L)]
    xs = [edgpu.random_state(o.dimension, 100 + m, "mixed") for m, o in enumerate(oprs)]
    ys = [torch.empty_like(x) for x in xs]
    ref = [torch.empty_like(x) for x in xs]
    for o, x, y in zip(oprs, xs, ref):
        edgpu.mul_(y, o, x, precision="mixed")
    b = edgpu.Batch(oprs)
    for use_graph in (False, True, True):
        for y in ys:
            y.zero_()
        b.mul_(ys, xs, precision="mixed", use_graph=use_graph)
        torch.cuda.synchronize()
        for y, r in zip(ys, ref):
            assert torch.equal(y, r)


def test_full_size_properties_chain24(edgpu):
    """Size-independent checks at the benchmark size: Hermiticity, linearity, mixed vs FP64,
    determinism, and dimension conservation over all 24 momenta."""
    import torch
    L = 24
    hs, rh, opr = chain_op(edgpu, L)
    N = rh.dimension
    u = edgpu.random_state(N, 1, "fp64")
    v = edgpu.random_state(N, 2, "fp64")
    Hu, Hv = torch.empty_like(u), torch.empty_like(v)
    edgpu.mul_(Hu, opr, u)
    edgpu.mul_(Hv, opr, v)
    lhs = torch.vdot(u, Hv).item()
    rhs = torch.vdot(v, Hu).item().conjugate()
    assert abs(lhs - rhs) < 1e-12 * max(1.0, abs(lhs))
    w = (0.3 - 0.2j) * u + 1.7 * v
    Hw = torch.empty_like(w)
    edgpu.mul_(Hw, opr, w)
    assert torch.linalg.vector_norm(Hw - ((0.3 - 0.2j) * Hu + 1.7 * Hv)).item() < 1e-12 * torch.linalg.vector_norm(Hw).item()
    Hu2 = torch.empty_like(u)
    edgpu.mul_(Hu2, opr, u)
    assert torch.equal(Hu, Hu2)
    u32, H32 = u.to(torch.complex64), torch.empty(N, dtype=torch.complex64, device="cuda")
    edgpu.mul_(H32, opr, u32, precision="mixed")
    assert (torch.linalg.vector_norm(H32.to(torch.complex128) - Hu) / torch.linalg.vector_norm(Hu)).item() < 1e-6
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0), lazy=True)
    dims = [edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, m)).dimension for m in range(L)]
    assert sum(dims) == math.comb(24, 12)
    assert dims[0] == 112720


def test_reduced_sector_random_bond_gradients(edgpu):
    """The benchmark's gradient setting at a smaller size: chain L=12, per-bond couplings J_b drawn from a
    seed, 2Sz=0, momentum 0.  The terms do not commute with the translations, so the adjoint goes
    through the scatter path.  Checked: dL/dJ_b against the oracle and central differences (h=1e-6),
    dL/dx against directional central differences."""
    import torch
    from edgpu import lattice
    L = 12
    rng = np.random.default_rng(4)
    J = 0.5 + rng.random(L)
    hs, _ = edgpu.spin_half_system(L)
    hsr = edgpu.represent(edgpu.HilbertSpaceSector(hs, 0))
    rh = edgpu.symmetry_reduce(hsr, edgpu.translation_symops(L, 0))
    m, r, c, a, ids = lattice.heisenberg_coupled(hs, lattice.chain_bonds(L))
    opr = edgpu.OperatorRepresentation.from_terms(rh, m, r, c, a, coupling_ids=ids, couplings=J)
    assert not opr.is_invariant
    N = rh.dimension
    sites = O.spin_half_sites(L)
    parent = O.hs_get_basis_list(sites, [(0,)])
    bw, off = O.bit_layout(sites)
    maps, amps = O.translation_symops((L, 1), (0, 0))
    red = O.symmetry_reduce(parent, bw, off, maps, amps)
    x = O.complex_gaussian(N, 5)
    gy = O.complex_gaussian(N, 6)
    xd, gyd = torch.from_numpy(x).cuda(), torch.from_numpy(gy).cuda()
    g = edgpu.coupling_grad(opr, xd, gyd, precision="fp64")
    for b in range(L):
        tb = [(int(m[t]), int(r[t]), int(c[t]), complex(a[t])) for t in range(len(m)) if ids[t] == b]
        want = np.vdot(gy, O.apply_rows(red, tb, x)).real
        assert abs(g[b] - want) < 1e-12 * max(1.0, abs(want))
    yv = torch.empty_like(xd)

    def loss(Jv, xv):
        opr.set_couplings(Jv)
        edgpu.mul_(yv, opr, xv, precision="fp64")
        torch.cuda.synchronize()
        return np.vdot(gy, yv.cpu().numpy()).real

    for b in (0, 7):
        Jp, Jm = J.copy(), J.copy()
        Jp[b] += 1e-6
        Jm[b] -= 1e-6
        assert abs((loss(Jp, xd) - loss(Jm, xd)) / 2e-6 - g[b]) < 1e-6
    opr.set_couplings(J)
    gx = torch.empty_like(xd)
    edgpu.mul_adjoint_(gx, opr, gyd, precision="fp64")
    torch.cuda.synchronize()
    gxn = gx.cpu().numpy()
    for seed in (1, 2):
        v = O.complex_gaussian(N, 100 + seed)
        vd = torch.from_numpy(v).cuda()
        fd = (loss(J, xd + 1e-6 * vd) - loss(J, xd - 1e-6 * vd)) / 2e-6
        assert abs(fd - np.vdot(gxn, v).real) < 1e-6
