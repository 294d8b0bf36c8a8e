"""Translations times the point group C4v on the 4x4 square torus (128 elements, the symmorphic
space-group reduction of examples/spinhalfsquare_large.jl) through the general permutation path.

For the two momenta whose little group is all of C4v (Gamma and M) and each of its four
one-dimensional irreps, with amplitude exp(-i k.t) chi(p) for the element t o p: representatives
bit-exact against the oracle's symmetry_reduce (symmetry_reduce_generic.jl:22-106), the J1-J2
product against the oracle's reduced rows in FP64 (1e-12) and mixed precision (1e-5), through the
term scan and through the pair-flip schedule's target table, and the lowest eigenvalue from Lanczos
against the dense reduced matrix."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

L1 = L2 = 4
N_SITES = L1 * L2

# C4v about site (0, 0): (name, class, (x, y) -> (x', y'))
POINT = [
    ("E", "E", lambda x, y: (x, y)),
    ("C4", "C4", lambda x, y: (-y, x)),
    ("C2", "C2", lambda x, y: (-x, -y)),
    ("C4^3", "C4", lambda x, y: (y, -x)),
    ("sx", "sv", lambda x, y: (-x, y)),
    ("sy", "sv", lambda x, y: (x, -y)),
    ("sd", "sd", lambda x, y: (y, x)),
    ("sd'", "sd", lambda x, y: (-y, -x)),
]
CHARACTERS = {
    "A1": {"E": 1, "C2": 1, "C4": 1, "sv": 1, "sd": 1},
    "A2": {"E": 1, "C2": 1, "C4": 1, "sv": -1, "sd": -1},
    "B1": {"E": 1, "C2": 1, "C4": -1, "sv": 1, "sd": -1},
    "B2": {"E": 1, "C2": 1, "C4": -1, "sv": -1, "sd": 1},
}


def space_group(k, irrep):
    """(site maps, amplitudes) of T x C4v, identity first: site i -> t(p(i))."""
    maps, amps = [], []
    for b in range(L2):
        for a in range(L1):
            ph = np.exp(-2j * np.pi * (k[0] * a / L1 + k[1] * b / L2))
            for _, cls, f in POINT:
                m = []
                for s in range(N_SITES):
                    x, y = s % L1, s // L1
                    px, py = f(x, y)
                    m.append((px + a) % L1 + L1 * ((py + b) % L2))
                maps.append(m)
                amps.append(ph * CHARACTERS[irrep][cls])
    return np.array(maps, dtype=np.int32), np.array(amps)


def test_library_maps_equal_test_maps():
    from edgpu import lattice
    for k in ((0, 0), (2, 2)):
        for irrep in ("A1", "B2"):
            m1, a1 = space_group(k, irrep)
            m2, a2 = lattice.square_c4v_maps(4, k, irrep)
            assert np.array_equal(m1, m2) and np.allclose(a1, a2)


@pytest.mark.parametrize("k", [(0, 0), (2, 2)])
@pytest.mark.parametrize("irrep", ["A1", "A2", "B1", "B2"])
def test_square4x4_translations_times_c4v(k, irrep):
    import torch
    import edgpu as E
    from edgpu import lattice
    hs, _ = E.spin_half_system(N_SITES)
    nn = lattice.torus_bonds(L1, L2, lattice.SQUARE_NN)
    nnn = lattice.torus_bonds(L1, L2, [(1, 1), (1, -1)])
    jj = [1.0] * len(nn) + [0.5] * len(nnn)
    H = lattice.xxz_hamiltonian(hs, nn + nnn, jj, jj)
    terms = O.heisenberg_terms(N_SITES, nn + nnn, jj, jj)
    maps, amps = space_group(k, irrep)
    assert len(maps) == 128
    hsr = E.represent(E.HilbertSpaceSector(hs, 0))
    ops = [(E.SitePermutation(m), complex(a)) for m, a in zip(maps, amps)]
    rh = E.symmetry_reduce(hsr, ops)
    sites = O.spin_half_sites(N_SITES)
    parent = O.hs_get_basis_list(sites, [(0,)])
    bw, off = O.bit_layout(sites)
    red = O.symmetry_reduce(parent, bw, off, maps, amps)
    assert np.array_equal(rh.basis_list, red.basis_list)
    N = rh.dimension
    if N == 0:
        return
    opr = E.represent(rh, H)
    x = O.complex_gaussian(N, 11)
    want = O.apply_rows(red, terms, x)
    for table in (False, True):
        if table:
            assert opr.build_targets(1 << 28)
        for prec, tol in (("fp64", 1e-12), ("mixed", 1e-5)):
            y = np.zeros(N, dtype=np.complex128)
            E.mul_(y, opr, x, precision=prec)
            assert np.linalg.norm(y - want) <= tol * max(np.linalg.norm(want), 1e-300), (table, prec)
    # lowest eigenvalue against the dense reduced matrix
    Hd = np.stack([O.apply_rows(red, terms, np.eye(N, dtype=np.complex128)[:, j]) for j in range(N)], axis=1)
    assert np.allclose(Hd, Hd.conj().T, atol=1e-12)
    e_dense = np.linalg.eigvalsh(Hd)[0]
    r = E.lanczos(opr, min(N, 120), precision="fp64", reorth=True)
    assert abs(r.e0 - e_dense) < 1e-9 * max(1.0, abs(e_dense)), (r.e0, e_dense)
    torch.cuda.synchronize()


def test_square6x6_translations_times_c4v_sampled_rows_and_e0():
    """6x6 J1-J2 (J2/J1 = 0.5), 2Sz=0, A1 at Gamma of T x C4v (288 elements): 31,566,122
    representatives (Burnside), sampled orbit minimality and completeness, sampled product rows through
    the target table and the slab table against the oracle's orbit-by-orbit row formula, and the
    ground-state energy against the translation-only k=(0,0) sector's (the ground state is in A1)."""
    import torch
    import edgpu as E
    from edgpu import lattice
    L = 6
    n = L * L
    hs, _ = E.spin_half_system(n)
    nn = lattice.torus_bonds(L, L, lattice.SQUARE_NN)
    nnn = lattice.torus_bonds(L, L, [(1, 1), (1, -1)])
    jj = [1.0] * len(nn) + [0.5] * len(nnn)
    H = lattice.xxz_hamiltonian(hs, nn + nnn, jj, jj)
    terms = O.heisenberg_terms(n, nn + nnn, jj, jj)
    maps, amps = lattice.square_c4v_maps(L, (0, 0), "A1")
    hsr = E.represent(E.HilbertSpaceSector(hs, 0), lazy=True)
    rh = E.symmetry_reduce(hsr, lattice.square_c4v_symops(L, (0, 0), "A1"))
    N = rh.dimension
    assert N == O.sector_dimension(maps, np.zeros(len(maps), dtype=int), 1, n // 2) == 31566122
    basis = rh.basis_list
    assert np.all(basis[1:] > basis[:-1])
    ot = O.OrbitTables(n, n // 2, maps, amps, basis)
    rng = np.random.default_rng(41)
    sample = np.unique(np.concatenate([rng.integers(0, N, 2000), np.arange(16), np.arange(N - 16, N)]))
    rep, kept, nd, _ = ot.orbit_info(basis[sample])
    assert np.array_equal(rep, basis[sample]) and kept.all()
    assert np.array_equal(nd, rh.orbit_sizes()[sample])
    parent_states = np.array([int(sum(1 << int(b) for b in rng.choice(n, n // 2, replace=False)))
                              for _ in range(5000)], dtype=np.uint64)
    prep, pkept, _, _ = ot.orbit_info(parent_states)
    assert np.all((O.lookup(basis, prep) >= 0) == pkept)
    opr = E.represent(rh, H)
    free, _ = torch.cuda.mem_get_info()
    assert opr.build_targets(int(0.5 * free))
    x = O.complex_gaussian(N, 5)
    vals, st, _ = ot.rows(terms, x, sample)
    assert (st == 0).all()
    xd = torch.from_numpy(x).cuda()
    for slabs in (False, True):
        if slabs:
            free, _ = torch.cuda.mem_get_info()
            assert opr.build_slabs(slab_bytes=112 << 20, max_bytes=int(0.5 * free))
        for prec, tol in (("fp64", 1e-12), ("mixed", 1e-5)):
            xx = xd if prec == "fp64" else xd.to(torch.complex64)
            y = torch.empty_like(xx)
            E.mul_(y, opr, xx, precision=prec)
            torch.cuda.synchronize()
            ys = y.cpu().numpy().astype(np.complex128)[sample]
            assert np.max(np.abs(ys - vals)) <= tol * np.max(np.abs(vals)), (slabs, prec)
    r = E.lanczos(opr, 300, precision="fp64", reorth=False, seed=7, tol=1e-11)
    assert abs(r.e0 - (-18.13714754007)) < 1e-8, r.e0
