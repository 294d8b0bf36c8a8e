"""The coupling gradient of the pair-flip kernel with diagonal terms of every mask size.

The pair-flip gradient kernel groups the diagonal records by site pair when every record's mask has
at most two bits (one value per pair, coupling and bit pattern), and scans the records one by one
otherwise.  Both are checked against the oracle's Re<gy|H_c x> for every coupling c, on chain L=12,
2Sz=0, momentum 0 (terms that do not commute with the translations), with per-bond exchange
couplings plus diagonal records on one site (a field), on no site (a constant) and, in the second
operator, on three sites.  FP64 within 1e-12 relative, mixed precision within 1e-5 of the scale."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _operator(E, L, with_three_site):
    from edgpu import lattice
    hs, _ = E.spin_half_system(L)
    hsr = E.represent(E.HilbertSpaceSector(hs, 0))
    rh = E.symmetry_reduce(hsr, E.translation_symops(L, 0))
    m, r, c, a, ids = lattice.heisenberg_coupled(hs, lattice.chain_bonds(L))
    m, r, c, a, ids = [list(v) for v in (m, r, c, a, ids)]
    n_c = L
    rng = np.random.default_rng(17)
    # a field on every third site, one coupling per site: records for both values of the bit
    for i in range(0, L, 3):
        for bit, amp in ((1, 0.5), (0, -0.3)):
            m.append(1 << i)
            r.append(bit << i)
            c.append(bit << i)
            a.append(amp)
            ids.append(n_c)
        n_c += 1
    # a constant with its own coupling, and a second constant on an exchange coupling
    for cid in (n_c, 2):
        m.append(0)
        r.append(0)
        c.append(0)
        a.append(0.7)
        ids.append(cid)
    n_c += 1
    # a two-site diagonal record on a pair that is not a bond, complex amplitude
    m.append((1 << 0) | (1 << 5))
    r.append(1 << 5)
    c.append(1 << 5)
    a.append(0.2 - 0.1j)
    ids.append(n_c)
    n_c += 1
    if with_three_site:
        m.append(0b111 << 3)
        r.append(0b101 << 3)
        c.append(0b101 << 3)
        a.append(0.4)
        ids.append(n_c)
        n_c += 1
    J = 0.5 + rng.random(n_c)
    arr = (np.array(m, dtype=np.uint64), np.array(r, dtype=np.uint64), np.array(c, dtype=np.uint64),
           np.array(a, dtype=np.complex128), np.array(ids, dtype=np.int32))
    opr = E.OperatorRepresentation.from_terms(rh, *arr[:4], coupling_ids=arr[4], couplings=J)
    return opr, arr, J


@pytest.mark.parametrize("with_three_site", [False, True])
def test_pair_flip_gradient_with_diagonal_records(with_three_site):
    import torch
    import edgpu as E
    L = 12
    opr, (m, r, c, a, ids), J = _operator(E, L, with_three_site)
    assert not opr.is_invariant
    assert opr.build_targets(1 << 28)
    assert opr.grad_kernel("fp64") == "pair-flip table" and opr.grad_kernel("mixed") == "pair-flip table"
    sites = O.spin_half_sites(L)
    parent = O.hs_get_basis_list(sites, [(0,)])
    bw, off = O.bit_layout(sites)
    maps, amps = O.translation_symops((L, 1), (0, 0))
    red = O.symmetry_reduce(parent, bw, off, maps, amps)
    N = opr.dimension
    x = O.complex_gaussian(N, 5)
    gy = O.complex_gaussian(N, 6)
    xd, gyd = torch.from_numpy(x).cuda(), torch.from_numpy(gy).cuda()
    yd = torch.empty_like(xd)
    g = E.coupling_grad(opr, xd, gyd, precision="fp64", y=yd)
    gm = E.coupling_grad(opr, xd.to(torch.complex64), gyd.to(torch.complex64), precision="mixed")
    torch.cuda.synchronize()
    terms = [(int(m[t]), int(r[t]), int(c[t]), complex(a[t]) * J[ids[t]]) for t in range(len(m))]
    y_ref = O.apply_rows(red, terms, x)
    assert np.linalg.norm(yd.cpu().numpy() - y_ref) <= 1e-12 * np.linalg.norm(y_ref)
    scale = max(abs(np.vdot(gy, O.apply_rows(red, [(int(m[t]), int(r[t]), int(c[t]), complex(a[t]))], x)).real)
                for t in range(len(m)))
    for cid in range(len(J)):
        tc = [(int(m[t]), int(r[t]), int(c[t]), complex(a[t])) for t in range(len(m)) if ids[t] == cid]
        want = np.vdot(gy, O.apply_rows(red, tc, x)).real
        assert abs(g[cid] - want) < 1e-12 * max(1.0, abs(want)), (cid, g[cid], want)
        assert abs(gm[cid] - want) < 1e-5 * max(1.0, scale), (cid, gm[cid], want)
