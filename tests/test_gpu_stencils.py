"""Projection, momentum, boundary and reduction kernels on the GPU against the CPU oracle."""
import numpy as np
import pytest

from gpu_common import grid_for, is_bound_for, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _fields(n, seed, k=4):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(k):
        f = O.field(n)
        f[:] = rng.standard_normal(f.shape)
        out.append(np.asfortranarray(f))
    return out


def _setup(n=(12, 10, 8), l=(1.0, 2.0, 1.5), cbc="PPPPNN", gr=1.3):
    import torch
    dl = [l[d] / n[d] for d in range(3)]
    dli = [1 / x for x in dl]
    dzc, dzf, dzci, dzfi = grid_for(n, l, cbc, gr)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    return dl, dli, dzc, dzf, dzci, dzfi, T(dzci), T(dzfi)


def test_fillps(require_gpu):
    from cans_gb300 import cans
    n = (12, 10, 8)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n)
    u, v, w, p = _fields(n, 1)
    d = [cans.to_device(x) for x in (u, v, w, p)]
    O.fillps(n, dli, dzfi, 7.3, u, v, w, p)
    cans.fillps(n, dli, dzfi_d, 7.3, *d)
    got = cans.fview(d[3])
    assert np.abs(got - p).max() <= 1e-13 * np.abs(p).max()


def test_correc(require_gpu):
    from cans_gb300 import cans
    n = (12, 10, 8)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n)
    u, v, w, p = _fields(n, 2)
    d = [cans.to_device(x) for x in (u, v, w, p)]
    O.correc(n, dli, dzci, 0.013, p, u, v, w)
    cans.correc(n, dli, dzci_d, 0.013, d[3], d[0], d[1], d[2])
    for g, want in zip(d[:3], (u, v, w)):
        assert np.abs(cans.fview(g) - want).max() <= 1e-14 * np.abs(want).max()


@pytest.mark.parametrize("impl", [0, 1])
def test_updatep(require_gpu, impl):
    from cans_gb300 import cans
    n = (12, 10, 8)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n)
    pp, p = _fields(n, 3, 2)
    d = [cans.to_device(x) for x in (pp, p)]
    O.updatep(n, dli, dzci, dzfi, -0.0021, impl, pp, p)
    cans.updatep(n, dli, dzci_d, dzfi_d, -0.0021, impl, d[0], d[1])
    assert np.abs(cans.fview(d[1]) - p).max() <= 1e-13 * np.abs(p).max()


@pytest.mark.parametrize("impdiff,forced", [(0, (0, 0, 0)), (0, (1, 0, 0)), (1, (1, 1, 0))])
def test_rk_substep(require_gpu, impdiff, forced):
    """rk (src/rk.f90:24) with mom_xyz_ad, bulk forcing and the dudtrko update."""
    import torch
    from cans_gb300 import cans
    n = (12, 10, 8)
    l = (1.0, 2.0, 1.5)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n, l)
    vol = l[0] * l[1] * l[2]
    gvr_c, gvr_f = dl[0] * dl[1] * dzc / vol, dl[0] * dl[1] * dzf / vol
    u, v, w, p = _fields(n, 4)
    rng = np.random.default_rng(9)
    dto = [np.asfortranarray(rng.standard_normal(n)) for _ in range(3)]
    d = [cans.to_device(x) for x in (u, v, w, p)]
    dto_d = [torch.from_numpy(np.ascontiguousarray(x.transpose(2, 1, 0))).cuda() for x in dto]
    T = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    rkpar = (25. / 60., -17. / 60.)
    velf, bforce = (1.0, 0.3, 0.0), (0.1, -0.2, 0.05)
    f_ref = O.rk(rkpar, n, dli, dzci, dzfi, gvr_c, gvr_f, 0.01, 1e-3, p, forced, velf, bforce, impdiff,
                 dto[0], dto[1], dto[2], u, v, w)
    f = cans.rk(rkpar, n, dli, dzci_d, dzfi_d, T(gvr_c), T(gvr_f), 0.01, 1e-3, d[3], forced, velf, bforce, impdiff,
                dto_d[0], dto_d[1], dto_d[2], d[0], d[1], d[2])
    for g, want in zip(d[:3], (u, v, w)):
        assert np.abs(cans.fview(g) - want).max() <= 1e-12 * np.abs(want).max()
    for g, want in zip(dto_d, dto):
        assert np.abs(g.cpu().numpy().transpose(2, 1, 0) - want).max() <= 1e-12 * np.abs(want).max()
    assert np.allclose(f, f_ref, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("cbcvel,cbcpre", [("PPDDDD" * 3, "PPNNNN"), ("PPPPDD" * 3, "PPPPNN"),
                                           ("PP" * 9, "PPPPPP"), ("NNDDNN" + "DDNNNN" + "DDDDDD", "NNNNNN")])
@pytest.mark.parametrize("mode", [(False, 2, 2), (False, -1, 2), (True, 1, 0)])
def test_bounduvw_boundp(require_gpu, cbcvel, cbcpre, mode):
    from cans_gb300 import cans
    n = (8, 7, 6)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n, cbc=cbcpre)
    bcv = list(np.linspace(-0.5, 0.7, 18))
    bcp = list(np.linspace(0.1, 0.6, 6))
    is_bound = is_bound_for(cbcpre)
    u, v, w, p = _fields(n, 5)
    d = [cans.to_device(x) for x in (u, v, w, p)]
    keep, hn, ht = mode
    O.bounduvw(cbcvel, n, bcv, is_bound, dl, dzc, dzf, u, v, w, keep, hn, ht)
    cans.bounduvw(cbcvel, n, bcv, is_bound, dl, dzc, dzf, d[0], d[1], d[2], keep, hn, ht)
    for side in (2, 1):
        O.boundp(cbcpre, n, bcp, is_bound, dl, dzc, p, side)
        cans.boundp(cbcpre, n, bcp, is_bound, dl, dzc, d[3], side)
    for g, want in zip(d, (u, v, w, p)):
        assert np.array_equal(cans.fview(g), want)


def test_updt_rhs_b(require_gpu):
    from cans_gb300 import cans
    n = (8, 7, 6)
    is_bound = [1, 1, 1, 1, 1, 1]
    rhsb = [0.1, -0.2, 0.3, -0.4, 0.5, -0.6]
    (p,) = _fields(n, 6, 1)
    d = cans.to_device(p)
    O.updt_rhs_b("cfc", "DDDDNN", n, is_bound, rhsb, p, alpha=-0.3)
    cans.updt_rhs_b("cfc", "DDDDNN", n, is_bound, rhsb, d, alpha=-0.3)
    assert np.array_equal(cans.fview(d), p)


def test_reductions(require_gpu):
    import torch
    from cans_gb300 import cans
    n = (20, 18, 16)
    l = (1.0, 2.0, 1.5)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n, l)
    u, v, w, p = _fields(n, 7)
    d = [cans.to_device(x) for x in (u, v, w, p)]
    tot, mx = O.chkdiv(n, l, dli, dzfi, u, v, w)
    tot_g, mx_g = cans.chkdiv(n, l, dli, dzfi_d, d[0], d[1], d[2])
    assert mx_g == mx and abs(tot_g - tot) <= 1e-13 * abs(tot)
    dt = O.chkdt(n, dl, dzci, dzfi, 1e-3, 1e-300, 0, 0, u, v, w)
    dt_g = cans.chkdt(n, dl, dzci_d, dzfi_d, 1e-3, 1e-300, 0, 0, d[0], d[1], d[2])
    assert dt_g == dt
    gvr = torch.tensor(dzf * 0.01, dtype=torch.float64, device="cuda")
    m = O.bulk_mean(n, dzf * 0.01, p)
    assert abs(cans.bulk_mean(n, gvr, d[3]) - m) <= 1e-13 * abs(m) + 1e-16
