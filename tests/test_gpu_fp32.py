"""The FP32 run (FP32 fields and stencils, FP64-accurate pressure correction) against the
oracle.  Inputs are FP32-representable, so both sides start from the same values; the FP32
kernels round at FP32 (unit roundoff 6e-8), hence the FP32-level tolerances."""
import numpy as np
import pytest

from gpu_common import grid_for, is_bound_for, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _fields32(n, seed, k=4):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(k):
        f = O.field(n)
        f[:] = rng.standard_normal(f.shape).astype(np.float32).astype(np.float64)
        out.append(np.asfortranarray(f))
    return out


def _setup(n=(14, 12, 10), l=(1.0, 2.0, 1.5), cbc="PPPPNN", gr=1.3):
    import torch
    dl = [l[d] / n[d] for d in range(3)]
    dli = [1 / x for x in dl]
    dzc, dzf, dzci, dzfi = grid_for(n, l, cbc, gr)
    # the FP32 kernels take FP32 grid arrays; the oracle gets the same (rounded) values
    dzci, dzfi = dzci.astype(np.float32).astype(np.float64), dzfi.astype(np.float32).astype(np.float64)
    T32 = lambda a: torch.tensor(a, dtype=torch.float32, device="cuda")
    return dl, dli, dzc, dzf, dzci, dzfi, T32(dzci), T32(dzfi)


def _dev32(x):
    import torch
    from cans_gb300 import cans
    return cans.to_device(x, dtype=torch.float32)


def _host(t):
    from cans_gb300 import cans
    return cans.fview(t).astype(np.float64)


def test_fillps_f32(require_gpu):
    from cans_gb300 import cans
    n = (14, 12, 10)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n)
    u, v, w, p = _fields32(n, 1)
    d = [_dev32(x) for x in (u, v, w)]
    pd = cans.to_device(p)
    O.fillps(n, dli, dzfi, 7.3, u, v, w, p)
    cans.fillps_f32(n, dli, dzfi_d, 7.3, *d, pd)
    i3 = (slice(1, -1),) * 3
    assert rel_l2(cans.fview(pd)[i3], p[i3]) <= 2e-6


def test_correc_f32(require_gpu):
    from cans_gb300 import cans
    n = (14, 12, 10)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n)
    u, v, w, pp = _fields32(n, 2)
    # an FP64 pp with low-order bits below FP32 resolution
    pp = np.asfortranarray(pp + 1e-9 * np.random.default_rng(0).standard_normal(pp.shape))
    d = [_dev32(x) for x in (u, v, w)]
    ppd = cans.to_device(pp)
    O.correc(n, dli, dzci, 0.013, pp, u, v, w)
    cans.correc_f32(n, dli, dzci_d, 0.013, ppd, *d)
    for g, want in zip(d, (u, v, w)):
        assert np.abs(_host(g) - want).max() <= 4e-7 * np.abs(want).max()


def test_updatep_f32(require_gpu):
    from cans_gb300 import cans
    n = (14, 12, 10)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n)
    pp, p = _fields32(n, 3, 2)
    d = _dev32(p)
    ppd = cans.to_device(pp)
    O.updatep(n, dli, dzci, dzfi, 0., 0, pp, p)
    cans.updatep_f32(n, dli, dzci_d, dzfi_d, 0., 0, ppd, d)
    i3 = (slice(1, -1),) * 3
    assert np.abs(_host(d)[i3] - p[i3]).max() <= 4e-7 * np.abs(p).max()
    with pytest.raises(cans.CansError):
        cans.updatep_f32(n, dli, dzci_d, dzfi_d, -0.1, 1, ppd, d)  # implicit form: not in the FP32 run


@pytest.mark.parametrize("forced", [(0, 0, 0), (1, 0, 0)])
def test_rk_f32(require_gpu, forced):
    """rk + mom_xyz_ad in FP32, out of place and in place (bit-identical), against the FP64
    oracle on the same FP32-representable inputs."""
    import torch
    from cans_gb300 import cans
    n = (14, 12, 10)
    l = (1.0, 2.0, 1.5)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n, l)
    vol = l[0] * l[1] * l[2]
    gvr_c = (dl[0] * dl[1] * dzc / vol).astype(np.float32).astype(np.float64)
    gvr_f = (dl[0] * dl[1] * dzf / vol).astype(np.float32).astype(np.float64)
    u, v, w, p = _fields32(n, 4)
    rng = np.random.default_rng(9)
    dto = [np.asfortranarray(rng.standard_normal(n).astype(np.float32).astype(np.float64)) for _ in range(3)]
    T32 = lambda a: torch.tensor(a, dtype=torch.float32, device="cuda")
    to32 = lambda x: torch.from_numpy(np.ascontiguousarray(x.transpose(2, 1, 0))).to("cuda", torch.float32)
    rkpar = (25. / 60., -17. / 60.)
    velf, bforce = (1.0, 0.3, 0.0), (0.1, -0.2, 0.05)
    ins = [_dev32(x) for x in (u, v, w, p)]
    outs = [cans.field(n, "cuda", torch.float32) for _ in range(3)]
    dto_a = [to32(x) for x in dto]
    f = cans.rk_f32(rkpar, n, dli, dzci_d, dzfi_d, T32(gvr_c), T32(gvr_f), 0.01, 1e-3, ins[3], forced, velf, bforce,
                    *dto_a, ins[0], ins[1], ins[2], *outs, cans.rk_f32_work(n, False))
    # in place on copies
    ip = [x.clone() for x in ins[:3]]
    dto_b = [to32(x) for x in dto]
    f2 = cans.rk_f32(rkpar, n, dli, dzci_d, dzfi_d, T32(gvr_c), T32(gvr_f), 0.01, 1e-3, ins[3], forced, velf,
                     bforce, *dto_b, ip[0], ip[1], ip[2], ip[0], ip[1], ip[2], cans.rk_f32_work(n, True))
    i3 = (slice(1, -1),) * 3
    for a, b in zip(outs, ip):
        assert torch.equal(a[1:-1, 1:-1, 1:-1], b[1:-1, 1:-1, 1:-1])
    for a, b in zip(dto_a, dto_b):
        assert torch.equal(a, b)
    assert np.array_equal(f, f2)
    f_ref = O.rk(rkpar, n, dli, dzci, dzfi, gvr_c, gvr_f, 0.01, 1e-3, p, forced, velf, bforce, 0,
                 dto[0], dto[1], dto[2], u, v, w)
    for g, want in zip(outs, (u, v, w)):
        assert np.abs(_host(g)[i3] - want[i3]).max() <= 1e-6 * np.abs(want).max()
    for g, want in zip(dto_a, dto):
        got = g.cpu().numpy().astype(np.float64).transpose(2, 1, 0)
        assert rel_l2(got, want) <= 1e-5
    assert np.allclose(f, f_ref, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("cbcvel,cbcpre", [("PPDDDD" * 3, "PPNNNN"), ("PPPPDD" * 3, "PPPPNN"),
                                           ("PP" * 9, "PPPPPP"), ("NNDDNN" + "DDNNNN" + "DDDDDD", "NNNNNN")])
def test_bounds_f32(require_gpu, cbcvel, cbcpre):
    """Ghost fills of FP32 fields: copies bit-exact, the BC formulas at FP32 rounding."""
    from cans_gb300 import cans
    n = (8, 7, 6)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n, cbc=cbcpre)
    bcv = list(np.linspace(-0.5, 0.7, 18))
    bcp = list(np.linspace(0.1, 0.6, 6))
    is_bound = is_bound_for(cbcpre)
    u, v, w, p = _fields32(n, 5)
    d = [_dev32(x) for x in (u, v, w, p)]
    O.bounduvw(cbcvel, n, bcv, is_bound, dl, dzc, dzf, u, v, w, False, 2, 2)
    cans.bounduvw_f32(cbcvel, n, bcv, is_bound, dl, dzc, dzf, d[0], d[1], d[2], False, 2, 2)
    O.boundp(cbcpre, n, bcp, is_bound, dl, dzc, p, 2)
    cans.boundp_f32(cbcpre, n, bcp, is_bound, dl, dzc, d[3], 2)
    for g, want in zip(d, (u, v, w, p)):
        assert np.abs(_host(g) - want).max() <= 4e-7 * max(1.0, np.abs(want).max())


def test_reductions_f32(require_gpu):
    from cans_gb300 import cans
    import torch
    n = (20, 18, 16)
    l = (1.0, 2.0, 1.5)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n, l)
    u, v, w, p = _fields32(n, 7)
    d = [_dev32(x) for x in (u, v, w, p)]
    tot, mx = O.chkdiv(n, l, dli, dzfi, u, v, w)
    tot_g, mx_g = cans.chkdiv_f32(n, l, dli, dzfi_d, d[0], d[1], d[2])
    assert abs(mx_g - mx) <= 1e-6 * mx and abs(tot_g - tot) <= 1e-6 * abs(tot)
    dt = O.chkdt(n, dl, dzci, dzfi, 1e-3, 1e-300, 0, 0, u, v, w)
    dt_g = cans.chkdt_f32(n, dl, dzci_d, dzfi_d, 1e-3, 1e-30, 0, 0, d[0], d[1], d[2])
    assert abs(dt_g - dt) <= 1e-6 * dt
    gw = (dzf * 0.01).astype(np.float32).astype(np.float64)
    m = O.bulk_mean(n, gw, p)
    assert abs(cans.bulk_mean_f32(n, torch.tensor(gw, dtype=torch.float32, device="cuda"), d[3]) - m) <= \
        1e-6 * np.abs(p).max() * gw[1:-1].sum() * n[0] * n[1]


def _tgv_case(n, precision):
    return dict(ng=[n, n, n], l=[2 * np.pi] * 3, gtype=1, gr=0., cfl=0.5, dtmax=1e5, dt_f=-1., visci=1600.,
                icheck=5, cbcvel="PP" * 9, cbcpre="PP" * 3, bcvel=[0.] * 18, bcpre=[0.] * 6, precision=precision)


def test_fp32_run_taylor_green(require_gpu):
    """TGV 32^3, 10 steps: the FP32 run against the oracle's FP64 run, per field."""
    from cans_gb300 import cans
    from cans_gb300.driver import Simulation
    from test_gpu_run import _tgv_fields
    n = 32
    u, v, w, p = _tgv_fields(n, 2 * np.pi, 2 * np.pi / n)
    u, v, w, p = (x.astype(np.float32).astype(np.float64) for x in (u, v, w, p))
    r = O.Run(_tgv_case(n, "fp64"))
    r.u[:] = u; r.v[:] = v; r.w[:] = w; r.p[:] = p
    r.start()
    sim = Simulation(_tgv_case(n, "fp32"))
    sim.set_fields(u, v, w, p)
    sim.start()
    assert abs(sim.dt - r.dt) <= 1e-6 * r.dt
    sim.dt, sim.dti = r.dt, 1. / r.dt  # same time step on both sides
    r.step(10)
    sim.step(10)
    errs = {c: rel_l2(_host(getattr(sim, c))[1:-1, 1:-1, 1:-1], getattr(r, c)[1:-1, 1:-1, 1:-1])
            for c in ("u", "v")}
    print("FP32 TGV 32^3 after 10 steps, rel L2 vs oracle:", errs, "divmax", sim.divmax)
    assert max(errs.values()) <= 1e-5, errs
    assert sim.divmax <= 1e-4 and not sim.kill


def test_fp32_run_forced_channel(require_gpu):
    """Stretched channel with constant flow rate, 6 steps: FP32 run vs the oracle's run."""
    from cans_gb300.driver import Simulation
    n = [32, 16, 24]
    case = dict(ng=n, l=[4.0, 2.0, 2.0], gtype=1, gr=1.4, cfl=0.5, dtmax=1e5, dt_f=-1., visci=5600., icheck=3,
                cbcvel="PPPPDD" * 3, cbcpre="PPPPNN", bcvel=[0.] * 18, bcpre=[0.] * 6,
                is_forced=[1, 0, 0], velf=[1., 0., 0.])
    r = O.Run(case)
    zc = r.grid()["zc"]
    u = O.field(n)
    u[1:-1, 1:-1, 1:-1] = (6. * (zc[1:-1] / 2.) * (1. - zc[1:-1] / 2.))[None, None, :]
    v, w, p = O.field(n), O.field(n), O.field(n)
    for f, s in ((u, 1), (v, 2), (w, 3)):
        O.add_noise(n, s, 0.1, f)
    u, v, w = (x.astype(np.float32).astype(np.float64) for x in (u, v, w))
    r.u[:] = u; r.v[:] = v; r.w[:] = w
    r.start()
    sim = Simulation(dict(case, precision="fp32"))
    sim.set_fields(u, v, w, p)
    sim.start()
    sim.dt, sim.dti = r.dt, 1. / r.dt
    r.step(6)
    sim.step(6)
    errs = {c: rel_l2(_host(getattr(sim, c))[1:-1, 1:-1, 1:-1], getattr(r, c)[1:-1, 1:-1, 1:-1])
            for c in ("u", "v", "w")}
    print("FP32 channel after 6 steps, rel L2 vs oracle:", errs, "divmax", sim.divmax)
    assert errs["u"] <= 1e-6 and errs["v"] <= 1e-4 and errs["w"] <= 1e-4, errs
    assert not sim.kill


def test_correc_updatep_fused_equals_separate(require_gpu):
    """cans_correc_updatep_f32 writes exactly what correc_f32 + updatep_f32 write."""
    import torch
    from cans_gb300 import cans
    n = (14, 12, 10)
    dl, dli, dzc, dzf, dzci, dzfi, dzci_d, dzfi_d = _setup(n)
    u, v, w, p = _fields32(n, 12)
    pp = np.asfortranarray(_fields32(n, 13, 1)[0] * 1e-3 + 1e-12)
    a = [_dev32(x) for x in (u, v, w, p)]
    b = [x.clone() for x in a]
    ppd = cans.to_device(pp)
    cans.correc_f32(n, dli, dzci_d, 0.013, ppd, *a[:3])
    cans.updatep_f32(n, dli, dzci_d, dzfi_d, 0., 0, ppd, a[3])
    cans.correc_updatep_f32(n, dli, dzci_d, 0.013, ppd, *b)
    for x, y in zip(a, b):
        assert torch.equal(x, y)
