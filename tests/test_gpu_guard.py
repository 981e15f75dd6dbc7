"""Guard bands: every caller-owned array a kernel family touches sits inside a larger
allocation whose padding before and after holds a sentinel value; after the calls the padding
must be bit-for-bit unchanged (no write past either end of any field).  compute-sanitizer is
not available on the GPUs these tests run on, so out-of-bounds writes are caught this way."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PAD = 4096


class Guard:
    """Tensors carved out of padded buffers filled with a sentinel."""

    def __init__(self):
        self.bufs = []

    def tensor(self, shape, dtype, fill=None):
        import torch
        n = int(np.prod(shape))
        sentinel = {torch.float32: -7.77e37, torch.float64: -7.77e77}.get(dtype, 0xA5)
        buf = torch.full((PAD + n + PAD,), sentinel, dtype=dtype, device="cuda")
        view = buf[PAD:PAD + n].view(*shape)
        view.zero_() if fill is None else view.copy_(fill)
        self.bufs.append((buf, sentinel))
        return view

    def field(self, n, dtype=None, fill=None):
        import torch
        return self.tensor((n[2] + 2, n[1] + 2, n[0] + 2), dtype or torch.float64, fill)

    def check(self, what):
        import torch
        torch.cuda.synchronize()
        for b, s in self.bufs:
            assert bool((b[:PAD] == s).all()) and bool((b[-PAD:] == s).all()), f"{what}: write outside a field"


def _grid(n, l, cbc="PPPPNN", gr=1.3):
    from oracle import oracle as O
    dzc, dzf, zc, zf = O.initgrid(1, n[2], gr, l[2], cbc[4:6] == "PP")
    return dzc, dzf, zc, zf


def test_guard_fp64_families(require_gpu):
    import torch
    from cans_gb300 import cans
    n, l = [20, 12, 14], [2.0, 1.0, 1.0]
    dl = [l[d] / n[d] for d in range(3)]
    dli = [1. / x for x in dl]
    dzc, dzf, zc, zf = _grid(n, l)
    G = Guard()
    T = lambda a: G.tensor((len(a),), torch.float64, torch.tensor(a, dtype=torch.float64))
    dzci, dzfi = T(1. / dzc), T(1. / dzf)
    vol = l[0] * l[1] * l[2]
    gvr_c, gvr_f = T(dl[0] * dl[1] * dzc / vol), T(dl[0] * dl[1] * dzf / vol)
    rnd = lambda: torch.randn((n[2] + 2, n[1] + 2, n[0] + 2), dtype=torch.float64, device="cuda")
    u, v, w, p, pp = (G.field(n, fill=rnd()) for _ in range(5))
    dto = [G.tensor((n[2], n[1], n[0]), torch.float64) for _ in range(3)]
    work = G.tensor((int(cans.lib().cans_rk_work_doubles(cans._ints(n), 1)),), torch.float64)
    cvel, cpre = "PPPPDD" * 3, "PPPPNN"
    isb = [1, 1, 0, 0, 1, 1]
    cans.initflow("poi", [0.] * 18, n, l, dl, zc, zf, dzc, dzf, 1e-3, [1, 0, 0], [1., 0., 0.], [0.] * 3, True,
                  u, v, w, p)
    G.check("initflow")
    cans.bounduvw(cvel, n, [0.1] * 18, isb, dl, dzc, dzf, u, v, w)
    cans.boundp(cpre, n, [0.] * 6, isb, dl, dzc, p)
    G.check("bounduvw/boundp")
    for impdiff in (0, 1):
        cans.rk((32. / 60., 0.), n, dli, dzci, dzfi, gvr_c, gvr_f, 1e-3, 1e-3, p, [1, 0, 0], [1., 0., 0.],
                [0.1, 0., 0.], impdiff, *dto, u, v, w, work=work)
    G.check("rk")
    cans.fillps(n, dli, dzfi, 100., u, v, w, pp)
    plan = cans.Plan(n, dli, 1. / dzc, 1. / dzf, cpre, [0.] * 6, "ccc")
    cans.updt_rhs_b("ccc", cpre, n, isb, plan.rhsb, pp)
    pp[1:-1, 1:-1, 1:-1] -= pp[1:-1, 1:-1, 1:-1].mean()
    plan.solve(pp)
    plan.solve_adjoint(pp)
    plan.solve_helmholtz(-0.01, isb, pp)
    G.check("fillps/updt_rhs_b/solve")
    cans.correc(n, dli, dzci, 1e-3, pp, u, v, w)
    for impdiff in (0, 1):
        cans.updatep(n, dli, dzci, dzfi, -0.001, impdiff, pp, p)
    G.check("correc/updatep")
    cans.chkdiv(n, l, dli, dzfi, u, v, w)
    cans.chkdt(n, dl, dzci, dzfi, 1e-3, 1e-3, 0, 0, u, v, w)
    cans.bulk_mean(n, gvr_f, u)
    G.check("reductions")
    plan32 = cans.Plan(n, dli, 1. / dzc, 1. / dzf, cpre, [0.] * 6, "ccc", precision=cans.FP32)
    plan32.solve_refined(pp, dli, dzci, dzfi, rtol=0.0, max_iter=2)
    G.check("refined solve")
    gu, gv, gw, gp = (G.field(n, fill=rnd()) for _ in range(4))
    cans.fillps_adjoint(n, dli, dzfi, 100., gp, gu, gv, gw)
    cans.correc_adjoint(n, dli, dzci, 1e-3, gu, gv, gw, gp)
    G.check("adjoints")


def test_guard_fp32_families(require_gpu):
    import torch
    from cans_gb300 import cans
    n, l = [20, 12, 14], [2.0, 1.0, 1.0]
    dl = [l[d] / n[d] for d in range(3)]
    dli = [1. / x for x in dl]
    dzc, dzf, zc, zf = _grid(n, l)
    G = Guard()
    T32 = lambda a: G.tensor((len(a),), torch.float32, torch.tensor(a, dtype=torch.float32))
    dzci, dzfi = T32(1. / dzc), T32(1. / dzf)
    vol = l[0] * l[1] * l[2]
    gvr_c, gvr_f = T32(dl[0] * dl[1] * dzc / vol), T32(dl[0] * dl[1] * dzf / vol)
    rnd = lambda: torch.randn((n[2] + 2, n[1] + 2, n[0] + 2), dtype=torch.float32, device="cuda")
    u, v, w, p, u2, v2, w2 = (G.field(n, torch.float32, rnd()) for _ in range(7))
    pp = G.field(n, torch.float64)
    dto = [G.tensor((n[2], n[1], n[0]), torch.float32) for _ in range(3)]
    nb = int(lib_bytes(n))
    work = G.tensor((nb,), torch.uint8)
    cvel, cpre = "PPPPDD" * 3, "PPPPNN"
    isb = [1, 1, 0, 0, 1, 1]
    cans.bounduvw_f32(cvel, n, [0.1] * 18, isb, dl, dzc, dzf, u, v, w)
    cans.boundp_f32(cpre, n, [0.] * 6, isb, dl, dzc, p)
    G.check("bounds f32")
    cans.rk_f32((32. / 60., 0.), n, dli, dzci, dzfi, gvr_c, gvr_f, 1e-3, 1e-3, p, [1, 0, 0], [1., 0., 0.],
                [0., 0., 0.], *dto, u, v, w, u2, v2, w2, work)
    G.check("rk f32")
    cans.fillps_f32(n, dli, dzfi, 100., u2, v2, w2, pp)
    plan = cans.Plan(n, dli, 1. / dzc, 1. / dzf, cpre, [0.] * 6, "ccc", precision=cans.FP32)
    pp[1:-1, 1:-1, 1:-1] -= pp[1:-1, 1:-1, 1:-1].mean()
    d64 = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    plan.solve_refined(pp, dli, d64(1. / dzc), d64(1. / dzf), rtol=0.0, max_iter=2)
    q = G.field(n, torch.float32, pp.float())
    plan.solve(q)
    G.check("fillps f32 / solves")
    cans.correc_updatep_f32(n, dli, dzci, 1e-3, pp, u2, v2, w2, p)
    cans.correc_f32(n, dli, dzci, 1e-3, pp, u2, v2, w2)
    cans.updatep_f32(n, dli, dzci, dzfi, 0., 0, pp, p)
    G.check("correc/updatep f32")
    cans.chkdiv_f32(n, l, dli, dzfi, u2, v2, w2)
    cans.chkdt_f32(n, dl, dzci, dzfi, 1e-3, 1e-3, 0, 0, u2, v2, w2)
    cans.bulk_mean_f32(n, gvr_f, u2)
    G.check("reductions f32")


def lib_bytes(n):
    from cans_gb300 import cans
    return cans.lib().cans_rk_f32_work_bytes(cans._ints(n), 0)
