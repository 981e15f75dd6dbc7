"""Hand-written adjoints: dot-product tests <F x, y> = <x, F^T y> for every linear
operator of the substep, a Jacobian test of the momentum/RK adjoint against central
differences of the forward kernel, and the gradient of the kinetic energy after several
RK3 steps (checkpointed reverse mode) against central finite differences of the GPU model
and of the oracle (FP64 reference), through a torch.autograd.Function used only here."""
import numpy as np
import pytest

from gpu_common import grid_for, is_bound_for

pytestmark = pytest.mark.gpu


def _rand(shape, seed):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(shape, generator=g, dtype=torch.float64).cuda()


def _dot(a, b):
    return float((a * b).sum())


def _close(x, y, tol):
    return abs(x - y) <= tol * max(abs(x), abs(y), 1e-300)


@pytest.mark.parametrize("n,cbc,c_or_f,gr", [((16, 12, 10), "PPPPNN", "ccc", 1.4), ((12, 10, 9), "NNNNNN", "ccc", 1.2),
                                             ((12, 10, 9), "DDDDDD", "fcc", 1.2), ((12, 10, 9), "DDDDDD", "ccf", 1.3),
                                             ((10, 8, 6), "PPNNPP", "ccc", 0.0), ((12, 10, 8), "PPDDDD", "cfc", 1.1)])
def test_solver_adjoint_dot_product(require_gpu, n, cbc, c_or_f, gr):
    from cans_gb300 import cans
    l = (1.0, 1.3, 2.0)
    dli = [n[d] / l[d] for d in range(3)]
    _, _, dzci, dzfi = grid_for(n, l, cbc, gr)
    plan = cans.Plan(n, dli, dzci, dzfi, cbc, [0.0] * 6, c_or_f)
    shape = (n[2] + 2, n[1] + 2, n[0] + 2)
    x = _rand(shape, 1)
    y = _rand(shape, 2)
    i = (slice(1, -1),) * 3
    sx = x.clone()
    plan.solve(sx)
    sty = y.clone()
    plan.solve_adjoint(sty)
    lhs = _dot(sx[i], y[i])
    rhs = _dot(x[i], sty[i])
    assert _close(lhs, rhs, 1e-11)
    hx = x.clone()
    plan.solve_helmholtz(-0.01, [0] * 6, hx)
    hy = y.clone()
    plan.solve_helmholtz_adjoint(-0.01, hy)
    assert _close(_dot(hx[i], y[i]), _dot(x[i], hy[i]), 1e-11)


def _grid(n, l, cbcpre, gr):
    import torch
    dzc, dzf, dzci, dzfi = grid_for(n, l, cbcpre, gr)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    dl = [l[d] / n[d] for d in range(3)]
    return dl, [1 / x for x in dl], dzc, dzf, T(dzci), T(dzfi)


def test_linear_stencil_adjoints_dot_product(require_gpu):
    from cans_gb300 import cans
    n = (10, 9, 8)
    l = (1.0, 1.2, 1.5)
    dl, dli, dzc, dzf, dzci, dzfi = _grid(n, l, "PPNNNN", 1.3)
    shape = (n[2] + 2, n[1] + 2, n[0] + 2)
    i = (slice(1, -1),) * 3
    u, v, w = (_rand(shape, s) for s in (3, 4, 5))
    gp = _rand(shape, 6)
    # fillps: pp = D(u, v, w) on the interior
    pp = _rand(shape, 7)
    cans.fillps(n, dli, dzfi, 3.0, u, v, w, pp)
    gu, gv, gw = (0 * u for _ in range(3))
    cans.fillps_adjoint(n, dli, dzfi, 3.0, gp, gu, gv, gw)
    assert _close(_dot(pp[i], gp[i]), _dot(u, gu) + _dot(v, gv) + _dot(w, gw), 1e-12)
    # correc: (u, v, w) -= G p over the haloed ranges; linear part in p
    p = _rand(shape, 8)
    z = [0 * u for _ in range(3)]
    cans.correc(n, dli, dzci, 0.07, p, *z)
    lam = [_rand(shape, s) for s in (9, 10, 11)]
    gpc = 0 * p
    cans.correc_adjoint(n, dli, dzci, 0.07, *lam, gpc)
    assert _close(sum(_dot(a, b) for a, b in zip(z, lam)), _dot(p, gpc), 1e-12)
    # boundary fills: linear part (zero boundary values), every mode
    is_bound = is_bound_for("PPNNNN")
    for cbcvel, cbcpre in (("PPDDDD" * 3, "PPNNNN"), ("NNDDNN" + "DDNNNN" + "DDDDDD", "NNNNNN")):
        ib = is_bound_for(cbcpre)
        for keep, hn, ht in ((False, 2, 2), (False, -1, 2), (True, 1, 0)):
            f = [_rand(shape, s) for s in (12, 13, 14)]
            fx = [a.clone() for a in f]
            cans.bounduvw(cbcvel, n, [0.0] * 18, ib, dl, dzc, dzf, *fx, keep, hn, ht)
            g = [_rand(shape, s) for s in (15, 16, 17)]
            gx = [a.clone() for a in g]
            cans.bounduvw_adjoint(cbcvel, n, [0.0] * 18, ib, dl, dzc, dzf, *gx, keep, hn, ht)
            assert _close(sum(_dot(a, b) for a, b in zip(fx, g)), sum(_dot(a, b) for a, b in zip(f, gx)), 1e-12)
        for side in (2, 1):
            q = _rand(shape, 18)
            qx = q.clone()
            cans.boundp(cbcpre, n, [0.0] * 6, ib, dl, dzc, qx, side)
            r = _rand(shape, 19)
            rx = r.clone()
            cans.boundp_adjoint(cbcpre, n, [0.0] * 6, ib, dl, dzc, rx, side)
            assert _close(_dot(qx, r), _dot(q, rx), 1e-12)
    # updatep (explicit): p += pp
    gpp = 0 * p
    cans.updatep_adjoint(n, 0, gp, gpp)
    assert _close(_dot(gpp, pp), _dot(gp[i], pp[i]), 1e-13)
    # updatep (implicit diffusion): p += pp + alpha lap(pp), lap reading the ghost cells of pp
    alpha = -0.037
    po = 0 * p
    cans.updatep(n, dli, dzci, dzfi, alpha, 1, pp, po)
    gpp = 0 * p
    cans.updatep_adjoint(n, 1, gp, gpp, dli, dzci, dzfi, alpha)
    assert _close(_dot(po[i], gp[i]), _dot(pp, gpp), 1e-12)


@pytest.mark.parametrize("impdiff", [0, 1])
def test_rk_adjoint_matches_jacobian(require_gpu, impdiff):
    """<J dx, y> by central differences of cans_rk against <dx, J^T y> from cans_rk_adjoint,
    with explicit and with implicit diffusion (the diffusion then enters the new velocity with
    half the substep weight and stays out of dudtrko)."""
    import torch
    from cans_gb300 import cans
    n = (10, 9, 8)
    l = (1.0, 1.2, 1.5)
    dl, dli, dzc, dzf, dzci, dzfi = _grid(n, l, "PPNNNN", 1.3)
    shape = (n[2] + 2, n[1] + 2, n[0] + 2)
    flat = (n[2], n[1], n[0])
    vol = l[0] * l[1] * l[2]
    T = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    gvr_c, gvr_f = T(dl[0] * dl[1] * dzc / vol), T(dl[0] * dl[1] * dzf / vol)
    rkpar, dt, visc = (25. / 60., -17. / 60.), 0.013, 3e-3
    bforce = np.array([0.2, -0.1, 0.05])
    x = [_rand(shape, s) for s in (20, 21, 22, 23)]  # u, v, w, p
    xd = [_rand(flat, s) for s in (24, 25, 26)]      # dudtrko
    dx = [_rand(shape, s) for s in (27, 28, 29, 30)]
    dxd = [_rand(flat, s) for s in (31, 32, 33)]
    dbf = np.array([0.3, 0.7, -0.4])
    y = [_rand(shape, s) for s in (34, 35, 36)]
    yd = [_rand(flat, s) for s in (37, 38, 39)]
    i = (slice(1, -1),) * 3
    rkwork = torch.empty(int(cans.lib().cans_rk_work_doubles(cans._ints(n), impdiff)), dtype=torch.float64,
                         device="cuda")

    def F(eps):
        a = [t + eps * d for t, d in zip(x, dx)]
        b = [t + eps * d for t, d in zip(xd, dxd)]
        cans.rk(rkpar, n, dli, dzci, dzfi, gvr_c, gvr_f, dt, visc, a[3], (0, 0, 0), (0, 0, 0), bforce + eps * dbf,
                impdiff, b[0], b[1], b[2], a[0], a[1], a[2], work=rkwork)
        return _dot(a[0], y[0]) + _dot(a[1], y[1]) + _dot(a[2], y[2]) + sum(_dot(p, q) for p, q in zip(b, yd))

    eps = 1e-5
    fd = (F(eps) - F(-eps)) / (2 * eps)
    g = [t.clone() for t in y]
    gd = [t.clone() for t in yd]
    gp = torch.zeros(shape, dtype=torch.float64, device="cuda")
    work = cans.rk_adjoint_work(n)
    gbf = cans.rk_adjoint(rkpar, n, dli, dzci, dzfi, dt, visc, x[0], x[1], x[2], g[0], g[1], g[2], gd[0], gd[1], gd[2],
                          gp, work, is_impdiff=impdiff)
    ad = sum(_dot(a, b) for a, b in zip(g, dx[:3])) + _dot(gp, dx[3]) + sum(_dot(a, b) for a, b in zip(gd, dxd)) + \
        float(np.dot(gbf, dbf))
    assert _close(fd, ad, 1e-7), (fd, ad)


# ------------------------------------------------------------------ full gradient check
def _duct_case(n, gr=1.2, dt=0.02):
    return dict(ng=list(n), l=[6.0, 2.0, 2.0], gtype=1, gr=gr, cfl=0.5, dt_f=dt, visci=4410.0, icheck=0,
                cbcvel="PPDDDD" * 3, bcvel=[0.0] * 18, cbcpre="PPNNNN", bcpre=[0.0] * 6, is_impdiff=0,
                is_forced=[0, 0, 0])


def _duct_init(n, seed):
    """perturbed laminar square-duct profile (interior arrays, (n3, n2, n1))"""
    import torch
    y = (np.arange(n[1]) + 0.5) / n[1] * 2 - 1
    z = (np.arange(n[2]) + 0.5) / n[2] * 2 - 1
    prof = 2.25 * np.outer(1 - z ** 2, 1 - y ** 2)[:, :, None] * np.ones(n[0])[None, None, :]
    rng = np.random.default_rng(seed)
    u = prof + 0.1 * rng.uniform(-1, 1, (n[2], n[1], n[0]))
    v = 0.1 * rng.uniform(-1, 1, (n[2], n[1], n[0]))
    w = 0.1 * rng.uniform(-1, 1, (n[2], n[1], n[0]))
    T = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    return T(u), T(v), T(w)


def _make_fn():
    import torch

    class KineticEnergy(torch.autograd.Function):
        """J(u0, v0, w0, bforce) through AdjointRun: forward = the GPU model, backward = the
        hand-written adjoint (gradient-check harness only)."""

        @staticmethod
        def forward(ctx, u0, v0, w0, bf, run, nsteps):
            ctx.run = run
            return torch.tensor(run.forward(u0, v0, w0, bf.tolist(), nsteps), dtype=torch.float64)

        @staticmethod
        def backward(ctx, gj):
            du, dv, dw, dbf = ctx.run.backward()
            g = float(gj)
            return g * du, g * dv, g * dw, g * torch.tensor(dbf, dtype=torch.float64), None, None

    return KineticEnergy


def test_energy_gradient_vs_finite_differences_and_oracle(require_gpu):
    import torch
    from cans_gb300 import cans
    from cans_gb300.adjoint import AdjointRun
    from oracle import oracle as O
    n = (24, 16, 16)
    nsteps = 6
    case = _duct_case(n)
    run = AdjointRun(case, ckpt_every=2)
    u0, v0, w0 = _duct_init(n, 11)
    bf = torch.tensor([0.02, 0.004, -0.003], dtype=torch.float64)
    KE = _make_fn()
    xs = [t.clone().requires_grad_(True) for t in (u0, v0, w0)]
    bfg = bf.clone().requires_grad_(True)
    J = KE.apply(xs[0], xs[1], xs[2], bfg, run, nsteps)
    J.backward()
    grads = [t.grad for t in xs]
    gbf = bfg.grad.numpy()
    # central differences of the GPU model along seeded random directions
    rng = np.random.default_rng(11)
    for e in range(3):
        d = [torch.tensor(rng.standard_normal((n[2], n[1], n[0])), device="cuda") for _ in range(3)]
        ad = sum(_dot(g, di) for g, di in zip(grads, d))
        eps = 1e-5
        jp = run.forward(*[t + eps * di for t, di in zip((u0, v0, w0), d)], bf.tolist(), nsteps)
        jm = run.forward(*[t - eps * di for t, di in zip((u0, v0, w0), d)], bf.tolist(), nsteps)
        fd = (jp - jm) / (2 * eps)
        assert _close(fd, ad, 1e-6), (e, fd, ad)
    for c in range(3):
        db = np.zeros(3)
        db[c] = 1.0
        eps = 1e-5
        jp = run.forward(u0, v0, w0, (bf.numpy() + eps * db).tolist(), nsteps)
        jm = run.forward(u0, v0, w0, (bf.numpy() - eps * db).tolist(), nsteps)
        fd = (jp - jm) / (2 * eps)
        if c == 0:
            assert _close(fd, gbf[c], 1e-6), (c, fd, gbf[c])
        else:
            # a uniform force across the walled directions is a pure gradient, which the
            # projection absorbs: dJ/dbf is zero there, the difference quotient is rounding
            noise = 1e-15 * abs(float(J)) / eps * 100
            assert abs(fd) <= noise and abs(gbf[c]) <= noise, (c, fd, gbf[c])
    # FP64 reference: central differences of the oracle's whole-run driver, one direction
    d = [torch.tensor(rng.standard_normal((n[2], n[1], n[0])), device="cuda") for _ in range(3)]
    ad = sum(_dot(g, di) for g, di in zip(grads, d))

    def oracle_energy(sign, eps=1e-5):
        r = O.Run(dict(case, bforce=bf.tolist()))
        for name, t, di in zip(("u", "v", "w"), (u0, v0, w0), d):
            a = getattr(r, name)
            a[...] = 0.0
            a[1:-1, 1:-1, 1:-1] = (t + sign * eps * di).cpu().numpy().transpose(2, 1, 0)
        r.start()
        r.step(nsteps)
        g = r.grid()
        dxdy = case["l"][0] / n[0] * case["l"][1] / n[1]
        wf = g["dzf"][1:-1][None, None, :] * dxdy
        wc = g["dzc"][1:-1][None, None, :] * dxdy
        i = (slice(1, -1),) * 3
        return 0.5 * float((r.u[i] ** 2 * wf).sum() + (r.v[i] ** 2 * wf).sum() + (r.w[i] ** 2 * wc).sum())

    fd_ref = (oracle_energy(1) - oracle_energy(-1)) / 2e-5
    assert _close(fd_ref, ad, 1e-6), (fd_ref, ad)


def test_energy_gradient_implicit_diffusion(require_gpu):
    """The checkpointed reverse mode through steps with implicit diffusion (rk with the
    diffusion split off, the three velocity Helmholtz solves, updatep with alpha lap(pp)):
    dJ against central differences of the GPU model along seeded directions."""
    import torch
    from cans_gb300.adjoint import AdjointRun
    n = (24, 16, 16)
    nsteps = 4
    case = dict(_duct_case(n, dt=0.04), is_impdiff=1, visci=600.0)
    run = AdjointRun(case, ckpt_every=2)
    u0, v0, w0 = _duct_init(n, 5)
    bf = [0.02, 0.0, 0.0]
    run.forward(u0, v0, w0, bf, nsteps)
    du, dv, dw, dbf = run.backward()
    rng = np.random.default_rng(5)
    for e in range(3):
        d = [torch.tensor(rng.standard_normal((n[2], n[1], n[0])), device="cuda") for _ in range(3)]
        ad = sum(_dot(g, di) for g, di in zip((du, dv, dw), d))
        eps = 1e-5
        jp = run.forward(*[t + eps * di for t, di in zip((u0, v0, w0), d)], bf, nsteps)
        jm = run.forward(*[t - eps * di for t, di in zip((u0, v0, w0), d)], bf, nsteps)
        fd = (jp - jm) / (2 * eps)
        assert _close(fd, ad, 1e-6), (e, fd, ad)
    eps = 1e-5
    jp = run.forward(u0, v0, w0, [bf[0] + eps, 0., 0.], nsteps)
    jm = run.forward(u0, v0, w0, [bf[0] - eps, 0., 0.], nsteps)
    assert _close((jp - jm) / (2 * eps), dbf[0], 1e-6), ((jp - jm) / (2 * eps), dbf[0])
