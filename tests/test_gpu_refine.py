"""FP32 transforms + FP64 refinement against the FP64 oracle (the refined precision form of the solve)."""
import numpy as np
import pytest

from gpu_common import gauge_rel_l2, grid_for, random_field, rel_l2, singular
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = [
    ((64, 48, 32), (4.0, 2.0, 2.0), "PPPPNN", 1.4),
    ((32, 40, 24), (1.0, 2.0, 1.0), "PPNNNN", 1.2),
    ((30, 20, 16), (1.0, 1.0, 1.0), "DDNNDD", 1.1),
    ((16, 16, 16), (6.2831853, 6.2831853, 6.2831853), "PPPPPP", 0.0),
    ((24, 16, 20), (1.0, 1.0, 2.0), "NNDDNN", 1.3),
    ((512, 12, 10), (4.0, 1.0, 2.0), "PPDDNN", 1.3),           # FP32 register-FFT x pass
    ((10, 512, 12), (1.0, 4.0, 2.0), "NNPPNN", 1.3),           # FP32 register-FFT y pass
    ((256, 12, 10), (2.0, 1.0, 2.0), "NNPPNN", 1.3),           # FP32 persistent passes, 256
    ((12, 1024, 6), (1.0, 4.0, 2.0), "PPDDNN", 1.3),           # FP32 persistent passes, 1024
    # the partitioned z pass (the default for few columns): 16-row segments, ragged last
    # segment (37 = 2*16 + 5, 129 = 8*16 + 1), 24 and 32 segments (384, 512 rows: the
    # benchmark grids), Dirichlet z
    ((16, 12, 37), (4.0, 2.0, 2.0), "PPPPNN", 1.4),
    ((8, 8, 129), (4.0, 2.0, 2.0), "PPPPNN", 1.3),
    ((16, 16, 384), (4.0, 2.0, 2.0), "PPNNDD", 1.2),
    ((24, 20, 512), (12.566, 6.283, 2.0), "PPPPNN", 1.4),
    ((22, 26, 16), (1.0, 1.0, 1.0), "PPNNNN", 1.2),           # prime factors 11, 13 (direct-DFT stages)
]


def _setup(n, l, cbc, gr, seed=2):
    from cans_gb300 import cans
    dl = [l[d] / n[d] for d in range(3)]
    dli = [1 / x for x in dl]
    dzc, dzf, dzci, dzfi = grid_for(n, l, cbc, gr)
    ref = O.initsolver(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc")
    p = random_field(n, seed, zero_mean=singular(cbc), dzf=dzf)
    want = p.copy(order="F")
    solve = lambda x: O.solver(n, ref["normfft"], ref["lambdaxy"], ref["a"], ref["b"], ref["c"], cbc, "ccc", x)
    solve(want)
    # accuracy reference: the oracle's FP64 solve plus one refinement step with an
    # extended-precision residual (the FP64 solve alone carries ~1e-11 of rounding error on
    # the ill-conditioned 512-row stretched columns)
    e = O.field(n)
    e[1:-1, 1:-1, 1:-1] = O.poisson_residual_ld(n, dli, cbc, ref["a"], ref["b"], ref["c"], want, p)
    solve(e)
    want[1:-1, 1:-1, 1:-1] += e[1:-1, 1:-1, 1:-1]
    return dl, dli, dzc, dzf, dzci, dzfi, p, want


@pytest.mark.parametrize("n,l,cbc,gr", CASES)
def test_fp32_solve_is_fp32_accurate(require_gpu, n, l, cbc, gr):
    import torch
    from cans_gb300 import cans
    dl, dli, dzc, dzf, dzci, dzfi, p, want = _setup(n, l, cbc, gr)
    plan = cans.Plan(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc", precision=cans.FP32)
    d = cans.to_device(p, dtype=torch.float32)
    plan.solve(d)
    got = cans.fview(d).astype(np.float64)[1:-1, 1:-1, 1:-1]
    w = want[1:-1, 1:-1, 1:-1]
    err = gauge_rel_l2(got, w, dzf) if singular(cbc) else rel_l2(got, w)
    assert err < 1e-4, err


@pytest.mark.parametrize("n,l,cbc,gr", CASES)
def test_refined_reaches_fp64_accuracy(require_gpu, n, l, cbc, gr):
    import torch
    from cans_gb300 import cans
    dl, dli, dzc, dzf, dzci, dzfi, p, want = _setup(n, l, cbc, gr)
    plan = cans.Plan(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc", precision=cans.FP32)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    d = cans.to_device(p)
    it, rr = plan.solve_refined(d, dli, T(dzci), T(dzfi), rtol=1e-14, max_iter=8)
    got = cans.fview(d)[1:-1, 1:-1, 1:-1]
    w = want[1:-1, 1:-1, 1:-1]
    err = gauge_rel_l2(got, w, dzf) if singular(cbc) else rel_l2(got, w)
    # against the extended-precision reference: the flat 1e-12 target of the refined path
    assert err <= 1e-12, (err, it, rr)
    assert it <= 4 and rr <= 1e-14, (it, rr)
    # ghost cells untouched
    g = cans.fview(d)
    assert np.all(g[0] == 0) and np.all(g[:, :, -1] == 0)


def test_refined_matches_fp64_gpu_path(require_gpu):
    """Same RHS through the FP64 plan and the FP32+refinement plan, modulo the constant: the
    back-substitution of the singular column carries the rounding of its last rows into the
    constant, so only the mean-free part is comparable between two algorithms."""
    import torch
    from cans_gb300 import cans
    n, l, cbc, gr = (64, 48, 40), (4.0, 2.0, 2.0), "PPPPNN", 1.4
    dl, dli, dzc, dzf, dzci, dzfi, p, want = _setup(n, l, cbc, gr, seed=9)
    p64 = cans.Plan(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc")
    p32 = cans.Plan(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc", precision=cans.FP32)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    a, b = cans.to_device(p), cans.to_device(p)
    p64.solve(a)
    p32.solve_refined(b, dli, T(dzci), T(dzfi), rtol=1e-14, max_iter=8)
    ga, gb = cans.fview(a)[1:-1, 1:-1, 1:-1], cans.fview(b)[1:-1, 1:-1, 1:-1]
    assert gauge_rel_l2(gb, ga, dzf) <= 1e-12


def test_accuracy_against_extended_precision(require_gpu):
    """A stretched channel column set (512 rows, tanh gr=1.4, the z grid of the 512^3 channel)
    with low-wavenumber x/y modes: the FP64 path and FP32+refinement are both compared with
    an extended-precision solution of the same discrete operator.  Refinement (flux-form
    FP64 residual) is at least as accurate as the plain FP64 path."""
    import torch
    from cans_gb300 import cans
    from gpu_common import solve_extended
    n, l, cbc, gr = (8, 8, 512), (4 * np.pi, 2 * np.pi, 2.0), "PPPPNN", 1.4
    dl, dli, dzc, dzf, dzci, dzfi, p, want = _setup(n, l, cbc, gr, seed=21)
    p64 = cans.Plan(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc")
    p32 = cans.Plan(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc", precision=cans.FP32)
    rhs = p[1:-1, 1:-1, 1:-1].copy()
    exact, _ = solve_extended(n, dli, p64.a, p64.b, p64.c, rhs)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    d64, d32 = cans.to_device(p), cans.to_device(p)
    p64.solve(d64)
    p32.solve_refined(d32, dli, T(dzci), T(dzfi), rtol=1e-15, max_iter=8)
    e64 = gauge_rel_l2(cans.fview(d64)[1:-1, 1:-1, 1:-1], exact, dzf)
    e32 = gauge_rel_l2(cans.fview(d32)[1:-1, 1:-1, 1:-1], exact, dzf)
    print(f"vs extended precision: fp64 path {e64:.2e}, fp32+refinement {e32:.2e}")
    assert e32 <= max(1.5 * e64, 1e-13), (e32, e64)
    assert e32 <= 1e-12


@pytest.mark.parametrize("n,l,cbc,gr", CASES[:3])
def test_fixed_corrections_schedule(require_gpu, n, l, cbc, gr):
    """max_iter = K with rtol = 0: K + 1 FP32 solves, the last correction added by its
    x-backward pass.  The error against the oracle falls with K, two corrections reach the
    FP64 accuracy, and the result equals (bit for bit) the verified run that stops after the
    same corrections (same order of FP64 additions: fold in the residual pass, then add)."""
    import torch
    from cans_gb300 import cans
    dl, dli, dzc, dzf, dzci, dzfi, p, want = _setup(n, l, cbc, gr, seed=5)
    plan = cans.Plan(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc", precision=cans.FP32)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    w = want[1:-1, 1:-1, 1:-1]
    errs = []
    outs = {}
    for k in (0, 1, 2, 3):
        d = cans.to_device(p)
        it, rr = plan.solve_refined(d, dli, T(dzci), T(dzfi), rtol=0.0, max_iter=k)
        assert it == k
        got = cans.fview(d)[1:-1, 1:-1, 1:-1]
        errs.append(gauge_rel_l2(got, w, dzf) if singular(cbc) else rel_l2(got, w))
        outs[k] = d
    assert errs[0] < 1e-4 and errs[1] < errs[0] and errs[2] <= 1e-12, errs
    # a verified run (every residual evaluated) that stops after `it` corrections sums the
    # same corrections in the same order as the fixed schedule with max_iter = it
    d = cans.to_device(p)
    it, rr = plan.solve_refined(d, dli, T(dzci), T(dzfi), rtol=1e-9, max_iter=8)
    assert it in outs and rr <= 1e-9
    assert torch.equal(d, outs[it])


def test_two_corrections_at_least_as_accurate_as_fp64_path(require_gpu):
    """The benchmark's schedule (two corrections, rtol = 0) on a 128^3 channel grid: its
    error against a converged refinement is no larger than the FP64 path's."""
    import torch
    from cans_gb300 import cans
    n, l, cbc, gr = (128, 128, 128), (4.0, 2.0, 2.0), "PPPPNN", 1.4
    dl, dli, dzc, dzf, dzci, dzfi, p, _ = _setup(n, l, cbc, gr, seed=7)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    plan32 = cans.Plan(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc", precision=cans.FP32)
    plan64 = cans.Plan(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc")
    ref, k2, x64 = cans.to_device(p), cans.to_device(p), cans.to_device(p)
    plan32.solve_refined(ref, dli, T(dzci), T(dzfi), rtol=0.0, max_iter=5)
    plan32.solve_refined(k2, dli, T(dzci), T(dzfi), rtol=0.0, max_iter=2)
    plan64.solve(x64)
    i3 = (slice(1, -1),) * 3
    r = cans.fview(ref)[i3]
    e2 = gauge_rel_l2(cans.fview(k2)[i3], r, dzf)
    e64 = gauge_rel_l2(cans.fview(x64)[i3], r, dzf)
    assert e2 <= e64, (e2, e64)


Z_CASES = [CASES[0], CASES[2], CASES[3], CASES[4], CASES[9], CASES[10], CASES[12],
           # many tiles per CTA of the tiled z pass (its buffers cycle through several phases)
           ((256, 128, 16), (4.0, 2.0, 2.0), "PPPPNN", 1.2),
           ((128, 128, 24), (6.2831853, 6.2831853, 6.2831853), "PPPPPP", 0.0),
           # the shapes of the reference's two-dimensional examples: ny = 2 (differentially
           # heated cavity) and nz = 4 (2-D Taylor-Green vortex: two-row z tiles)
           ((128, 2, 128), (1.0, 0.015625, 1.0), "NNPPNN", 0.0),
           ((32, 32, 4), (6.2831853, 6.2831853, 0.125), "PPPPPP", 0.0)]


def _zmodes(plan):
    """the z passes the plan offers: 0 column sweep, 1 partitioned (registers), 2 TMA-tiled"""
    from cans_gb300 import cans
    modes = []
    for mode in (0, 1, 2):
        try:
            plan.set_zpass(mode)
        except cans.CansError as e:
            assert e.status == cans.ENOTSUP
            continue
        assert plan.zpass == mode
        modes.append(mode)
    plan.set_zpass(-1)
    return modes


@pytest.mark.parametrize("n,l,cbc,gr", Z_CASES)
def test_all_z_passes(require_gpu, n, l, cbc, gr):
    """Every z pass of an FP32 plan (column sweep, partitioned, TMA-tiled): each FP32-accurate,
    and the refined solves of each reach the same FP64 accuracy; no bounded wait expires."""
    import torch
    from cans_gb300 import cans
    dl, dli, dzc, dzf, dzci, dzfi, p, want = _setup(n, l, cbc, gr, seed=17)
    plan = cans.Plan(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc", precision=cans.FP32)
    modes = _zmodes(plan)
    assert 0 in modes and 2 in modes  # every case here has a column count divisible by 4
    assert plan.zpass == 2  # the automatic choice
    T = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    w = want[1:-1, 1:-1, 1:-1]
    cmp = (lambda a: gauge_rel_l2(a, w, dzf)) if singular(cbc) else (lambda a: rel_l2(a, w))
    errs = {}
    for mode in modes:
        plan.set_zpass(mode)
        d32 = cans.to_device(p, dtype=torch.float32)
        plan.solve(d32)
        d = cans.to_device(p)
        plan.solve_refined(d, dli, T(dzci), T(dzfi), rtol=0.0, max_iter=3)
        errs[mode] = (cmp(cans.fview(d32).astype(np.float64)[1:-1, 1:-1, 1:-1]), cmp(cans.fview(d)[1:-1, 1:-1, 1:-1]))
        assert plan.check()
    print("z passes (fp32 error, refined error):", errs)
    for mode in modes:
        assert errs[mode][0] < 1e-5 and errs[mode][1] <= 1e-12, errs
    plan.set_zpass(-1)


@pytest.mark.parametrize("cbc,c_or_f", [("PPNNNN", "ccc"), ("PPPPPP", "ccc"), ("PPPPDD", "ccf")])
def test_fp32_helmholtz_all_z_passes(require_gpu, cbc, c_or_f):
    """solve_helmholtz (src/solve_helmholtz.f90:28) on an FP32 plan against the FP64 oracle,
    through every z pass: the shift 1/alpha enters the on-the-fly factors of the partitioned
    and tiled passes (FP32 tolerance 1e-5)."""
    from cans_gb300 import cans
    from gpu_common import is_bound_for
    n, l = (12, 10, 14), (1.0, 1.0, 1.0)
    dl = [l[d] / n[d] for d in range(3)]
    dli = [1 / x for x in dl]
    dzc, dzf, dzci, dzfi = grid_for(n, l, cbc, 1.2 if cbc[4] != "P" else 0.0)
    bc = [0.3, -0.2, 0.5, 1.0, -0.7, 0.25]
    ref = O.initsolver(n, dli, dzci, dzfi, cbc, bc, c_or_f)
    plan = cans.Plan(n, dli, dzci, dzfi, cbc, bc, c_or_f, precision=cans.FP32)
    is_bound = is_bound_for(cbc)
    modes = _zmodes(plan)
    assert 2 in modes
    for mode in modes:
        plan.set_zpass(mode)
        for alpha in (-0.013, -0.021):
            p = random_field(n, 7)
            d = cans.to_device(p)
            O.solve_helmholtz(n, ref["normfft"], alpha, ref["lambdaxy"], ref["a"], ref["b"], ref["c"], ref["rhsb"],
                              is_bound, cbc, c_or_f, p)
            plan.solve_helmholtz(alpha, is_bound, d)
            got = cans.fview(d)
            assert rel_l2(got[1:-1, 1:-1, 1:-1], p[1:-1, 1:-1, 1:-1]) <= 1e-5, (mode, alpha)
