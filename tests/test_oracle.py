"""The CPU oracle against the reference's golden vector and independent definitions."""
import json
import os

import numpy as np
import pytest
import scipy.fft as sf

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _hc(x):
    n = x.shape[0]
    X = np.fft.rfft(x, axis=0)
    hc = np.zeros_like(x)
    hc[: n // 2 + 1] = X.real[: n // 2 + 1]
    for k in range(1, (n + 1) // 2):
        hc[n - k] = X.imag[k]
    return hc


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 13, 16, 22, 34, 48, 61, 64, 69, 97, 112, 384])
def test_r2r_kinds_match_scipy(n):
    """FFTW r2r semantics (src/fft.f90:260-313 kinds) vs pocketfft and numpy."""
    rng = np.random.default_rng(n)
    x = rng.standard_normal((n, 4))
    cases = [(O.R2HC, _hc(x)), (O.HC2R, None),
             (O.REDFT10, sf.dct(x, 2, axis=0)), (O.REDFT01, sf.dct(x, 3, axis=0)),
             (O.RODFT10, sf.dst(x, 2, axis=0)), (O.RODFT01, sf.dst(x, 3, axis=0)),
             (O.REDFT11, sf.dct(x, 4, axis=0)), (O.RODFT11, sf.dst(x, 4, axis=0)),
             (O.RODFT00, sf.dst(x, 1, axis=0))]
    if n >= 2:
        cases.append((O.REDFT00, sf.dct(x, 1, axis=0)))
    for kind, ref in cases:
        if kind == O.HC2R:
            y = O.r2r(O.HC2R, _hc(x))
            ref = x * n
        else:
            y = O.r2r(kind, x)
        err = np.abs(y - ref).max() / np.abs(ref).max()
        assert err < 5e-15 * max(1.0, np.log2(max(n, 2))), (kind, err)


def test_r2r_direct_sums_long_double():
    """DCT-II / DST-II against O(N^2) sums in extended precision."""
    n = 24
    x = np.random.default_rng(1).standard_normal(n)
    j = np.arange(n, dtype=np.longdouble)
    k = j[:, None]
    pi = np.longdouble(np.pi)
    dct2 = 2 * (np.cos(pi * (2 * j + 1) * k / (2 * n)) * x.astype(np.longdouble)).sum(axis=1)
    dst2 = 2 * (np.sin(pi * (2 * j + 1) * (k + 1) / (2 * n)) * x.astype(np.longdouble)).sum(axis=1)
    assert np.abs(O.r2r(O.REDFT10, x) - dct2.astype(float)).max() < 1e-14
    assert np.abs(O.r2r(O.RODFT10, x) - dst2.astype(float)).max() < 1e-14


def test_eigenvalues_tridmatrix():
    """src/initsolver.f90:85-187 on a few BC pairs."""
    lam = O.eigenvalues(8, "PP", "c")
    assert np.allclose(lam, -2 * (1 - np.cos(2 * np.arange(8) * np.pi / 8)))
    lam = O.eigenvalues(8, "NN", "c")
    assert np.allclose(lam, -2 * (1 - np.cos(np.arange(8) * np.pi / 8)))
    lam = O.eigenvalues(8, "DD", "f")
    assert lam[-1] == 0.0 and np.allclose(lam[:-1], -2 * (1 - np.cos(np.arange(1, 8) * np.pi / 8)))
    dzc, dzf, zc, zf = O.initgrid(1, 16, 1.4, 2.0, False)
    assert abs(zf[16] - 2.0) < 1e-14 and np.all(dzf[1:17] > 0)
    a, b, c = O.tridmatrix("NN", 16, 1 / dzc, 1 / dzf, "c")
    assert b[0] == -c[0] and b[-1] == -a[-1]


def _poisson_residual(n, dli, dzci, dzfi, cbc, p, rhs):
    """lap(p) - rhs on the interior (the operator of src/debug.f90:91-132)."""
    from numpy import s_
    i, j, k = s_[1:n[0] + 1], s_[1:n[1] + 1], s_[1:n[2] + 1]
    lap = ((p[2:, j, k] - 2 * p[i, j, k] + p[:-2, j, k]) * dli[0] ** 2
           + (p[i, 2:, k] - 2 * p[i, j, k] + p[i, :-2, k]) * dli[1] ** 2
           + ((p[i, j, 2:] - p[i, j, k]) * dzci[1:n[2] + 1] - (p[i, j, k] - p[i, j, :-2]) * dzci[0:n[2]])
           * dzfi[1:n[2] + 1])
    return lap - rhs[i, j, k]


@pytest.mark.parametrize("cbc", ["PPPPNN", "PPNNNN", "NNDDPP", "DDNNDD", "PPPPPP"])
def test_solver_inverts_laplacian(cbc):
    """solver() output satisfies the 7-point Poisson equation with the BC ghosts of boundp."""
    n = [12, 10, 9]
    l = [1.3, 0.7, 2.0]
    dl = [l[d] / n[d] for d in range(3)]
    dli = [1 / x for x in dl]
    zper = cbc[4:] == "PP"
    dzc, dzf, zc, zf = O.initgrid(1, n[2], 0.0 if zper else 1.4, l[2], zper)
    dzci, dzfi = 1 / dzc, 1 / dzf
    s = O.initsolver(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc")
    rng = np.random.default_rng(3)
    p = O.field(n)
    p[1:-1, 1:-1, 1:-1] = rng.standard_normal(n)
    if "D" not in cbc:  # compatible RHS: remove the volume-weighted mean
        wts = dzf[1:-1][None, None, :] * np.ones(n)
        p[1:-1, 1:-1, 1:-1] -= (p[1:-1, 1:-1, 1:-1] * wts).sum() / wts.sum()
    rhs = p.copy()
    O.solver(n, s["normfft"], s["lambdaxy"], s["a"], s["b"], s["c"], cbc, "ccc", p)
    is_bound = [1, 1] + [0 if cbc[2 * d:2 * d + 2] == "PP" else 1 for d in (1, 2) for _ in (0, 1)]
    O.boundp(cbc, n, [0.] * 6, is_bound, dl, dzc, p)
    res = _poisson_residual(n, dli, dzci, dzfi, cbc, p, rhs)
    assert np.abs(res).max() < 1e-9 * np.abs(rhs).max() * max(dli) ** 2 / 10


def test_projection_is_divergence_free():
    """src/sanity.f90:206-284: noise velocity -> fillps -> solver -> correc -> chkdiv < small."""
    n = [16, 12, 10]
    l = [1.0, 1.0, 1.0]
    cbcvel = "PPDDDD" * 3
    cbcpre = "PPNNNN"
    dl = [l[d] / n[d] for d in range(3)]
    dli = [1 / x for x in dl]
    dzc, dzf, zc, zf = O.initgrid(1, n[2], 1.2, l[2], False)
    dzci, dzfi = 1 / dzc, 1 / dzf
    s = O.initsolver(n, dli, dzci, dzfi, cbcpre, [0.] * 6, "ccc")
    is_bound = [1, 1, 1, 1, 1, 1]
    u, v, w, p = O.field(n), O.field(n), O.field(n), O.field(n)
    for f, seed in ((u, 123), (v, 456), (w, 789)):
        O.add_noise(n, seed, 0.5, f)
    dt = np.arccos(np.float32(-1.0)).astype(np.float64)
    O.bounduvw(cbcvel, n, [0.] * 18, is_bound, dl, dzc, dzf, u, v, w, False, O.HALO_LOWER)
    O.fillps(n, dli, dzfi, 1 / dt, u, v, w, p)
    O.updt_rhs_b("ccc", cbcpre, n, is_bound, s["rhsb"], p)
    O.solver(n, s["normfft"], s["lambdaxy"], s["a"], s["b"], s["c"], cbcpre, "ccc", p)
    O.boundp(cbcpre, n, [0.] * 6, is_bound, dl, dzc, p)
    O.correc(n, dli, dzci, dt, p, u, v, w)
    O.bounduvw(cbcvel, n, [0.] * 18, is_bound, dl, dzc, dzf, u, v, w, True, O.HALO_UPPER, O.HALO_NONE)
    divtot, divmax = O.chkdiv(n, l, dli, dzfi, u, v, w)
    small = np.finfo(float).eps * 10 ** (np.finfo(float).precision // 2)
    assert divmax < small


def test_lid_driven_cavity_golden():
    """Pin: the reference's own regression (tests/lid_driven_cavity/test.py:5-8), 1500 steps."""
    case = json.load(open(os.path.join(GOLD, "ldc_re1000_case.json")))
    ref = np.loadtxt(os.path.join(GOLD, "ldc_re1000_vprofile.txt"))
    r = O.Run(case)
    r.start()
    r.step(case["nstep"])
    n = case["ng"]
    prof = r.v[1, n[1] // 2 + 1, 1:n[2] + 1]
    np.testing.assert_allclose(r.grid()["zc"][1:n[2] + 1], ref[:, 0], rtol=1e-7)
    np.testing.assert_allclose(prof, ref[:, 1], rtol=1e-7, atol=0)


def test_reference_pivot_rule_misses_stretched_zero_mode():
    """Documents a property of the reference's pin (src/solver.f90:137-147): on the 512-row
    tanh grid (gr = 1.4) of the channel case the last pivot of the lambda = 0 column is
    |den| = O(1e-11) above its tolerance eps*max(|b+lam|,|a*d|), so the constant pressure mode
    is not pinned and its value is set by rounding."""
    dzc, dzf, zc, zf = O.initgrid(1, 512, 1.4, 2.0, False)
    a, b, c = O.tridmatrix("NN", 512, 1 / dzc, 1 / dzf, "c")
    d = c[0] / b[0]
    for k in range(1, 512):
        bl, ad = b[k], a[k] * d
        den = bl - ad
        if k < 511:
            d = c[k] / den
    pt = np.finfo(float).eps * max(abs(bl), abs(ad))
    assert abs(den) > pt  # not pinned by the reference's test
    assert abs(den) < 1e-9 * abs(bl)  # yet numerically singular


def test_scalar_substep_conserves_mean_with_source():
    """rk_scal restatement: with zero velocity and periodic ghosts the volume-weighted mean of
    the scalar changes by exactly f12*ssource (diffusion conserves it), and a forced scalar
    reports f = scalf - mean."""
    n = (8, 6, 5)
    rng = np.random.default_rng(4)
    s = O.field(n)
    s[1:-1, 1:-1, 1:-1] = rng.standard_normal(n)

    def periodic(a):
        a[0], a[-1] = a[-2], a[1]
        a[:, 0], a[:, -1] = a[:, -2], a[:, 1]
        a[:, :, 0], a[:, :, -1] = a[:, :, -2], a[:, :, 1]

    periodic(s)
    z = O.field(n)
    dzci = np.ones(n[2] + 2) * n[2]
    dzfi = np.ones(n[2] + 2) * n[2]
    gvr = np.ones(n[2] + 2) / (n[0] * n[1] * n[2])
    dli = [float(n[0]), float(n[1]), float(n[2])]
    rkpar, dt, src = (32. / 60., 0.), 0.01, 0.7
    mean0 = O.bulk_mean(n, gvr, s)
    dso = np.zeros(n, order="F")
    f = O.rk_scal(rkpar, n, dli, dzci, dzfi, gvr, 0.05, dt, z, z, z, 1, 2.0, src, 0, dso, s)
    mean1 = O.bulk_mean(n, gvr, s)
    assert abs((mean1 - mean0) - rkpar[0] * dt * src) < 1e-14
    assert abs(f - (2.0 - mean1)) < 1e-15


def test_run_with_passive_scalar():
    """Whole-run oracle with one scalar: without buoyancy the velocity is bit-identical to a
    run without the scalar; a uniform scalar with homogeneous Neumann walls stays uniform."""
    n = [8, 6, 10]
    base = dict(ng=n, l=[2.0, 1.0, 2.0], gtype=1, gr=1.2, cfl=0.5, visci=200., icheck=2,
                cbcvel="PPPPDD" * 3, cbcpre="PPPPNN", is_forced=[1, 0, 0], velf=[1., 0., 0.], is_impdiff=1)
    sc = dict(base, nscal=1, alphai=[140.], cbcscal=["PPPPNN"], bcscal=[[0.] * 6], gacc=[0., 0., -1.], beta=0.5)
    runs = [O.Run(base), O.Run(sc)]
    rng = np.random.default_rng(5)
    uyz, vxz = rng.standard_normal((n[1], n[2])), rng.standard_normal((n[0], n[2]))
    for r in runs:  # u(y, z) and v(x, z): discretely divergence-free from the first substep
        r.u[1:-1, 1:-1, 1:-1] = 1.0 + 0.2 * uyz[None, :, :]
        r.v[1:-1, 1:-1, 1:-1] = 0.2 * vxz[:, None, :]
    runs[1].s[1:-1, 1:-1, 1:-1] = 0.7
    for r in runs:
        r.start()
        r.step(3)
    for name in ("u", "v", "w", "p"):
        assert np.array_equal(getattr(runs[0], name), getattr(runs[1], name))
    assert np.abs(runs[1].s[1:-1, 1:-1, 1:-1] - 0.7).max() < 1e-13


def test_fortran_es_format():
    """es24.16e3 records of the reference's text output (src/output.f90:16-17)."""
    from cans_gb300 import output
    assert output.es(1.0) == " 1.0000000000000000E+000"
    assert output.es(-0.5) == "-5.0000000000000000E-001"
    assert output.es(2.0 ** -20) == " 9.5367431640625000E-007"
    assert output.es(-3 * 2.0 ** 1000).endswith("E+301")
    assert output.es(0.0) == " 0.0000000000000000E+000"
    assert output.es(123456.789) == " 1.2345678900000000E+005"
    assert output.record([1.0, 2.0]) == " 1.0000000000000000E+000  2.0000000000000000E+000 "
    assert float(output.es(np.pi)) == float(f"{np.pi:.16e}")


def test_statistics_oracle_identities():
    """out1d of a field constant on planes returns that constant; out1d_chan variances of
    such a field are zero and its uw vanishes with w = 0."""
    n = (6, 5, 4)
    l, dl = (1.0, 2.0, 3.0), (1. / 6, 2. / 5, 3. / 4)
    u, v, w = O.field(n), O.field(n), O.field(n)
    prof = np.arange(n[2] + 2, dtype=float)
    u[:] = prof[None, None, :]
    got = O.out1d(n, l, dl, 3, np.ones(n[2] + 2), u)
    assert np.allclose(got, prof[1:-1], rtol=1e-14)
    st = O.out1d_chan(n, l, dl, u, v, w)
    assert np.allclose(st[0], prof[1:-1], rtol=1e-14)
    assert np.abs(st[3]).max() < 1e-12 and np.abs(st[6]).max() == 0.


@pytest.mark.parametrize("cbc", ["PPPPNN", "PPNNNN", "NNDDNN", "PPPPPP", "DDPPDD"])
def test_extended_residual_refinement(cbc):
    """orc_poisson_residual_ld applies the operator the solver inverts: the residual of an FP64
    oracle solve is at rounding level, and one extended-precision refinement step x + S(r)
    agrees with the dense long-double solve (tests/gpu_common.solve_extended) better than the
    FP64 solve itself (periodic x/y cases; solve_extended handles only those)."""
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    from gpu_common import gauge_rel_l2, grid_for, random_field, rel_l2, singular, solve_extended
    n, l = (12, 10, 64), (4 * np.pi, 2 * np.pi, 2.0)
    dl = [l[d] / n[d] for d in range(3)]
    dli = [1 / x for x in dl]
    dzc, dzf, dzci, dzfi = grid_for(n, l, cbc, 1.4)
    s = O.initsolver(n, dli, dzci, dzfi, cbc, [0.] * 6, "ccc")
    rhs = random_field(n, 3, zero_mean=singular(cbc), dzf=dzf)
    x = rhs.copy(order="F")
    O.solver(n, s["normfft"], s["lambdaxy"], s["a"], s["b"], s["c"], cbc, "ccc", x)
    r = O.poisson_residual_ld(n, dli, cbc, s["a"], s["b"], s["c"], x, rhs)
    i3 = (slice(1, -1),) * 3
    assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(rhs[i3]), np.linalg.norm(r)
    e = O.field(n)
    e[i3] = r
    O.solver(n, s["normfft"], s["lambdaxy"], s["a"], s["b"], s["c"], cbc, "ccc", e)
    xt = x[i3] + e[i3]
    if cbc[:4] == "PPPP" and cbc[4:] != "PP":
        exact, _ = solve_extended(n, dli, s["a"], s["b"], s["c"], rhs[i3])
        cmp = (lambda a, b: gauge_rel_l2(a, b, dzf)) if singular(cbc) else rel_l2
        e64, et = cmp(x[i3], exact), cmp(xt, exact)
        assert et <= max(0.1 * e64, 1e-15), (et, e64)
    # a second step changes nothing measurable
    r2 = O.poisson_residual_ld(n, dli, cbc, s["a"], s["b"], s["c"], np.asfortranarray(np.pad(xt, 1)), rhs)
    assert np.linalg.norm(r2) <= np.linalg.norm(r) + 1e-300
