"""Whole time steps on the GPU: the reference's golden vector and field-by-field parity."""
import json
import os

import numpy as np
import pytest

from gpu_common import gauge_rel_l2, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_lid_driven_cavity_golden_gpu(require_gpu):
    """tests/lid_driven_cavity of the reference, 1500 steps on the GPU, rtol 1e-7 vs its fixture."""
    from cans_gb300.driver import Simulation
    from cans_gb300 import cans
    case = json.load(open(os.path.join(GOLD, "ldc_re1000_case.json")))
    ref = np.loadtxt(os.path.join(GOLD, "ldc_re1000_vprofile.txt"))
    sim = Simulation(case)
    sim.start()
    sim.step(case["nstep"])
    n = case["ng"]
    v = cans.fview(sim.v)
    np.testing.assert_allclose(v[1, n[1] // 2 + 1, 1:n[2] + 1], ref[:, 1], rtol=1e-7, atol=0)
    assert sim.divmax < 1e-12


def _tgv_case(n):
    return dict(ng=[n, n, n], l=[2 * np.pi] * 3, gtype=1, gr=0., cfl=0.5, dtmax=1e5, dt_f=-1., visci=1600.,
                icheck=10, cbcvel="PP" * 9, cbcpre="PP" * 3, bcvel=[0.] * 18, bcpre=[0.] * 6)


def _tgv_fields(n, l, dl):
    """initflow 'tgv' (src/initflow.f90:102-117) with the analytic pressure."""
    i = np.arange(1, n + 1)
    xc = (i - .5) * dl / l * 2 * np.pi
    xf = (i - .0) * dl / l * 2 * np.pi
    zc = xc
    u, v, w, p = (O.field([n] * 3) for _ in range(4))
    X, Y, Z = np.meshgrid(xf, xc, zc, indexing="ij")
    u[1:-1, 1:-1, 1:-1] = np.sin(X) * np.cos(Y) * np.cos(Z)
    X, Y, Z = np.meshgrid(xc, xf, zc, indexing="ij")
    v[1:-1, 1:-1, 1:-1] = -np.cos(X) * np.sin(Y) * np.cos(Z)
    X, Y, Z = np.meshgrid(xc, xc, zc, indexing="ij")
    p[1:-1, 1:-1, 1:-1] = (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.) / 16.
    return u, v, w, p


def test_taylor_green_field_by_field(require_gpu):
    """Triperiodic TGV 32^3: every field after 10 steps agrees with the oracle run."""
    from cans_gb300.driver import Simulation
    from cans_gb300 import cans
    n = 32
    case = _tgv_case(n)
    u, v, w, p = _tgv_fields(n, 2 * np.pi, 2 * np.pi / n)
    r = O.Run(case)
    r.u[:] = u; r.v[:] = v; r.w[:] = w; r.p[:] = p
    r.start()
    sim = Simulation(case)
    sim.set_fields(u, v, w, p)
    sim.start()
    assert sim.dt == r.dt
    r.step(10)
    sim.step(10)
    for name in ("u", "v", "w"):
        got = cans.fview(getattr(sim, name))[1:-1, 1:-1, 1:-1]
        want = getattr(r, name)[1:-1, 1:-1, 1:-1]
        assert rel_l2(got, want) < 1e-11, name
    # pressure of a triperiodic problem: defined up to a constant (zero-mode gauge)
    got, want = cans.fview(sim.p)[1:-1, 1:-1, 1:-1], r.p[1:-1, 1:-1, 1:-1]
    assert gauge_rel_l2(got, want, r.grid()["dzf"]) < 1e-11
    assert abs(sim.dt - r.dt) <= 1e-13 * r.dt


@pytest.mark.parametrize("refine", [None, {"rtol": 1e-13, "max_iter": 6}])
def test_channel_forced_field_by_field(require_gpu, refine):
    """Stretched-grid channel with constant flow rate, seeded noise, 5 steps vs the oracle;
    also with the pressure solved on an FP32 plan with FP64 refinement."""
    from cans_gb300.driver import Simulation
    from cans_gb300 import cans
    n = [32, 16, 24]
    case = dict(ng=n, l=[4.0, 2.0, 2.0], gtype=1, gr=1.4, cfl=0.5, dtmax=1e5, dt_f=-1., visci=5600., icheck=2,
                cbcvel="PPPPDD" * 3, cbcpre="PPPPNN", bcvel=[0.] * 18, bcpre=[0.] * 6,
                is_forced=[1, 0, 0], velf=[1., 0., 0.])
    if refine:
        case["pressure_refine"] = refine
    r = O.Run(case)
    zc = r.grid()["zc"]
    u = O.field(n)
    u[1:-1, 1:-1, 1:-1] = (6. * (zc[1:-1] / 2.) * (1. - zc[1:-1] / 2.))[None, None, :]
    v, w, p = O.field(n), O.field(n), O.field(n)
    for f, s in ((u, 1), (v, 2), (w, 3)):
        O.add_noise(n, s, 0.1, f)
    r.u[:] = u; r.v[:] = v; r.w[:] = w
    r.start()
    sim = Simulation(case)
    sim.set_fields(u, v, w, p)
    sim.start()
    r.step(5)
    sim.step(5)
    for name in ("u", "v", "w"):
        got = cans.fview(getattr(sim, name))[1:-1, 1:-1, 1:-1]
        want = getattr(r, name)[1:-1, 1:-1, 1:-1]
        assert rel_l2(got, want) < 1e-11, name
    got, want = cans.fview(sim.p)[1:-1, 1:-1, 1:-1], r.p[1:-1, 1:-1, 1:-1]
    assert gauge_rel_l2(got, want, r.grid()["dzf"]) < 1e-11


@pytest.mark.parametrize("is_impdiff", [0, 1])
def test_buoyant_channel_with_scalar(require_gpu, is_impdiff):
    """Heated channel with a Boussinesq scalar (Dirichlet walls s = 1 / 0), forced flow,
    seeded noise: velocity, pressure and scalar after 4 steps agree with the oracle run."""
    from cans_gb300.driver import Simulation
    from cans_gb300 import cans
    n = [24, 16, 20]
    case = dict(ng=n, l=[3.0, 1.5, 1.0], gtype=1, gr=1.2, cfl=0.5, dtmax=1e5, dt_f=-1., visci=900., icheck=2,
                cbcvel="PPPPDD" * 3, cbcpre="PPPPNN", bcvel=[0.] * 18, bcpre=[0.] * 6,
                is_forced=[1, 0, 0], velf=[1., 0., 0.], is_impdiff=is_impdiff,
                nscal=1, alphai=[600.], cbcscal=["PPPPDD"], bcscal=[[0., 0., 0., 0., 1., 0.]], ssource=[0.3],
                gacc=[0., 0., -9.8], beta=0.02, is_boussinesq_buoyancy=True)
    r = O.Run(case)
    zc = r.grid()["zc"]
    u = O.field(n)
    u[1:-1, 1:-1, 1:-1] = (6. * zc[1:-1] * (1. - zc[1:-1]))[None, None, :]
    v, w, p, s = O.field(n), O.field(n), O.field(n), O.field(n)
    s[1:-1, 1:-1, 1:-1] = (1. - zc[1:-1])[None, None, :]
    for f, seed in ((u, 1), (v, 2), (w, 3), (s, 4)):
        O.add_noise(n, seed, 0.05, f)
    r.u[:] = u; r.v[:] = v; r.w[:] = w; r.s[:] = s
    r.start()
    sim = Simulation(case)
    sim.set_fields(u, v, w, p, scalars=[s])
    sim.start()
    assert abs(sim.dt - r.dt) <= 1e-13 * r.dt
    r.step(4)
    sim.step(4)
    for name in ("u", "v", "w"):
        got = cans.fview(getattr(sim, name))[1:-1, 1:-1, 1:-1]
        want = getattr(r, name)[1:-1, 1:-1, 1:-1]
        assert rel_l2(got, want) < 1e-11, name
    got = cans.fview(sim.scalars[0]["val"])
    assert rel_l2(got, r.s) < 1e-11
    got, want = cans.fview(sim.p)[1:-1, 1:-1, 1:-1], r.p[1:-1, 1:-1, 1:-1]
    assert gauge_rel_l2(got, want, r.grid()["dzf"]) < 1e-11


def test_taylor_green_64_100_steps(require_gpu):
    """The TGV 64^3 protocol: 100 steps field by field against the oracle run (relative L2
    <= 1e-12 per velocity component after step 1; the drift is checked at step 100)."""
    from cans_gb300.driver import Simulation
    from cans_gb300 import cans
    n = 64
    case = _tgv_case(n)
    u, v, w, p = _tgv_fields(n, 2 * np.pi, 2 * np.pi / n)
    r = O.Run(case)
    r.u[:] = u; r.v[:] = v; r.w[:] = w; r.p[:] = p
    r.start()
    sim = Simulation(case)
    sim.set_fields(u, v, w, p)
    sim.start()
    errs = []
    for step in range(100):
        r.step(1)
        sim.step(1)
        if step in (0, 9, 49, 99):
            e = max(rel_l2(cans.fview(getattr(sim, c))[1:-1, 1:-1, 1:-1], getattr(r, c)[1:-1, 1:-1, 1:-1])
                    for c in ("u", "v", "w"))
            errs.append(e)
    print("TGV 64^3 drift (steps 1, 10, 50, 100):", errs)
    assert errs[0] <= 1e-12, errs
    assert errs[-1] <= 1e-12, errs
