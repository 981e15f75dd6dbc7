"""Run-time failure detection of the time loop (src/main.f90:489-510): a too-small time step
or a too-large / NaN divergence stops the run.  The failures are made on the host -- fake
reductions on CPU, or a NaN written into a field before a GPU step -- never by a GPU fault."""
import numpy as np
import pytest


def _bare_sim(monkeypatch, dt_cfl, divtot, divmax, masked=False):
    """A Simulation with no device state whose chkdt/chkdiv return the given values."""
    from cans_gb300 import cans, driver
    sim = driver.Simulation.__new__(driver.Simulation)
    sim.n, sim.l, sim.dl, sim.dli = [4, 4, 4], [1.] * 3, [.25] * 3, [4.] * 3
    sim.dzci = sim.dzfi = sim.u = sim.v = sim.w = None
    sim.visc, sim.alpha_max, sim.is_impdiff = 1e-3, 0., 0
    sim.cfl, sim.dtmax, sim.dt_f = 0.95, 1e5, -1.
    sim.icheck, sim.istep, sim.kill = 1, 7, False
    sim.fp32, sim.small = False, driver.SMALL

    class _Plan:
        def check(self):
            return True
    sim.plan_p = _Plan()
    sim.is_mask_divergence_check = masked
    monkeypatch.setattr(cans, "chkdt", lambda *a, **k: dt_cfl)
    monkeypatch.setattr(cans, "chkdiv", lambda *a, **k: (divtot, divmax))
    return sim


def test_small_matches_reference_definition():
    from cans_gb300.driver import SMALL
    # epsilon(1._dp) * 10**(precision(1._dp)/2) = 2.220446049250313e-16 * 1e7
    assert SMALL == np.finfo(np.float64).eps * 1e7


def test_healthy_step_passes(monkeypatch):
    sim = _bare_sim(monkeypatch, 1e-2, 1e-16, 1e-14)
    sim.check()
    assert not sim.kill and sim.dt == pytest.approx(0.95e-2)


@pytest.mark.parametrize("dt_cfl,divtot,divmax,why", [
    (1e-10, 1e-16, 1e-14, "time step is too small"),
    (1e-2, 1e-16, 1e-6, "maximum divergence is too large"),
    (1e-2, float("nan"), 0., "maximum divergence is too large"),
])
def test_failed_check_kills_the_run(monkeypatch, dt_cfl, divtot, divmax, why):
    from cans_gb300.driver import SimulationAborted
    sim = _bare_sim(monkeypatch, dt_cfl, divtot, divmax)
    with pytest.raises(SimulationAborted, match=why):
        sim.check()
    assert sim.kill
    with pytest.raises(SimulationAborted):
        sim.step(1)  # no further step runs once killed


def test_masked_divergence_check(monkeypatch):
    sim = _bare_sim(monkeypatch, 1e-2, float("nan"), 1.0, masked=True)
    sim.check()  # is_mask_divergence_check skips the divergence abort, as the reference does
    assert not sim.kill


@pytest.mark.gpu
def test_nan_velocity_stops_gpu_run(require_gpu):
    """A NaN written into u on the host side of the loop: the step's divergence check
    (cans_chkdiv -> CANS_ENONFINITE) stops the run at the next check."""
    from cans_gb300 import cans
    from cans_gb300.driver import Simulation, SimulationAborted
    n = [16, 12, 10]
    case = dict(ng=n, l=[2.0, 1.0, 1.0], gtype=1, gr=1.2, cfl=0.5, dtmax=1e5, dt_f=-1., visci=100., icheck=1,
                cbcvel="PPPPDD" * 3, cbcpre="PPPPNN", bcvel=[0.] * 18, bcpre=[0.] * 6)
    sim = Simulation(case)
    sim.start()
    sim.step(1)
    assert not sim.kill
    sim.u[5, 6, 7] = float("nan")
    with pytest.raises(SimulationAborted, match="divergence"):
        sim.step(1)
    assert sim.kill and np.isnan(sim.divtot)
    with pytest.raises(cans.CansError) as e:
        cans.chkdiv(n, sim.l, sim.dli, sim.dzfi, sim.u, sim.v, sim.w)
    assert e.value.status == cans.ENONFINITE


@pytest.mark.gpu
def test_solver_reports_nonfinite_rhs(require_gpu):
    """A NaN (and an Inf) written into the right-hand side: the solve itself stays
    asynchronous, cans_plan_check reports CANS_ENONFINITE once and clears the record."""
    import torch
    from cans_gb300 import cans
    n = [16, 12, 10]
    dli = [8., 12., 10.]
    dzci = dzfi = np.full(n[2] + 2, 10.)
    for prec in (cans.FP64, cans.FP32):
        plan = cans.Plan(n, dli, dzci, dzfi, "PPPPNN", [0.] * 6, "ccc", precision=prec)
        p = cans.field(n)
        p[1:-1, 1:-1, 1:-1] = torch.randn((n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
        p[1:-1, 1:-1, 1:-1] -= p[1:-1, 1:-1, 1:-1].mean()
        plan.solve(p) if prec == cans.FP64 else plan.solve(p.float())
        assert plan.check()
        for bad in (float("nan"), float("inf")):
            q = p.clone()
            q[5, 6, 7] = bad
            plan.solve(q) if prec == cans.FP64 else plan.solve(q.float())
            assert not plan.check()
            assert plan.check()  # the record was cleared


@pytest.mark.gpu
def test_bounded_device_wait_expires(require_gpu):
    """A device wait that nothing releases (an mbarrier no thread arrives on) gives up after
    its limit and the kernel returns; the context stays usable for the next solve.  This is
    the wait of the TMA-tiled z pass, which then reports CANS_ETIMEOUT through
    cans_plan_check; no GPU fault is involved."""
    import torch
    from cans_gb300 import cans
    assert cans.selftest_wait_timeout(20000)
    n = [16, 12, 10]
    plan = cans.Plan(n, [8., 12., 10.], np.full(n[2] + 2, 10.), np.full(n[2] + 2, 10.), "PPPPNN", [0.] * 6,
                     "ccc", precision=cans.FP32)
    p = cans.field(n).float()
    p[1:-1, 1:-1, 1:-1] = torch.randn((n[2], n[1], n[0]), device="cuda")
    p[1:-1, 1:-1, 1:-1] -= p[1:-1, 1:-1, 1:-1].mean()
    plan.solve(p)
    assert plan.check()
