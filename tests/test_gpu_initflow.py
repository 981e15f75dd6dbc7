"""initflow (src/initflow.f90:16-259) on the GPU against the oracle's restatement, and a run
started from it through the driver's `inivel` key."""
import numpy as np
import pytest

from gpu_common import rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = ["zer", "uni", "cou", "poi", "iop", "tbl", "log", "hcl", "hcp", "tgv", "tgw", "ant", "pdc", "hdc"]


@pytest.mark.parametrize("inivel", CASES)
@pytest.mark.parametrize("wallturb", [False, True])
def test_initflow_matches_oracle(require_gpu, inivel, wallturb):
    from cans_gb300 import cans
    if wallturb and inivel not in ("pdc", "hdc", "poi"):
        pytest.skip("the vortex pair is used with the wall-turbulence cases")
    n, l = [24, 16, 20], [3.0, 1.5, 2.0]
    dl = [l[d] / n[d] for d in range(3)]
    dzc, dzf, zc, zf = O.initgrid(1, n[2], 1.3, l[2], False)
    bcvel = [0.] * 18
    bcvel[4], bcvel[5] = 0.3, -0.7  # bcvel(0:1,3,1): the Couette / reversed-Poiseuille walls
    args = (bcvel, n, l, dl, zc, zf, dzc, dzf, 1. / 180., [1, 0, 0], [1.3, 0., 0.], [0.4, 0., 0.], wallturb)
    want = [O.field(n) for _ in range(4)]
    O.initflow(inivel, *args, *want)
    got = [cans.field(n) for _ in range(4)]
    cans.initflow(inivel, *args, *got)
    i3 = (slice(1, -1),) * 3
    for name, g, w in zip("uvwp", got, want):
        g = cans.fview(g)[i3]
        scale = max(np.abs(w[i3]).max(), 1e-300)
        # the oracle's set_mean sums sequentially, the GPU by blocks: ~1e-13 apart
        assert np.abs(g - w[i3]).max() <= 1e-12 * scale, (inivel, name, np.abs(g - w[i3]).max(), scale)


def test_unknown_case_rejected(require_gpu):
    from cans_gb300 import cans
    n = [4, 4, 4]
    dzc, dzf, zc, zf = O.initgrid(1, 4, 0., 1., False)
    f = [cans.field(n) for _ in range(4)]
    with pytest.raises(cans.CansError) as e:
        cans.initflow("xyz", [0.] * 18, n, [1.] * 3, [.25] * 3, zc, zf, dzc, dzf, 1e-3, [0] * 3, [0.] * 3, [0.] * 3,
                      False, *f)
    assert e.value.status == cans.EINVAL


def test_channel_run_from_initflow(require_gpu):
    """A forced channel started by the driver from inivel = 'log' (noise and bulk rescaling
    included) equals, step by step, the oracle's run started from the oracle's initflow."""
    from cans_gb300 import cans
    from cans_gb300.driver import Simulation
    n = [32, 16, 24]
    case = dict(ng=n, l=[4.0, 2.0, 2.0], gtype=1, gr=1.4, cfl=0.5, dtmax=1e5, dt_f=-1., visci=5600., icheck=2,
                cbcvel="PPPPDD" * 3, cbcpre="PPPPNN", bcvel=[0.] * 18, bcpre=[0.] * 6,
                is_forced=[1, 0, 0], velf=[1., 0., 0.], inivel="log")
    r = O.Run(case)
    g = r.grid()
    dl = [case["l"][d] / n[d] for d in range(3)]
    u, v, w, p = (O.field(n) for _ in range(4))
    O.initflow("log", case["bcvel"], n, case["l"], dl, g["zc"], g["zf"], g["dzc"], g["dzf"], 1. / 5600.,
               case["is_forced"], case["velf"], [0.] * 3, False, u, v, w, p)
    r.u[:] = u; r.v[:] = v; r.w[:] = w; r.p[:] = p
    r.start()
    sim = Simulation(case)
    sim.start()
    i3 = (slice(1, -1),) * 3
    assert rel_l2(cans.fview(sim.u)[i3], r.u[i3]) <= 1e-14
    r.step(4)
    sim.step(4)
    for name in ("u", "v", "w"):
        assert rel_l2(cans.fview(getattr(sim, name))[i3], getattr(r, name)[i3]) < 1e-11, name
