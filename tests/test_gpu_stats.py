"""Profile statistics (out1d, out1d_chan, out2d_duct of src/output.f90) on the GPU against
the CPU oracle, and the text files the driver writes from them."""
import os

import numpy as np
import pytest

from gpu_common import grid_for
from oracle import oracle as O

pytestmark = pytest.mark.gpu

N = (20, 12, 9)
L = (2.0, 1.5, 1.0)


def _fields(seed, k=3, mean=1.0):
    rng = np.random.default_rng(seed)
    out = []
    for q in range(k):
        f = O.field(N)
        f[:] = (mean if q == 0 else 0.) + 0.3 * rng.standard_normal(f.shape)
        out.append(np.asfortranarray(f))
    return out


def _close(got, want, tol=1e-12):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape
    for g, w in zip(got.reshape(got.shape[0], -1), want.reshape(want.shape[0], -1)):
        assert np.abs(g - w).max() <= tol * max(1.0, np.abs(w).max())


@pytest.mark.parametrize("idir", [1, 2, 3])
def test_out1d(require_gpu, idir):
    import torch
    from cans_gb300 import cans
    dl = [L[d] / N[d] for d in range(3)]
    dzc, dzf, _, _ = grid_for(N, L, "PPPPNN", 1.4)
    p, = _fields(3, 1)
    want = O.out1d(N, L, dl, idir, dzf, p)
    got = cans.out1d(N, L, dl, idir, torch.tensor(dzf, device="cuda"), cans.to_device(p)).cpu().numpy()
    _close(got[None], want[None])


def test_out1d_chan(require_gpu):
    from cans_gb300 import cans
    dl = [L[d] / N[d] for d in range(3)]
    u, v, w = _fields(4)
    want = O.out1d_chan(N, L, dl, u, v, w)
    got = cans.out1d_chan(N, L, dl, *[cans.to_device(x) for x in (u, v, w)]).cpu().numpy()
    _close(got, want)


@pytest.mark.parametrize("idir", [1, 2])
def test_out2d_duct(require_gpu, idir):
    from cans_gb300 import cans
    dl = [L[d] / N[d] for d in range(3)]
    u, v, w = _fields(5 + idir)
    if idir == 2:
        u, v = v, u  # streamwise velocity with the nonzero mean
    want = O.out2d_duct(N, L, dl, idir, u, v, w)
    got = cans.out2d_duct(N, L, dl, idir, *[cans.to_device(x) for x in (u, v, w)]).cpu().numpy()
    _close(got, want)


def test_unused_directions_compute_nothing(require_gpu):
    """out1d_chan with idir != 3 and out2d_duct with idir = 3 leave the output untouched."""
    import torch
    from cans_gb300 import cans
    dl = [L[d] / N[d] for d in range(3)]
    d = [cans.to_device(x) for x in _fields(9)]
    out = torch.full((8 * N[0] * N[2],), 7.0, dtype=torch.float64, device="cuda")
    for fn, idir in ((cans.lib().cans_out1d_chan, 1), (cans.lib().cans_out2d_duct, 3)):
        rc = fn(cans._ints(N), cans._dbls(L), cans._dbls(dl), idir, *[cans._ptr(x) for x in d], cans._ptr(out), None)
        assert rc == 0
    assert bool((out == 7.0).all())


def test_driver_profile_files(require_gpu, tmp_path):
    """Simulation.out1d writes umean_z/vmean_z/wmean_z/velstats files that read back as the
    oracle's profiles; out0d appends time.out and forcing.out records."""
    from cans_gb300.driver import Simulation
    n = [16, 8, 12]
    case = dict(ng=n, l=[2.0, 1.0, 1.0], gtype=1, gr=1.2, visci=500., cbcvel="PPPPDD" * 3, cbcpre="PPPPNN",
                is_forced=[1, 0, 0], velf=[1., 0., 0.])
    sim = Simulation(case)
    u, v, w = (O.field(n) for _ in range(3))
    for f, seed in ((u, 1), (v, 2), (w, 3)):
        O.add_noise(n, seed, 0.2, f)
    u[1:-1, 1:-1, 1:-1] += 1.0
    sim.set_fields(u, v, w)
    sim.start()
    sim.step(2)
    sim.out1d(str(tmp_path), velstats=True)
    sim.out0d(str(tmp_path))
    from cans_gb300 import cans
    uh, vh, wh = (cans.fview(x) for x in (sim.u, sim.v, sim.w))
    dl = sim.dl
    fld = f"{sim.istep:07d}"
    for name, f, z in (("umean_z", uh, sim.zc), ("vmean_z", vh, sim.zc), ("wmean_z", wh, sim.zf)):
        rows = np.loadtxt(os.path.join(tmp_path, f"{name}_fld_{fld}.out"))
        np.testing.assert_array_equal(rows[:, 0], z[1:n[2] + 1])
        want = O.out1d(n, sim.l, dl, 3, np.asarray(sim.dzf), np.asfortranarray(f))
        assert np.abs(rows[:, 1] - want).max() <= 1e-12 * max(1., np.abs(want).max())
    rows = np.loadtxt(os.path.join(tmp_path, f"velstats_fld_{fld}.out"))
    want = O.out1d_chan(n, sim.l, dl, *[np.asfortranarray(x) for x in (uh, vh, wh)])
    _close(rows[:, 1:].T, want)
    t = np.loadtxt(os.path.join(tmp_path, "time.out"))
    assert t[0] == sim.istep and t[1] == sim.dt and t[2] == sim.time
    fr = np.loadtxt(os.path.join(tmp_path, "forcing.out"))
    assert fr.shape == (7,) and fr[0] == sim.time
    assert abs(fr[4] - 1.0) < 1e-12  # constant flow rate held by the forcing
