"""Restart checkpoints (src/load.f90:461-589 layout): file content, size check, and the
start/stop determinism of the reference's tests/start_stop (a run restarted from a
checkpoint continues like the uninterrupted run)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_checkpoint_roundtrip_and_layout(require_gpu, tmp_path):
    import torch
    from cans_gb300 import cans
    n = (10, 7, 5)
    rng = np.random.default_rng(3)
    a = np.asfortranarray(rng.standard_normal((n[0] + 2, n[1] + 2, n[2] + 2)))
    d = cans.to_device(a)
    path = tmp_path / "fld_u.bin"
    cans.save_field(path, n, d, 1.25, 42)
    assert os.path.getsize(path) == (n[0] * n[1] * n[2] + 2) * 8
    inner, t, it = cans.read_field_file(path, n)
    assert np.array_equal(inner, a[1:-1, 1:-1, 1:-1]) and t == 1.25 and it == 42
    z = torch.zeros_like(d)
    t, it = cans.load_field(path, n, z)
    assert (t, it) == (1.25, 42)
    got = cans.fview(z)
    assert np.array_equal(got[1:-1, 1:-1, 1:-1], a[1:-1, 1:-1, 1:-1])
    assert np.all(got[0] == 0) and np.all(got[:, 0] == 0) and np.all(got[:, :, -1] == 0)  # ghosts untouched


def test_checkpoint_rejects_wrong_size_and_missing_file(require_gpu, tmp_path):
    import torch
    from cans_gb300 import cans
    n = (6, 5, 4)
    d = torch.zeros((n[2] + 2, n[1] + 2, n[0] + 2), dtype=torch.float64, device="cuda")
    path = tmp_path / "fld_p.bin"
    cans.save_field(path, n, d, 0.0, 0)
    raw = open(path, "rb").read()
    open(path, "wb").write(raw[:-8])  # truncated
    with pytest.raises(cans.CansError) as e:
        cans.load_field(path, n, d)
    assert e.value.status == cans.EINVAL
    with pytest.raises(cans.CansError) as e:
        cans.load_field(tmp_path / "missing.bin", n, d)
    assert e.value.status == cans.EIO
    with pytest.raises(cans.CansError):
        cans.load_field(path, (6, 5, 5), d)  # another grid


def test_start_stop_continues_like_uninterrupted_run(require_gpu, tmp_path):
    """tests/start_stop of the reference: restart from a checkpoint and compare with the run
    that did not stop (fixed dt so the restart's first dt equals the running one)."""
    import torch
    from cans_gb300 import cans
    from cans_gb300.driver import Simulation
    case = dict(ng=[16, 12, 10], l=[1.0, 1.5, 1.0], gtype=1, gr=1.2, visci=400.0, dt_f=2e-3, icheck=0,
                cbcvel="PPDDDD" * 3, bcvel=[0.0] * 18, cbcpre="PPNNNN", bcpre=[0.0] * 6, bforce=[0.5, 0.0, 0.0])
    rng = np.random.default_rng(8)
    init = [np.asfortranarray(0.1 * rng.standard_normal((18, 14, 12))) for _ in range(3)]
    full = Simulation(case)
    full.set_fields(u=init[0], v=init[1], w=init[2])
    full.start()
    full.step(4)
    full.save(str(tmp_path))
    full.step(3)
    rest = Simulation(case)
    rest.start(restart_dir=str(tmp_path))
    assert rest.istep == 4 and rest.time == full.time - 3 * full.dt
    rest.step(3)
    torch.cuda.synchronize()
    for name in ("u", "v", "w", "p"):
        a, b = cans.fview(getattr(full, name))[1:-1, 1:-1, 1:-1], cans.fview(getattr(rest, name))[1:-1, 1:-1, 1:-1]
        assert np.abs(a - b).max() <= 1e-13 * max(np.abs(a).max(), 1e-30), name
