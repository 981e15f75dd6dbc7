"""Scalar transport (rk_scal, src/rk.f90:335-491), scalar forcing (bulk_forcing_s,
src/scal.f90:301-319) and the Boussinesq buoyancy term of rk (src/rk.f90:163-177) on the
GPU against the CPU oracle."""
import numpy as np
import pytest

from gpu_common import grid_for
from oracle import oracle as O

pytestmark = pytest.mark.gpu

N = (12, 10, 8)
L = (1.0, 2.0, 1.5)


def _fields(n, seed, k):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(k):
        f = O.field(n)
        f[:] = rng.standard_normal(f.shape)
        out.append(np.asfortranarray(f))
    return out


def _grid(n=N, l=L, cbc="PPPPNN", gr=1.3):
    dl = [l[d] / n[d] for d in range(3)]
    dzc, dzf, dzci, dzfi = grid_for(n, l, cbc, gr)
    vol = l[0] * l[1] * l[2]
    return dl, [1 / x for x in dl], dzc, dzf, dzci, dzfi, dl[0] * dl[1] * dzc / vol, dl[0] * dl[1] * dzf / vol


def _T(a):
    import torch
    return torch.tensor(a, dtype=torch.float64, device="cuda")


def _cell(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a.transpose(2, 1, 0))).cuda()


@pytest.mark.parametrize("impdiff,forced,source", [(0, 0, 0.0), (0, 1, 0.0), (1, 1, 0.4), (1, 0, -1.1)])
def test_rk_scal_substep(require_gpu, impdiff, forced, source):
    from cans_gb300 import cans
    dl, dli, dzc, dzf, dzci, dzfi, gvr_c, gvr_f = _grid()
    u, v, w, s = _fields(N, 11, 4)
    dso = np.asfortranarray(np.random.default_rng(12).standard_normal(N))
    d = [cans.to_device(x) for x in (u, v, w, s)]
    dso_d = _cell(dso)
    rkpar, dt, alpha, scalf = (32. / 60., -17. / 60.), 0.01, 2.3e-3, 0.75
    f_ref = O.rk_scal(rkpar, N, dli, dzci, dzfi, gvr_f, alpha, dt, u, v, w, forced, scalf, source, impdiff, dso, s)
    work = cans.rk_scal_work(N, impdiff)
    f = cans.rk_scal(rkpar, N, dli, _T(dzci), _T(dzfi), _T(gvr_f), alpha, dt, d[0], d[1], d[2], forced, scalf,
                     source, impdiff, dso_d, d[3], work)
    got = cans.fview(d[3])
    assert np.abs(got - s).max() <= 1e-12 * np.abs(s).max()
    assert np.abs(dso_d.cpu().numpy().transpose(2, 1, 0) - dso).max() <= 1e-12 * np.abs(dso).max()
    assert abs(f - f_ref) <= 1e-12 * max(1.0, abs(f_ref))
    if not forced:
        assert f == 0.0
    # the forcing step that follows the substep (src/main.f90:442-444)
    O.bulk_forcing_s(N, forced, f_ref, s)
    cans.bulk_forcing_s(N, forced, f, d[3])
    assert np.abs(cans.fview(d[3]) - s).max() <= 1e-12 * np.abs(s).max()


@pytest.mark.parametrize("impdiff", [0, 1])
def test_rk_buoyancy(require_gpu, impdiff):
    """rk with the buoyancy term of scalar s; gravity along every direction at once."""
    from cans_gb300 import cans
    dl, dli, dzc, dzf, dzci, dzfi, gvr_c, gvr_f = _grid()
    u, v, w, p, s = _fields(N, 21, 5)
    rng = np.random.default_rng(22)
    dto = [np.asfortranarray(rng.standard_normal(N)) for _ in range(3)]
    d = [cans.to_device(x) for x in (u, v, w, p, s)]
    dto_d = [_cell(x) for x in dto]
    rkpar, forced = (8. / 15., 0.), (1, 0, 0)
    velf, bforce, gacc, beta = (1.0, 0.0, 0.0), (0.1, -0.2, 0.05), (0.3, -9.81, 1.7), 0.21
    f_ref = O.rk_buoy(rkpar, N, dli, dzci, dzfi, gvr_c, gvr_f, 0.01, 1e-3, p, forced, velf, bforce, impdiff, gacc,
                      beta, s, dto[0], dto[1], dto[2], u, v, w)
    f = cans.rk_buoy(rkpar, N, dli, _T(dzci), _T(dzfi), _T(gvr_c), _T(gvr_f), 0.01, 1e-3, d[3], forced, velf,
                     bforce, impdiff, gacc, beta, d[4], dto_d[0], dto_d[1], dto_d[2], d[0], d[1], d[2])
    for g, want in zip(d[:3], (u, v, w)):
        assert np.abs(cans.fview(g) - want).max() <= 1e-12 * np.abs(want).max()
    for g, want in zip(dto_d, dto):
        assert np.abs(g.cpu().numpy().transpose(2, 1, 0) - want).max() <= 1e-12 * np.abs(want).max()
    assert np.allclose(f, f_ref, rtol=1e-12, atol=1e-14)


def test_rk_buoyancy_zero_gravity_is_rk(require_gpu):
    """With gacc = 0 the buoyant substep is bit-identical to the plain rk substep."""
    from cans_gb300 import cans
    dl, dli, dzc, dzf, dzci, dzfi, gvr_c, gvr_f = _grid()
    u, v, w, p, s = _fields(N, 31, 5)
    dto = [np.asfortranarray(np.random.default_rng(32 + i).standard_normal(N)) for i in range(3)]
    outs = []
    for buoy in (False, True):
        d = [cans.to_device(x) for x in (u, v, w, p, s)]
        dto_d = [_cell(x) for x in dto]
        args = ((1. / 3., -0.2), N, dli, _T(dzci), _T(dzfi), _T(gvr_c), _T(gvr_f), 0.01, 1e-3, d[3], (0, 0, 0),
                (0., 0., 0.), (0., 0., 0.), 0)
        if buoy:
            cans.rk_buoy(*args, (0., 0., 0.), 0.5, d[4], *dto_d, d[0], d[1], d[2])
        else:
            cans.rk(*args, *dto_d, d[0], d[1], d[2])
        outs.append([cans.fview(x) for x in d[:3]])
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
