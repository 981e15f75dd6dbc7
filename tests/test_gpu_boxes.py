"""Batched boxes (cans_boxes_*): lid-driven cavities of uneven size with implicit diffusion
and a fixed dt, advanced together by persistent launches and a captured CUDA graph.
Every box must evolve bit-identically to the single-box call sequence (driver.Simulation),
and one box is checked against the oracle's whole-run driver."""
import numpy as np
import pytest

from gpu_common import gauge_rel_l2, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _case(n, gr, re, lid=1.0):
    bcvel = [0.0] * 18
    bcvel[5] = lid  # u at the top z face
    dl = min(1.0 / n[0], 1.0 / n[1], 1.0 / n[2])
    return dict(ng=list(n), l=[1.0, 1.0, 1.0], gtype=1, gr=gr, visci=re, dt_f=0.5 * dl, icheck=0,
                cbcvel="DDDDDD" * 3, bcvel=bcvel, cbcpre="NNNNNN", bcpre=[0.0] * 6, is_impdiff=1)


CASES = [_case((32, 48, 40), 1.2, 400.0), _case((48, 32, 24), 0.0, 1000.0), _case((40, 40, 48), 1.1, 150.0),
         _case((64, 32, 32), 0.0, 700.0)]


def _init(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(3):
        a = np.zeros((n[0] + 2, n[1] + 2, n[2] + 2), order="F")
        a[1:-1, 1:-1, 1:-1] = 0.1 * rng.standard_normal(n)
        out.append(a)
    return out


def _singles(nsteps):
    from cans_gb300 import driver
    sims = []
    for b, c in enumerate(CASES):
        s = driver.Simulation(c)
        u, v, w = _init(c["ng"], 100 + b)
        s.set_fields(u=u, v=v, w=w)
        s.start()
        s.step(nsteps)
        sims.append(s)
    return sims


def _batched(nsteps, use_graph):
    import torch
    from cans_gb300 import cans, driver
    bx = driver.Boxes(CASES)
    for b, c in enumerate(CASES):
        u, v, w = _init(c["ng"], 100 + b)
        for name, a in (("u", u), ("v", v), ("w", w)):
            bx.boxes[b][name].copy_(cans.to_device(a))
    bx.start()
    bx.step(nsteps, use_graph=use_graph)
    bx.synchronize()
    torch.cuda.synchronize()
    return bx


@pytest.mark.parametrize("use_graph,nsteps", [(False, 2), (True, 3)])
def test_boxes_bit_identical_to_single_box_runs(require_gpu, use_graph, nsteps):
    import torch
    sims = _singles(nsteps)
    bx = _batched(nsteps, use_graph)
    if use_graph:
        assert bx.graph_nodes > 0
    for b, s in enumerate(sims):
        for name in ("u", "v", "w", "p", "pp", "dudtrko", "dvdtrko", "dwdtrko"):
            assert torch.equal(getattr(s, name), bx.boxes[b][name]), f"box {b} field {name}"


def test_boxes_match_oracle(require_gpu):
    from cans_gb300 import cans
    c = CASES[1]  # uniform z grid
    nsteps = 3
    run = O.Run(c)
    u, v, w = _init(c["ng"], 101)
    run.u[...] = u
    run.v[...] = v
    run.w[...] = w
    run.start()
    run.step(nsteps)
    bx = _batched(nsteps, True)
    box = bx.boxes[1]
    dzf = run.grid()["dzf"]
    for name in ("u", "v", "w"):
        got = cans.fview(box[name])[1:-1, 1:-1, 1:-1]
        want = getattr(run, name)[1:-1, 1:-1, 1:-1]
        assert rel_l2(got, want) <= 1e-12, name
    got = cans.fview(box["p"])[1:-1, 1:-1, 1:-1]
    assert gauge_rel_l2(got, run.p[1:-1, 1:-1, 1:-1], dzf) <= 1e-12
