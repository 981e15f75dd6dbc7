"""Batched solves (cans_batch_*): boxes of uneven size, the three velocity Helmholtz solves
and the pressure solve of each box in one persistent launch per pass.  Each batched result
must be bit-identical to the single-system call it replaces (those are checked against the
oracle in test_gpu_solver.py), and the Helmholtz solves are also checked against the oracle."""
import numpy as np
import pytest

from gpu_common import grid_for, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# closed boxes: Dirichlet velocity (face-centred along the component), Neumann pressure;
# sizes mix compile-time lengths (32, 64) with generic ones (24, 40, 48, 80)
BOXES = [((32, 48, 40), 1.3), ((48, 32, 24), 1.0), ((64, 40, 32), 1.2), ((40, 64, 48), 0.0), ((80, 32, 32), 1.1)]
CBCVEL = "DDDDDD" * 3
CBCPRE = "NNNNNN"


def _box(n, gr, seed):
    from cans_gb300 import cans
    l = [1.0, 1.0 * n[1] / n[0], 1.0]
    dl = [l[d] / n[d] for d in range(3)]
    dli = [1.0 / x for x in dl]
    dzc, dzf, dzci, dzfi = grid_for(n, l, CBCPRE, gr)
    bcvel = [0.0] * 18
    bcvel[5] = 1.0   # lid: u = 1 at the top z face
    bcvel[6 + 1] = 0.3
    plans = []
    for c in range(3):
        cf = ["c", "c", "c"]
        cf[c] = "f"
        plans.append(cans.Plan(n, dli, dzci, dzfi, CBCVEL[6 * c:6 * c + 6], bcvel[6 * c:6 * c + 6], "".join(cf)))
    plans.append(cans.Plan(n, dli, dzci, dzfi, CBCPRE, [0.0] * 6, "ccc"))
    rng = np.random.default_rng(seed)
    fields = []
    for _ in range(4):
        a = O.field(n)
        a[1:-1, 1:-1, 1:-1] = rng.standard_normal(n)
        fields.append(a)
    return dict(n=n, dli=dli, dzci=dzci, dzfi=dzfi, plans=plans, fields=fields, bcvel=bcvel)


def _setup():
    return [_box(n, gr, 10 + b) for b, (n, gr) in enumerate(BOXES)]


def test_batch_solve_bit_identical_to_single_calls(require_gpu):
    import torch
    from cans_gb300 import cans
    boxes = _setup()
    is_b = [1] * 6
    plans, single, batched, alpha = [], [], [], []
    for b, bx in enumerate(boxes):
        for c in range(4):
            plans.append(bx["plans"][c])
            single.append(cans.to_device(bx["fields"][c]))
            batched.append(cans.to_device(bx["fields"][c]))
            alpha.append(-0.5 * 1e-3 * (b + 1) * (c + 1) if c < 3 else 0.0)
    for pl, f, al in zip(plans, single, alpha):
        if al != 0.0:
            pl.solve_helmholtz(al, is_b, f)
        else:
            cans.updt_rhs_b("ccc", CBCPRE, pl.ng, is_b, pl.rhsb, f)
            pl.solve(f)
    B = cans.Batch(plans)
    B.solve(batched, alpha, [is_b] * len(plans))
    torch.cuda.synchronize()
    for s, (x, y) in enumerate(zip(single, batched)):
        assert torch.equal(x, y), f"system {s} differs"
    # second call: cached work table, same result
    again = [cans.to_device(bx["fields"][c]) for bx in boxes for c in range(4)]
    B.solve(again, alpha, [is_b] * len(plans))
    torch.cuda.synchronize()
    for x, y in zip(single, again):
        assert torch.equal(x, y)


def test_batch_helmholtz_matches_oracle(require_gpu):
    from cans_gb300 import cans
    boxes = _setup()
    is_b = [1] * 6
    plans, fields, alpha, want = [], [], [], []
    for b, bx in enumerate(boxes):
        n = bx["n"]
        for c in range(3):
            pl = bx["plans"][c]
            al = -0.5 * 2e-3 * (b + 1)
            cf = ["c", "c", "c"]
            cf[c] = "f"
            cf = "".join(cf)
            ref = O.initsolver(n, bx["dli"], bx["dzci"], bx["dzfi"], CBCVEL[6 * c:6 * c + 6],
                               bx["bcvel"][6 * c:6 * c + 6], cf)
            p = bx["fields"][c].copy(order="F")
            O.solve_helmholtz(n, ref["normfft"], al, ref["lambdaxy"], ref["a"], ref["b"], ref["c"], ref["rhsb"],
                              is_b, CBCVEL[6 * c:6 * c + 6], cf, p)
            plans.append(pl)
            fields.append(cans.to_device(bx["fields"][c]))
            alpha.append(al)
            want.append(p)
    cans.Batch(plans).solve(fields, alpha, [is_b] * len(plans))
    for f, w in zip(fields, want):
        got = cans.fview(f)
        assert rel_l2(got[1:-1, 1:-1, 1:-1], w[1:-1, 1:-1, 1:-1]) <= 1e-12


def test_batch_poisson_only_and_single_system(require_gpu):
    import torch
    from cans_gb300 import cans
    bx = _box((48, 40, 36), 1.2, 3)
    pl = bx["plans"][3]
    a = cans.to_device(bx["fields"][3])
    b = a.clone()
    pl.solve(a)
    cans.Batch([pl]).solve([b])
    assert torch.equal(a, b)


def test_batch_rejects_duplicate_and_fp32_plans(require_gpu):
    from cans_gb300 import cans
    bx = _box((32, 32, 32), 1.0, 4)
    with pytest.raises(cans.CansError):
        cans.Batch([bx["plans"][3], bx["plans"][3]])
    n = (32, 32, 32)
    _, _, dzci, dzfi = grid_for(n, [1, 1, 1], CBCPRE, 1.0)
    p32 = cans.Plan(n, [32.0] * 3, dzci, dzfi, CBCPRE, [0.0] * 6, "ccc", precision=cans.FP32)
    with pytest.raises(cans.CansError):
        cans.Batch([p32])


def test_autotuned_plans_stay_exact_and_batched_matches(require_gpu):
    """The autotuner may pick another radix order / lines per CTA: the solve must still match
    the oracle, and batched solves must still equal single solves bit for bit."""
    import torch
    from cans_gb300 import cans
    bx = _box((48, 80, 40), 1.2, 7)
    n = bx["n"]
    plans = bx["plans"]
    for pl in plans:
        ms = pl.autotune(force=True)
        assert all(x > 0 for x in ms)
        for d in range(2):
            radix, ncx, spec = pl.shape(d)
            assert ncx >= 1 and (spec == 0 or spec in (32, 64, 128, 256, 512, 1024))
            assert int(np.prod(radix)) > 0
    # pressure plan against the oracle (consistent right-hand side of the singular NN
    # problem, gauge-free comparison)
    ref = O.initsolver(n, bx["dli"], bx["dzci"], bx["dzfi"], CBCPRE, [0.0] * 6, "ccc")
    p = bx["fields"][3].copy(order="F")
    wz = (1.0 / bx["dzfi"])[1:-1][None, None, :] * np.ones(n)
    p[1:-1, 1:-1, 1:-1] -= (p[1:-1, 1:-1, 1:-1] * wz).sum() / wz.sum()
    rhs = p.copy(order="F")
    d = cans.to_device(rhs)
    O.solver(n, ref["normfft"], ref["lambdaxy"], ref["a"], ref["b"], ref["c"], CBCPRE, "ccc", p)
    plans[3].solve(d)
    from gpu_common import gauge_rel_l2
    dzf = 1.0 / bx["dzfi"]
    assert gauge_rel_l2(cans.fview(d)[1:-1, 1:-1, 1:-1], p[1:-1, 1:-1, 1:-1], dzf) <= 1e-12
    # batched == single with the tuned shapes
    alpha = [-1e-3, -2e-3, -3e-3, 0.0]
    is_b = [1] * 6
    single = [cans.to_device(f) for f in bx["fields"]]
    batched = [cans.to_device(f) for f in bx["fields"]]
    for pl, f, al in zip(plans, single, alpha):
        if al != 0.0:
            pl.solve_helmholtz(al, is_b, f)
        else:
            cans.updt_rhs_b("ccc", CBCPRE, pl.ng, is_b, pl.rhsb, f)
            pl.solve(f)
    cans.Batch(plans).solve(batched, alpha, [is_b] * 4)
    torch.cuda.synchronize()
    for x, y in zip(single, batched):
        assert torch.equal(x, y)
