"""Benchmark: Poisson solves/s and RK3-step Mcell/s at 512^3 on one GB300.

Workload (headline `value`): the Poisson/pressure solve of the reference's
src/solver_gpu.f90 on a 512^3 channel-type grid -- periodic x and y (FFT),
Neumann z walls on a tanh-stretched grid (gr = 1.4), Lx = 4*pi, Ly = 2*pi,
Lz = 2 -- FP64, with a seeded N(0,1) right-hand side (mean removed).  One step
is one in-place solve of the device field (inputs resident in HBM; every field
touched is 1 GB, far larger than the 129 MB L2).  Secondary: one full RK3 time
step (src/main.f90:437-473) of the 512^3 triperiodic Taylor-Green vortex.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference's solver (the
oracle, OpenMP on all host cores) on the same workload: the reference itself is
Fortran + MPI + FFTW and cannot be built on these machines.

Multi-GPU: the solve does not shard without an all-to-all; N ranks run N
independent replicas (weak scaling) and `value` is the total solves/s.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Poisson solves/s & RK3-step Mcell/s at 512^3; FP32+refine vs FP64 at equal error"
N_DEFAULT = 512
L_CH = (4 * np.pi, 2 * np.pi, 2.0)
BYTES_PER_CELL_PASS = 16  # each of the five passes reads and writes one FP64 value per cell



def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_for(kernel, workload):
    """DRAM bytes per launch from a committed ncu summary, if one exists for this kernel+workload."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            t = json.load(f)
        return t.get(workload, {}).get(kernel)
    except Exception:
        return None


def rank_barrier(world):
    """Barrier of the replica ranks around a timed region (no-op on one rank)."""
    if world > 1:
        import torch
        torch.distributed.barrier()


def max_over_ranks(ms, world, device):
    """The slowest rank's time: whole-job throughput is units of all ranks / this time."""
    if world == 1:
        return ms
    import torch
    t = torch.tensor([float(ms)], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_throughput(ms, world):
    """Solves per second of the whole job: world replicas, each one solve per ms."""
    return world / (ms * 1e-3)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", f"cans_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except Exception:
            rows = []
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, val in zip(names, r[3:7]):
                if val.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(rows[0][1]), "reasons": sorted(reasons),
                "samples": len(rows)}


_RHS_CACHE = {}


def host_rhs(n, dzf, seed=20260101):
    """seeded N(0,1) RHS (numpy PCG64) with the volume-weighted mean removed (compatible with
    Neumann z); interior as a C-ordered (n3, n2, n1) array -- the bytes of the device tensor
    interior and of the Fortran array p(1:n1,1:n2,1:n3).  The oracle solves the same values."""
    key = (tuple(n), seed)
    if key not in _RHS_CACHE:
        rng = np.random.default_rng(seed)
        inner = rng.standard_normal((n[2], n[1], n[0]))
        w = np.asarray(dzf)[1:-1][:, None, None]
        inner -= (inner * w).sum() / (w.sum() * n[0] * n[1])
        _RHS_CACHE.clear()
        _RHS_CACHE[key] = inner
    return _RHS_CACHE[key]


def make_rhs(n, dzf, device, seed=20260101):
    """the host_rhs values in a haloed device field"""
    import torch
    from cans_gb300 import cans
    p = cans.field(n, device)
    p[1:-1, 1:-1, 1:-1] = torch.from_numpy(host_rhs(n, dzf, seed)).to(device)
    return p


def bench_fp64(args, n, dli, dzc, dzf, dev, world):
    """The plain FP64 path: K in-place solves of the channel RHS (inputs resident)."""
    import torch
    from cans_gb300 import cans
    plan = cans.Plan(n, dli, 1. / dzc, 1. / dzf, "PPPPNN", [0.] * 6, "ccc")
    p = make_rhs(n, dzf, dev)
    ncell = n[0] * n[1] * n[2]
    for _ in range(args.warmup):
        plan.solve(p)
    torch.cuda.synchronize()
    rank_barrier(world)
    plan.set_timing(True)
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(args.steps):
        plan.solve(p)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    pass_ms, nrec = plan.get_timing()
    plan.set_timing(False)
    ms = max_over_ranks(ms, world, dev)
    names = ["solve_xfwd", "solve_yfwd", "solve_zthomas", "solve_ybwd", "solve_xbwd"]
    top = int(np.argmax(pass_ms))
    hbm, kind = peaks()
    achieved = BYTES_PER_CELL_PASS * ncell / (pass_ms[top] * 1e-3) / 1e9
    workload = f"poisson_{n[0]}x{n[1]}x{n[2]}_PPPPNN_fp64"
    roof = {"bound": "hbm", "kernel": names[top], "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
            "frac": round(achieved / hbm, 4), "peak_source": kind, "traffic": traffic_for(names[top], workload),
            "algorithmic_bytes_per_launch": BYTES_PER_CELL_PASS * ncell,
            "note": "FP64-pipe bound on GB300 (1.2 TFLOP/s FP64): 72% FP64 pipe busy in the transform passes"}
    return plan, p, {"value": round(job_throughput(ms, world), 4), "unit": "solves/s", "ms_per_step": round(ms, 4),
                     "pass_ms": {k: round(v, 4) for k, v in zip(names, pass_ms)}, "roofline": roof}


def bench_ours(args, rank, world):
    import torch
    from cans_gb300 import cans
    from cans_gb300.driver import initgrid
    dev = f"cuda:{rank % max(1, torch.cuda.device_count())}"
    torch.cuda.set_device(dev)
    n = [args.size] * 3
    dl = [L_CH[d] / n[d] for d in range(3)]
    dli = [1. / x for x in dl]
    dzc, dzf, zc, zf = initgrid(1, n[2], 1.4, L_CH[2], False)
    if args.skip_fp64 or args.only == "refined":  # profiling aid: only the FP32 + refinement leg
        return {"fp32_refined": bench_refined(args, n, dli, dzc, dzf, None, None, dev, world)}
    if args.only == "rk3":
        return {"rk3_step": bench_rk3(args.size, dev, 20)}
    if args.only == "rk3-fp32":  # profiling aid: the FP32 run of the TGV only
        return {"rk3_step_fp32": bench_rk3(args.size, dev, max(1, args.steps), legs=("fp32_run",))}
    if args.only == "fp32-solve":  # profiling aid: plain FP32 solves (the passes of the refinement)
        return {"fp32_solve": bench_fp32_solve(args, n, dli, dzc, dzf, dev)}
    if args.only == "mx":
        return {"poisson_mx": bench_mx(args, dev, world)}
    if args.only == "mx-run":
        return {"channel_mx_run": bench_mx_run(dev)}
    if args.only == "ch":
        return {"channel_ch": bench_ch(dev)}
    if args.only == "adjoint":
        return {"adjoint_duct": bench_adjoint(dev, nsteps=args.adjoint_steps, ndir=args.adjoint_dirs)}
    if args.only == "boxes":
        return {"batched_boxes": bench_boxes(max(args.boxes, 1), dev, max(1, min(args.steps, 5)),
                                             unbatched_boxes=0)}
    ncell = n[0] * n[1] * n[2]
    workload = f"poisson_{n[0]}x{n[1]}x{n[2]}_PPPPNN"
    plan64, p64, fp64 = bench_fp64(args, n, dli, dzc, dzf, dev, world)
    # headline: FP32 transforms + FP64 refinement at the FP64 path's accuracy
    with Clocks(torch.cuda.current_device()) as clk:
        ref = bench_refined(args, n, dli, dzc, dzf, plan64, p64, dev, world, e2e=True)
    del p64, plan64
    torch.cuda.empty_cache()
    sols = None
    if rank == 0 and not args.skip_cpu:
        # the solutions of the headline RHS, compared with the oracle's in the CPU leg
        sols = gpu_solutions(n, dli, dzc, dzf, dev, ref["corrections_per_solve"])
    hbm, kind = peaks()
    # dominant kernel of the refined solve (largest share of the launch list): the
    # double-float residual k_dfres, timed per launch by CUDA events on the plan's stream
    # inside the timed region; algorithmic bytes per launch = mean bytes/cell x cells
    res_bytes = ref["residual_bytes_per_cell"] * ncell
    achieved = res_bytes / (ref["residual_ms"] * 1e-3) / 1e9
    y_ms = 0.5 * (ref["fp32_pass_ms"]["solve_yfwd"] + ref["fp32_pass_ms"]["solve_ybwd"])
    roof = {"bound": "hbm", "kernel": "k_dfres (double-float residual of the refinement)",
            "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 4),
            "peak_source": kind, "traffic": traffic_for("residual", workload + "_fp32"),
            "algorithmic_bytes_per_launch": int(res_bytes), "kernel_ms": ref["residual_ms"],
            "next_kernel": {"kernel": "k_ylines_pt<512> (FP32 y transform, TMA-fed, in place)",
                            "achieved": round(8 * ncell / (y_ms * 1e-3) / 1e9, 1), "kernel_ms": round(y_ms, 4),
                            "algorithmic_bytes_per_launch": 8 * ncell,
                            "traffic": traffic_for("solve_y_fp32", workload + "_fp32")},
            "solve_passes_ms": ref["fp32_pass_ms"]}
    mx = None
    if not args.skip_mx and world == 1:
        torch.cuda.empty_cache()
        mx = bench_mx(args, dev, world)
    ch = None
    if not args.skip_ch and world == 1:
        torch.cuda.empty_cache()
        ch = bench_ch(dev)
    rk3 = None
    if not args.skip_rk3:
        torch.cuda.empty_cache()
        rk3 = bench_rk3(args.size, dev, 20)  # the TGV protocol: 3 warm-up + 20 timed steps
    mx_run = None
    if not args.skip_mx and world == 1:
        torch.cuda.empty_cache()
        mx_run = bench_mx_run(dev)
    out = {"metric": METRIC, "value": ref["value"], "unit": "solves/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ref["ms_per_step"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64 (FP32 transforms, FP64 residual/z/reductions)",
           "data": "synthetic (seeded N(0,1) RHS, mean removed)",
           "config": {"workload": workload, "grid": n, "bc_pressure": "PP,PP,NN",
                      "z_grid": "tanh gr=1.4", "domain": [round(x, 6) for x in L_CH],
                      "precision": "FP32 solve + FP64 iterative refinement, accuracy <= FP64 path",
                      "l2": "working set 2+ GB per solve >> 129 MB L2 (no flush needed)",
                      "parallelism": f"replicas x{world}"},
           "e2e": ref.pop("e2e"), "roofline": roof, "clocks": clk.summary(), "gpu_launches": ref["gpu_launches"],
           "fp32_refined": ref, "fp64_path": fp64,
           "speedup_refined_over_fp64": round(ref["value"] / fp64["value"], 3)}
    if sols is not None:
        out["_gpu_solutions"] = sols
    if rk3:
        out["rk3_step"] = rk3
    if mx:
        out["poisson_mx"] = mx
    if mx_run:
        out["channel_mx_run"] = mx_run
    if ch:
        out["channel_ch"] = ch
    if not args.skip_adjoint:
        torch.cuda.empty_cache()
        out["adjoint_duct"] = bench_adjoint(dev, nsteps=args.adjoint_steps, ndir=args.adjoint_dirs)
    if args.boxes > 0:
        torch.cuda.empty_cache()
        out["batched_boxes"] = bench_boxes(args.boxes, dev, max(1, min(args.steps, 5)),
                                           unbatched_boxes=min(args.boxes, 32))
    return out


def channel_case(n, l, dt_f=-1., precision="fp64", refine=False):
    """The channel of the CH / MX configurations: tanh z (gr = 1.4), no-slip walls at z = 0, Lz,
    periodic x/y, Re_b = 5600 (visc = 1/5600), constant flow rate U_b = 1, explicit diffusion"""
    case = dict(ng=list(n), l=list(l), gtype=1, gr=1.4, cfl=0.95, dtmax=1e5, dt_f=dt_f, visci=5600., icheck=10,
                cbcvel="PPPPDD" * 3, cbcpre="PPPPNN", bcvel=[0.] * 18, bcpre=[0.] * 6, is_forced=[1, 0, 0],
                velf=[1., 0., 0.], precision=precision)
    if refine:
        case["pressure_refine"] = {"rtol": 0.0, "max_iter": 2}
    return case


def channel_init(sim, seed=20260101):
    """initflow 'poi' (src/initflow.f90:56-58): the laminar profile 6 z/Lz (1 - z/Lz) U_b plus
    seeded uniform(-0.1, 0.1) U_b perturbations with their mean removed, rounded to FP32 so
    that the FP64 and FP32 runs start from the same values"""
    import torch
    n = sim.n
    dev = sim.u.device
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    zc = torch.tensor(sim.zc[1:-1], device=dev, dtype=torch.float64) / sim.l[2]

    def noise():
        x = 0.2 * (torch.rand((n[2], n[1], n[0]), generator=g, device=dev, dtype=torch.float64) - 0.5)
        return x - x.mean()

    vals = [(6. * zc * (1. - zc))[:, None, None] + noise(), noise(), noise()]
    for fld, x in zip((sim.u, sim.v, sim.w), vals):
        fld[1:-1, 1:-1, 1:-1] = x.float().double().to(fld.dtype)


def run_and_time(sim, warm, steps):
    """warm untimed steps, then `steps` steps timed with CUDA events on the current stream"""
    import torch
    from cans_gb300 import cans
    sim.step(warm)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = cans.launch_count()
    e0.record(st)
    sim.step(steps)
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, (cans.launch_count() - l0) // max(steps, 1)


def field_errors(sim, ref):
    """relative L2 of u, v, w and of the mean-free p of `sim` against the saved fields `ref`"""
    import torch
    out = {}
    for name in ("u", "v", "w", "p"):
        a = getattr(sim, name)[1:-1, 1:-1, 1:-1].double()
        b = ref[name]
        if name == "p":
            a, b = a - a.mean(), b - b.mean()
        out[name] = float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
    return out


def channel_legs(n, l, dev, warm, steps):
    """The FP64 run, the FP64 run with the refined FP32 pressure solve and the FP32 run of the
    channel, each `warm` + `steps` RK3 steps at one fixed dt (0.8 x the CFL-0.95 step of the
    initial field), with the per-field error of the other two against the FP64 run"""
    import torch
    from cans_gb300 import cans
    from cans_gb300.driver import Simulation
    ncell = n[0] * n[1] * n[2]
    sim = Simulation(channel_case(n, l), device=dev)
    channel_init(sim)
    sim.start()
    dt = 0.8 * sim.dt
    del sim
    torch.cuda.empty_cache()
    out, ref = {}, None
    for leg, prec, refine in (("fp64", "fp64", False), ("fp64_refined_pressure", "fp64", True),
                              ("fp32_run", "fp32", False)):
        sim = Simulation(channel_case(n, l, dt, prec, refine), device=dev)
        channel_init(sim)
        sim.start()
        ms, launches = run_and_time(sim, warm, steps)
        r = {"ms_per_step": round(ms, 3), "Mcell_steps_per_s": round(ncell / (ms * 1e-3) / 1e6, 2),
             "gpu_launches_per_step": launches}
        if prec == "fp32":
            r["precision"] = "FP32 fields and stencils, pressure correction FP32 solve + 2 FP64 refinement corrections"
            ub = cans.bulk_mean_f32(n, sim.gvr_f32, sim.u)
            divtot, divmax = cans.chkdiv_f32(n, sim.l, sim.dli, sim.dzfi32, sim.u, sim.v, sim.w)
        else:
            ub = cans.bulk_mean(n, sim.gvr_f, sim.u)
            divtot, divmax = cans.chkdiv(n, sim.l, sim.dli, sim.dzfi, sim.u, sim.v, sim.w)
        r.update({"bulk_velocity": ub, "divmax": divmax, "time": sim.time})
        if ref is None:
            ref = {name: getattr(sim, name)[1:-1, 1:-1, 1:-1].clone() for name in ("u", "v", "w", "p")}
        else:
            r["rel_l2_vs_fp64_run"] = field_errors(sim, ref)
        out[leg] = r
        del sim
        torch.cuda.empty_cache()
    del ref
    torch.cuda.empty_cache()
    out["dt"] = dt
    return out


def bench_ch(dev, steps=200):
    """The channel run (CH): 512 x 256 x 256, Lx = 4 pi, Ly = 2 pi, Lz = 2, tanh z (gr 1.4),
    Re_b 5600, constant flow rate, Poiseuille + uniform(-0.1, 0.1) noise; `steps` timed RK3
    steps after 3 warm-up steps: FP64, FP64 with the refined FP32 pressure solve, and the FP32
    run (per-field error of the latter two against the FP64 run after all steps)."""
    n = [512, 256, 256]
    out = {"workload": "channel_512x256x256_Reb5600_rk3", "steps": steps, "warmup_steps": 3}
    out.update(channel_legs(n, L_CH, dev, 3, steps))
    return out


def bench_mx_run(dev, steps=10):
    """The mixed-precision channel (MX): 1024 x 512 x 384, the CH geometry and flow; `steps`
    timed RK3 steps after 3 warm-up steps of the FP64 run and of the FP32 run (FP32 fields
    and stencils, FP64-accurate refined pressure), with the FP32 run's per-field error."""
    n = [1024, 512, 384]
    out = {"workload": "channel_1024x512x384_Reb5600_rk3", "steps": steps, "warmup_steps": 3}
    out.update(channel_legs(n, L_CH, dev, 3, steps))
    return out


def bench_fp32_solve(args, n, dli, dzc, dzf, dev):
    """Plain FP32 solves (cans_solver_f32) of the headline RHS rounded to FP32: the five FP32
    passes the refinement runs, for profiling them on their own"""
    import torch
    from cans_gb300 import cans
    plan = cans.Plan(n, dli, 1. / dzc, 1. / dzf, "PPPPNN", [0.] * 6, "ccc", precision=cans.FP32)
    src = make_rhs(n, dzf, dev).float()
    p = src.clone()
    for _ in range(args.warmup):
        p.copy_(src)
        plan.solve(p)
    torch.cuda.synchronize()
    plan.set_timing(True)
    for _ in range(args.steps):
        p.copy_(src)
        plan.solve(p)
    pass_ms, nrec = plan.get_timing()
    plan.set_timing(False)
    names = ["solve_xfwd", "solve_yfwd", "solve_zthomas", "solve_ybwd", "solve_xbwd"]
    return {"pass_ms": {k: round(v, 4) for k, v in zip(names, pass_ms)}, "solves": nrec}


def bench_mx(args, dev, world):
    """The 1024 x 512 x 384 channel (same BCs, tanh z and domain as the headline): FP64 path
    and FP32 + refinement (corrections calibrated as in the headline, accuracy checked)."""
    import torch
    from cans_gb300.driver import initgrid
    n = [1024, 512, 384]
    dl = [L_CH[d] / n[d] for d in range(3)]
    dli = [1. / x for x in dl]
    dzc, dzf, zc, zf = initgrid(1, n[2], 1.4, L_CH[2], False)
    a = argparse.Namespace(**vars(args))
    a.steps, a.warmup = max(3, min(args.steps, 5)), 3
    plan64, p64, fp64 = bench_fp64(a, n, dli, dzc, dzf, dev, world)
    ref = bench_refined(a, n, dli, dzc, dzf, plan64, p64, dev, world)
    del plan64, p64
    torch.cuda.empty_cache()
    return {"workload": "poisson_1024x512x384_PPPPNN", "unit": "solves/s",
            "fp32_refined": {k: ref[k] for k in ("value", "ms_per_step", "corrections_per_solve", "accuracy",
                                                 "fp32_pass_ms", "residual_ms")},
            "fp64_path": {k: fp64[k] for k in ("value", "ms_per_step", "pass_ms")},
            "speedup_refined_over_fp64": round(ref["value"] / fp64["value"], 3)}


def residual_bytes(k):
    """Mean algorithmic bytes per cell of the k residual launches of a fixed k-correction
    refinement: every launch reads the correction e (4 B), the residual hi/lo (8 B; the
    first reads the FP64 rhs instead, 8 B) and writes hi/lo (8 B); a launch that folds two
    pending corrections into x adds 4 B (the older correction), 8 B written (x) and, when
    x already holds corrections, 8 B read."""
    npend, has_x, tot = 1, False, 0
    for j in range(k):
        b = 20
        if npend == 2:
            b += 12 + (8 if has_x else 0)
            has_x, npend = True, 0
        tot += b
        npend += 1
    return tot / k


def bench_refined(args, n, dli, dzc, dzf, plan64, p64, dev, world, e2e=False):
    """FP32 plan + cans_solver_refined at the accuracy of the FP64 path.

    The number of corrections K is calibrated once per operator by a verified run
    (stop at ||r|| <= rtol ||rhs||); the timed solves then use max_iter = K with the last
    correction added by its own x-backward pass (no final residual).  Accuracy of the timed
    configuration is measured against a converged refinement (5 corrections, every residual
    evaluated) together with the FP64 path's error against the same reference."""
    import torch
    from cans_gb300 import cans
    plan = cans.Plan(n, dli, 1. / dzc, 1. / dzf, "PPPPNN", [0.] * 6, "ccc", precision=cans.FP32)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
    dzci, dzfi = T(1. / dzc), T(1. / dzf)
    rtol = args.rtol
    wz = torch.tensor(dzf[1:-1], device=dev, dtype=torch.float64)[:, None, None]
    dm = lambda f: f - (f * wz).sum() / (wz.sum() * n[0] * n[1])
    rel = lambda x, y: float(torch.linalg.vector_norm(dm(x - y)) / torch.linalg.vector_norm(dm(y)))
    # calibration: corrections needed to reach rtol (every residual evaluated)
    a = make_rhs(n, dzf, dev, seed=11)
    b = a.clone()
    k_cal, rr_cal = plan.solve_refined(b, dli, dzci, dzfi, rtol=rtol, max_iter=8)
    k_cal = max(1, k_cal)
    acc = {"calibrated_corrections": k_cal, "calibration_relres": rr_cal}
    if plan64 is not None:
        ref = a.clone()
        plan.solve_refined(ref, dli, dzci, dzfi, rtol=0.0, max_iter=5)
        x64 = a.clone()
        plan64.solve(x64)
        xk = a.clone()
        plan.solve_refined(xk, dli, dzci, dzfi, rtol=0.0, max_iter=k_cal)
        i3 = (slice(1, -1),) * 3
        acc.update({"reference": "refinement with 5 corrections, all residuals evaluated",
                    "error_vs_reference": rel(xk[i3], ref[i3]),
                    "fp64_path_error_vs_reference": rel(x64[i3], ref[i3]),
                    "error_vs_fp64_path_mean_removed": rel(xk[i3], x64[i3])})
        del ref, x64, xk
    del a, b
    src = make_rhs(n, dzf, dev)
    p = src.clone()
    for _ in range(args.warmup):
        p.copy_(src)
        plan.solve_refined(p, dli, dzci, dzfi, rtol=0.0, max_iter=k_cal)
    torch.cuda.synchronize()
    rank_barrier(world)
    st = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    l0 = cans.launch_count()
    # per-pass and per-residual-launch CUDA events on the plan's stream, over the timed solves
    plan.set_timing(True)
    for e0, e1 in ev:
        p.copy_(src)  # each step solves the same compatible RHS; the restore is outside the events
        e0.record(st)
        plan.solve_refined(p, dli, dzci, dzfi, rtol=0.0, max_iter=k_cal)
        e1.record(st)
    torch.cuda.synchronize()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev) / args.steps
    launches = cans.launch_count() - l0
    pass_ms, nrec = plan.get_timing()
    res_ms, nres = plan.get_residual_timing()
    plan.set_timing(False)
    rank_barrier(world)
    ms = max_over_ranks(ms, world, dev)
    e2e_out = None
    if e2e:
        # end to end through the C ABI with host buffers: every step copies its RHS from
        # pinned host memory, solves, and copies the solution back.  Four device buffers and
        # two copy streams pipeline the steps: the H2D of step k+1 and the D2H of step k-1
        # run on the copy engines while step k solves (the H2D target buffer's last D2H, of
        # step k+1-nbuf, has finished by then).  Host clock around all K steps, fill and
        # drain of the pipeline included.
        nbuf = 4
        k2 = max(nbuf, min(4 * args.steps, 24))
        host_in = [torch.empty(p.shape, dtype=torch.float64, pin_memory=True) for _ in range(nbuf)]
        host_out = [torch.empty(p.shape, dtype=torch.float64, pin_memory=True) for _ in range(nbuf)]
        for h in host_in:
            h.copy_(src.cpu())
        bufs = [p] + [torch.empty_like(p) for _ in range(nbuf - 1)]
        s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
        ev_in = [torch.cuda.Event() for _ in range(nbuf)]
        ev_solved = [torch.cuda.Event() for _ in range(nbuf)]
        ev_out = [torch.cuda.Event() for _ in range(nbuf)]
        torch.cuda.synchronize()
        rank_barrier(world)
        t0 = time.perf_counter()
        with torch.cuda.stream(s_in):
            bufs[0].copy_(host_in[0], non_blocking=True)
            ev_in[0].record(s_in)
        for kk in range(k2):
            b = kk % nbuf
            st.wait_event(ev_in[b])
            if kk + 1 < k2:
                nb = (kk + 1) % nbuf
                with torch.cuda.stream(s_in):
                    if kk + 1 >= nbuf:
                        s_in.wait_event(ev_out[nb])  # the buffer's previous solution is on the host
                    bufs[nb].copy_(host_in[nb], non_blocking=True)
                    ev_in[nb].record(s_in)
            plan.solve_refined(bufs[b], dli, dzci, dzfi, rtol=0.0, max_iter=k_cal)
            ev_solved[b].record(st)
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_solved[b])
                host_out[b].copy_(bufs[b], non_blocking=True)
                ev_out[b].record(s_out)
        torch.cuda.synchronize()
        ms_e2e = max_over_ranks((time.perf_counter() - t0) * 1e3 / k2, world, dev)
        nbytes = p.numel() * 8
        e2e_out = {"value": round(job_throughput(ms_e2e, world), 3), "unit": "solves/s", "h2d_bytes_per_step": nbytes,
                   "d2h_bytes_per_step": nbytes, "steps": k2,
                   "note": "pipelined: H2D(k+1) and D2H(k-1) overlap solve k (four buffers, two copy streams)"}
        del host_in, host_out, bufs
    names = ["solve_xfwd", "solve_yfwd", "solve_zthomas", "solve_ybwd", "solve_xbwd"]
    del p, plan
    torch.cuda.empty_cache()
    return {"value": round(job_throughput(ms, world), 3), "unit": "solves/s", "ms_per_step": round(ms, 4),
            "rtol": rtol, "corrections_per_solve": k_cal, "fp32_solves_per_solve": k_cal + 1,
            "residual_passes_per_solve": k_cal, "accuracy": acc, "gpu_launches": launches,
            "fp32_pass_ms": {k: round(v, 4) for k, v in zip(names, pass_ms)}, "residual_ms": round(res_ms, 4),
            "residual_launches_timed": nres, "residual_bytes_per_cell": residual_bytes(k_cal), "e2e": e2e_out}


def tgv_init(sim):
    """initflow 'tgv' (src/initflow.f90:102-117) with the analytic pressure of the TGV
    configuration, rounded to FP32 so that every leg starts from the same values"""
    import torch
    n = sim.n[0]
    dev = sim.u.device
    dl = 2 * np.pi / n
    x = (torch.arange(1, n + 1, device=dev, dtype=torch.float64) - 0.5) * dl
    xf = torch.arange(1, n + 1, device=dev, dtype=torch.float64) * dl
    put = lambda fld, val: fld[1:-1, 1:-1, 1:-1].copy_(val.float().double().to(fld.dtype))
    Z, Y, X = torch.meshgrid(x, x, xf, indexing="ij")
    put(sim.u, torch.sin(X) * torch.cos(Y) * torch.cos(Z))
    Z, Y, X = torch.meshgrid(x, xf, x, indexing="ij")
    put(sim.v, -torch.cos(X) * torch.sin(Y) * torch.cos(Z))
    Z, Y, X = torch.meshgrid(x, x, x, indexing="ij")
    put(sim.p, (torch.cos(2 * X) + torch.cos(2 * Y)) * (torch.cos(2 * Z) + 2.) / 16.)
    del X, Y, Z


def bench_rk3(size, dev, steps, legs=("fp64", "fp64_refined_pressure", "fp32_run")):
    """RK3 time steps of the 512^3 Taylor-Green vortex (Re 1600, explicit diffusion, fixed dt
    from CFL 0.5 at t = 0; 3 warm-up + `steps` timed steps): the FP64 path, the FP64 path with
    the pressure solved on an FP32 plan with two FP64 refinement corrections, and the FP32
    run (FP32 fields and stencils + the refined pressure); the latter two's velocity and
    pressure are compared with the FP64 path's after the same steps."""
    import torch
    from cans_gb300.driver import Simulation
    n = size
    ncell = n ** 3

    def case(dt_f, prec, refine):
        c = dict(ng=[n, n, n], l=[2 * np.pi] * 3, gtype=1, gr=0., cfl=0.5, dtmax=1e5, dt_f=dt_f, visci=1600.,
                 icheck=0, cbcvel="PP" * 9, cbcpre="PP" * 3, bcvel=[0.] * 18, bcpre=[0.] * 6, precision=prec)
        if refine:
            c["pressure_refine"] = {"rtol": 0.0, "max_iter": 2}
        return c

    sim = Simulation(case(-1., "fp64", False), device=dev)
    tgv_init(sim)
    sim.start()
    dt = sim.dt
    del sim
    torch.cuda.empty_cache()
    spec = {"fp64": ("fp64", False), "fp64_refined_pressure": ("fp64", True), "fp32_run": ("fp32", False)}
    out, ref = {"workload": f"tgv_{n}^3_rk3", "steps": steps, "warmup_steps": 3, "dt": dt}, None
    for leg in legs:
        prec, refine = spec[leg]
        sim = Simulation(case(dt, prec, refine), device=dev)
        tgv_init(sim)
        sim.start()
        ms, launches = run_and_time(sim, 3, steps)
        r = {"value": round(ncell / (ms * 1e-3) / 1e6, 2), "unit": "Mcell/s", "ms_per_step": round(ms, 3),
             "gpu_launches_per_step": launches}
        if refine or prec == "fp32":
            r["pressure_corrections"] = sim.p_refine["max_iter"]
        if ref is None and leg == "fp64":
            ref = {name: getattr(sim, name)[1:-1, 1:-1, 1:-1].clone() for name in ("u", "v", "w", "p")}
        elif ref is not None:
            r["rel_l2_vs_fp64_path"] = field_errors(sim, ref)
        out[leg] = r
        del sim
        torch.cuda.empty_cache()
    del ref
    torch.cuda.empty_cache()
    return out


def bx_cases(nbox, seed=7):
    """The batched closed-box workload: lid-driven cavities with nx, ny, nz drawn from
    {32, 48, ..., 128}, Re from U[100, 1000], lid u = 1 at the top, Dirichlet velocity and
    Neumann pressure walls, uniform unit cube grid, implicit diffusion, fixed dt (CFL 0.5 at
    the lid velocity)."""
    rng = np.random.default_rng(seed)
    sizes = np.arange(32, 129, 16)
    cases = []
    for _ in range(nbox):
        n = [int(x) for x in rng.choice(sizes, 3)]
        re = float(rng.uniform(100., 1000.))
        bcvel = [0.] * 18
        bcvel[5] = 1.0
        dlmin = min(1. / n[0], 1. / n[1], 1. / n[2])
        cases.append(dict(ng=n, l=[1., 1., 1.], gtype=1, gr=0., visci=re, dt_f=0.5 * dlmin, icheck=0,
                          cbcvel="DDDDDD" * 3, bcvel=bcvel, cbcpre="NNNNNN", bcpre=[0.] * 6, is_impdiff=1))
    return cases


def bench_boxes(nbox, dev, steps, autotune=True, unbatched_boxes=0):
    """Batched boxes: one persistent launch per stage over all boxes, a captured CUDA graph
    per time step; Mcell-steps/s over all boxes.  unbatched_boxes > 0 also times the
    single-box call sequence on that many boxes (a host-driven loop, for contrast)."""
    import torch
    from cans_gb300 import cans
    from cans_gb300.driver import Boxes, Simulation
    cases = bx_cases(nbox)
    cells = sum(c["ng"][0] * c["ng"][1] * c["ng"][2] for c in cases)
    t0 = time.perf_counter()
    bx = Boxes(cases, autotune=autotune, device=dev)
    setup_s = time.perf_counter() - t0
    bx.start()
    st = bx.stream
    out = {"workload": f"bx_{nbox}_lid_cavities_32-128_impdiff_fp64", "boxes": nbox, "cells": cells,
           "autotune": bool(autotune), "setup_s": round(setup_s, 2)}
    # graph: first call runs + captures, then replays
    bx.step(2, use_graph=True)
    bx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = cans.launch_count()
    e0.record(st)
    bx.step(steps, use_graph=True)
    e1.record(st)
    bx.synchronize()
    ms = e0.elapsed_time(e1) / steps
    out["graph"] = {"Mcell_steps_per_s": round(cells / (ms * 1e-3) / 1e6, 2), "ms_per_step": round(ms, 3),
                    "graph_launches_per_step": (cans.launch_count() - l0) // steps,
                    "kernel_nodes_per_step": bx.graph_nodes}
    # the same stages launched eagerly (no graph)
    e0.record(st)
    l0 = cans.launch_count()
    bx.step(steps, use_graph=False)
    e1.record(st)
    bx.synchronize()
    ms = e0.elapsed_time(e1) / steps
    out["eager"] = {"Mcell_steps_per_s": round(cells / (ms * 1e-3) / 1e6, 2), "ms_per_step": round(ms, 3),
                    "gpu_launches_per_step": (cans.launch_count() - l0) // steps}
    del bx
    torch.cuda.empty_cache()
    if unbatched_boxes:
        sims = []
        for c in cases[:unbatched_boxes]:
            s = Simulation(c, device=dev)
            s.start()
            sims.append(s)
        for s in sims:
            s.step(1)
        torch.cuda.synchronize()
        ub_cells = sum(c["ng"][0] * c["ng"][1] * c["ng"][2] for c in cases[:unbatched_boxes])
        t0 = time.perf_counter()
        for s in sims:
            s.step(1)
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        out["unbatched"] = {"boxes": unbatched_boxes, "Mcell_steps_per_s": round(ub_cells / sec / 1e6, 2),
                            "ms_per_step": round(sec * 1e3, 3),
                            "note": "single-box call sequence per box from Python (host clock)"}
        del sims
        torch.cuda.empty_cache()
    return out


def bench_adjoint(dev, n=(256, 128, 128), nsteps=50, ckpt=10, ndir=8, seed=11):
    """Square-duct differentiation workload: J = volume-integrated kinetic energy after
    `nsteps` RK3 steps (explicit diffusion, fixed dt), dJ/d(initial velocity) and
    dJ/d(uniform body force) by the hand-written adjoint with checkpoints every `ckpt`
    steps, checked against central differences of the same model along `ndir` seeded
    random directions (and the three body-force components)."""
    import torch
    from cans_gb300.adjoint import AdjointRun
    l = (6.0, 2.0, 2.0)
    dlmin = min(l[0] / n[0], l[1] / n[1], l[2] / n[2])
    case = dict(ng=list(n), l=list(l), gtype=1, gr=0.0, cfl=0.5, dt_f=0.5 * dlmin / 2.35, visci=4410.0, icheck=0,
                cbcvel="PPDDDD" * 3, bcvel=[0.0] * 18, cbcpre="PPNNNN", bcpre=[0.0] * 6, is_impdiff=0,
                is_forced=[0, 0, 0])
    y = (np.arange(n[1]) + 0.5) / n[1] * 2 - 1
    z = (np.arange(n[2]) + 0.5) / n[2] * 2 - 1
    rng = np.random.default_rng(seed)
    prof = 2.25 * np.outer(1 - z ** 2, 1 - y ** 2)[:, :, None] * np.ones(n[0])[None, None, :]
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
    u0 = T(prof + 0.1 * rng.uniform(-1, 1, prof.shape))
    v0 = T(0.1 * rng.uniform(-1, 1, prof.shape))
    w0 = T(0.1 * rng.uniform(-1, 1, prof.shape))
    bf = [0.01, 0.0, 0.0]
    run = AdjointRun(case, device=dev, ckpt_every=ckpt)
    run.forward(u0, v0, w0, bf, 2)  # warm-up (first launches, factorisations)
    run.backward()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J = run.forward(u0, v0, w0, bf, nsteps)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    du, dv, dw, dbf = run.backward()
    torch.cuda.synchronize()
    t_bwd = time.perf_counter() - t0
    errs = []
    eps = 1e-5
    for _ in range(ndir):
        d = [T(rng.standard_normal(prof.shape)) for _ in range(3)]
        ad = float(sum((g * di).sum() for g, di in zip((du, dv, dw), d)))
        jp = run.forward(*[a + eps * di for a, di in zip((u0, v0, w0), d)], bf, nsteps)
        jm = run.forward(*[a - eps * di for a, di in zip((u0, v0, w0), d)], bf, nsteps)
        fd = (jp - jm) / (2 * eps)
        errs.append(abs(fd - ad) / max(abs(fd), 1e-300))
    bchk = {}
    for c in range(3):
        b = list(bf)
        b[c] += eps
        jp = run.forward(u0, v0, w0, b, nsteps)
        b[c] -= 2 * eps
        jm = run.forward(u0, v0, w0, b, nsteps)
        fd = (jp - jm) / (2 * eps)
        # y, z: a uniform force across walls is a gradient the projection absorbs (dJ = 0)
        bchk["xyz"[c]] = {"fd": float(fd), "adjoint": float(dbf[c]),
                          "rel_err": float(abs(fd - dbf[c]) / max(abs(fd), 1e-300)) if c == 0 else None}
    return {"workload": f"duct_{n[0]}x{n[1]}x{n[2]}_ke_after_{nsteps}_rk3_steps_fp64", "J": J,
            "forward_ms_per_step": round(t_fwd / nsteps * 1e3, 3),
            "adjoint_ms_per_step": round(t_bwd / nsteps * 1e3, 3),
            "adjoint_over_forward": round(t_bwd / t_fwd, 2), "checkpoint_every": ckpt,
            "fd_directions": ndir, "fd_eps": eps, "max_rel_err_velocity": float(max(errs)),
            "bforce_check": bchk, "clock": "host, synchronised"}


def gpu_solutions(n, dli, dzc, dzf, dev, k):
    """The headline RHS solved by the FP64 path and by FP32 + k refinement corrections (the
    timed schedule), copied to the host ((n3, n2, n1) interiors) for the comparison with the
    oracle in the CPU leg"""
    import torch
    from cans_gb300 import cans
    out = {}
    plan = cans.Plan(n, dli, 1. / dzc, 1. / dzf, "PPPPNN", [0.] * 6, "ccc")
    p = make_rhs(n, dzf, dev)
    plan.solve(p)
    out["fp64_path"] = p[1:-1, 1:-1, 1:-1].cpu().numpy()
    del plan, p
    torch.cuda.empty_cache()
    plan = cans.Plan(n, dli, 1. / dzc, 1. / dzf, "PPPPNN", [0.] * 6, "ccc", precision=cans.FP32)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)
    p = make_rhs(n, dzf, dev)
    plan.solve_refined(p, dli, T(1. / dzc), T(1. / dzf), rtol=0.0, max_iter=k)
    out["fp32_refined"] = p[1:-1, 1:-1, 1:-1].cpu().numpy()
    del plan, p
    torch.cuda.empty_cache()
    return out


def bench_cpu(size, steps, warmup, threads=None, gpu=None):
    """The oracle (CPU restatement of src/solver.f90 with FFTW r2r semantics) on all host
    cores, solving the GPU arm's right-hand side (host_rhs): mean seconds per solve over
    `steps` solves after `warmup`.  With `gpu` (gpu_solutions) it also returns the accuracy
    block: each GPU solution against the oracle's, and every solution against an accuracy
    reference -- the oracle's solve plus one refinement step with an extended-precision
    residual (orc_poisson_residual_ld) -- relative L2 of the mean-free parts."""
    from oracle import oracle as O
    if threads:
        O.set_num_threads(threads)
    n = [size] * 3
    dl = [L_CH[d] / n[d] for d in range(3)]
    dli = [1. / x for x in dl]
    dzc, dzf, zc, zf = O.initgrid(1, n[2], 1.4, L_CH[2], False)
    s = O.initsolver(n, dli, 1. / dzc, 1. / dzf, "PPPPNN", [0.] * 6, "ccc")
    rhs = O.field(n)
    rhs[1:-1, 1:-1, 1:-1] = host_rhs(n, dzf).transpose(2, 1, 0)
    solve = lambda q: O.solver(n, s["normfft"], s["lambdaxy"], s["a"], s["b"], s["c"], "PPPPNN", "ccc", q)
    times = []
    p = None
    for it in range(warmup + steps):
        p = rhs.copy(order="F")
        t0 = time.perf_counter()
        solve(p)
        if it >= warmup:
            times.append(time.perf_counter() - t0)
    sec = float(np.mean(times))
    acc = None
    if gpu is not None:
        i3 = (slice(1, -1),) * 3
        xo = p[i3].transpose(2, 1, 0)  # (n3, n2, n1) view
        e = O.field(n)
        e[i3] = O.poisson_residual_ld(n, dli, "PPPPNN", s["a"], s["b"], s["c"], p, rhs)
        solve(e)
        xt = xo + e[i3].transpose(2, 1, 0)
        del e
        w = dzf[1:-1][:, None, None]
        wsum = w.sum() * n[0] * n[1]
        dm = lambda f: f - (f * w).sum() / wsum
        xt_m, xo_m = dm(xt), dm(xo)
        nt, no = np.linalg.norm(xt_m), np.linalg.norm(xo_m)
        acc = {"reference": "oracle FP64 solve + one refinement step with an extended-precision residual",
               "metric": "relative L2 of the volume-weighted mean-free parts",
               "oracle_fp64_vs_reference": float(np.linalg.norm(xo_m - xt_m) / nt)}
        for name, x in gpu.items():
            xm = dm(x)
            acc[f"{name}_vs_oracle"] = float(np.linalg.norm(xm - xo_m) / no)
            acc[f"{name}_vs_reference"] = float(np.linalg.norm(xm - xt_m) / nt)
    return sec, O.num_threads(), acc


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=N_DEFAULT)
    ap.add_argument("--skip-rk3", action="store_true")
    ap.add_argument("--skip-mx", action="store_true", help="skip the 1024x512x384 Poisson leg")
    ap.add_argument("--skip-ch", action="store_true", help="skip the 512x256x256 channel run")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-refine", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--rtol", type=float, default=1e-13)
    ap.add_argument("--boxes", type=int, default=256, help="batched closed-box leg (0: skip)")
    ap.add_argument("--skip-adjoint", action="store_true")
    ap.add_argument("--adjoint-steps", type=int, default=50)
    ap.add_argument("--adjoint-dirs", type=int, default=8)
    ap.add_argument("--only", choices=["refined", "rk3", "rk3-fp32", "fp32-solve", "adjoint", "boxes", "mx",
                                       "mx-run", "ch"], default=None,
                    help="profiling aid: run one secondary leg and print its JSON")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        sec, cores, _ = bench_cpu(args.size, args.steps, min(args.warmup, 1))
        val = 1.0 / sec
        out = {"metric": METRIC, "impl": "reference", "value": round(val, 5), "unit": "solves/s", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 2),
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic (seeded N(0,1) RHS, volume-weighted mean removed; the GPU arm's values)",
               "config": {"workload": f"poisson_{args.size}x{args.size}x{args.size}_PPPPNN",
                          "grid": [args.size] * 3, "bc_pressure": "PP,PP,NN", "z_grid": "tanh gr=1.4",
                          "domain": [round(x, 6) for x in L_CH],
                          "precision": "FP64 solve (the reference's CPU solver, src/solver.f90)"},
               "cpu_baseline": {"value": round(val, 5), "unit": "solves/s", "cores": cores, "kind": "port",
                                "sample": f"{args.steps} full {args.size}^3 solves of the C/OpenMP restatement "
                                          "of src/solver.f90 (reference Fortran/MPI/FFTW build unavailable)"},
               "e2e": {"value": round(val, 5), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    out = bench_ours(args, rank, world)
    if rank == 0:
        if not args.skip_cpu:
            sols = out.pop("_gpu_solutions", None)
            sec, cores, acc = bench_cpu(args.size, 3, 1, gpu=sols)
            out["cpu_baseline"] = {"value": round(1.0 / sec, 5), "unit": "solves/s", "cores": cores, "kind": "port",
                                   "sample": f"3 full {args.size}^3 FP64 solves (after 1 warm-up) of the C/OpenMP "
                                             "restatement of src/solver.f90 on the host cores, same RHS"}
            if acc is not None:
                out["accuracy_vs_oracle"] = acc
        out.pop("_gpu_solutions", None)
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
