"""Single-GPU time loop over the C ABI, mirroring src/main.f90:144-520.

`Simulation(case)` performs the set-up of src/main.f90:158-418 (grid, solver
plans, initial condition, boundary conditions, first dt) and `step()` one time
step of src/main.f90:437-510 (three RK3 substeps of rk / bounduvw / fillps /
updt_rhs_b / solver / boundp / correc / bounduvw / updatep / boundp, then the
dt and divergence checks every `icheck` steps).  All arithmetic runs in the
library's CUDA kernels; this module only orders the calls, exactly as the
Fortran host would.

`case` keys follow input.nml (&dns, &numerics): ng, l, gtype, gr, cfl, dtmax,
dt_f, visci, icheck, cbcvel (18 chars, cbcvel(0:1,3,3) order), bcvel (18),
cbcpre (6 chars), bcpre (6), bforce, is_forced, velf, is_impdiff, inivel; and the
&scalar keys (src/param.f90:144-151): nscal, alphai, cbcscal (6 chars each), bcscal
(6 each), ssource, is_sforced, scalf, gacc, beta, is_boussinesq_buoyancy.  Scalars are
advanced before the velocity in every substep (src/main.f90:440-451).  With
pressure_refine = {"rtol": r, "max_iter": K} the pressure solve runs on an FP32 plan with
FP64 iterative refinement (cans_solver_refined) instead of the FP64 path.
"""
import ctypes as C

import numpy as np

from . import cans
from . import output

RKCOEFF = ((32. / 60., 0. / 60.), (25. / 60., -17. / 60.), (45. / 60., -25. / 60.))  # src/param.f90:20-22
DBL_MAX = np.finfo(np.float64).max
# src/param.f90:18, small = epsilon(1._rp)*10**(precision(1._rp)/2) with rp = dp: precision is
# 15 decimal digits and 15/2 is integer division, so small = 2.22e-16 * 1e7
SMALL = np.finfo(np.float64).eps * 10 ** (15 // 2)
# the same with rp = sp (precision 6 digits): the threshold of the FP32 run
SMALL_SP = float(np.finfo(np.float32).eps) * 10 ** (6 // 2)


class SimulationAborted(RuntimeError):
    """The run stopped on a failed stability check (src/main.f90:489-510): the time step is
    too small, or the divergence is too large or NaN.  `Simulation.kill` is then True and,
    as in the reference, no further step runs and nothing is saved."""


def initgrid(gtype, n, gr, lz, is_periodic):
    """src/initgrid.f90:14-99 through the library's cans_initgrid."""
    arrs = [np.zeros(n + 2) for _ in range(4)]
    rc = cans.lib().cans_initgrid(int(gtype), int(n), float(gr), float(lz), int(is_periodic),
                                  *[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs])
    if rc != 0:
        raise cans.CansError(rc, "cans_initgrid")
    return arrs  # dzc, dzf, zc, zf


class Simulation:
    def __init__(self, case, device="cuda"):
        import torch
        self.case = case
        self.device = device
        n = [int(x) for x in case["ng"]]
        self.n = n
        self.l = [float(x) for x in case["l"]]
        self.dl = [self.l[d] / n[d] for d in range(3)]
        self.dli = [1. / x for x in self.dl]
        self.visc = 1. / case["visci"]
        self.cbcvel, self.cbcpre = case["cbcvel"], case["cbcpre"]
        self.bcvel = list(case.get("bcvel", [0.] * 18))
        self.bcpre = list(case.get("bcpre", [0.] * 6))
        self.bforce = list(case.get("bforce", [0.] * 3))
        self.is_forced = [int(x) for x in case.get("is_forced", [0] * 3)]
        self.velf = list(case.get("velf", [0.] * 3))
        self.is_impdiff = int(case.get("is_impdiff", 0))
        self.icheck = int(case.get("icheck", 10))
        self.is_mask_divergence_check = bool(case.get("is_mask_divergence_check", False))
        self.kill = False
        self.cfl, self.dtmax, self.dt_f = case.get("cfl", 0.95), case.get("dtmax", 1e5), case.get("dt_f", -1.)
        zper = self.cbcpre[4:6] == "PP"
        dzc, dzf, zc, zf = initgrid(case.get("gtype", 1), n[2], case.get("gr", 0.), self.l[2], zper)
        self.dzc, self.dzf, self.zc, self.zf = dzc, dzf, zc, zf
        self.dzci_h, self.dzfi_h = 1. / dzc, 1. / dzf
        vol = self.l[0] * self.l[1] * self.l[2]
        gvr_c = self.dl[0] * self.dl[1] * dzc / vol
        gvr_f = self.dl[0] * self.dl[1] * dzf / vol
        t = lambda a: torch.tensor(a, dtype=torch.float64, device=device)
        self.dzci, self.dzfi, self.gvr_c, self.gvr_f = t(self.dzci_h), t(self.dzfi_h), t(gvr_c), t(gvr_f)
        # is_bound on one GPU with x-aligned pencils (src/initmpi.f90:193-267)
        self.is_bound = [1, 1] + [0 if self.cbcpre[2 * d:2 * d + 2] == "PP" else 1 for d in (1, 2) for _ in (0, 1)]
        # pressure_refine = {"rtol": r, "max_iter": K}: the pressure solve runs on an FP32 plan
        # with FP64 iterative refinement (cans_solver_refined) instead of the FP64 path
        self.p_refine = dict(case["pressure_refine"]) if case.get("pressure_refine") else None
        # precision = "fp32": the FP32 run -- FP32 fields and stencils (the reference's
        # single-precision build, src/types.f90:12-18) with the pressure correction solved to
        # FP64 accuracy by refinement (two corrections unless pressure_refine says otherwise)
        self.fp32 = case.get("precision", "fp64") == "fp32"
        if self.fp32:
            if self.is_impdiff or int(case.get("nscal", 0)) > 0:
                raise ValueError("precision 'fp32' runs explicit diffusion without scalars")
            if self.p_refine is None:
                self.p_refine = {"rtol": 0.0, "max_iter": 2}
        self.small = SMALL_SP if self.fp32 else SMALL
        self.p_refine_iters = 0
        self.plan_p = cans.Plan(n, self.dli, self.dzci_h, self.dzfi_h, self.cbcpre, self.bcpre, "ccc",
                                precision=cans.FP32 if self.p_refine else cans.FP64)
        self.plans_v = []
        if self.is_impdiff:
            for c in range(3):
                cf = ["c", "c", "c"]
                cf[c] = "f"
                self.plans_v.append(cans.Plan(n, self.dli, self.dzci_h, self.dzfi_h, self.cbcvel[6 * c:6 * c + 6],
                                              self.bcvel[6 * c:6 * c + 6], "".join(cf)))
        fdt = torch.float32 if self.fp32 else torch.float64
        self.u, self.v, self.w, self.p = [cans.field(n, device, fdt) for _ in range(4)]
        self.pp = cans.field(n, device)
        self.dudtrko, self.dvdtrko, self.dwdtrko = [torch.zeros((n[2], n[1], n[0]), dtype=fdt,
                                                                device=device) for _ in range(3)]
        if self.fp32:
            # second velocity buffer: rk writes the new velocity there and the two are swapped
            self.unew, self.vnew, self.wnew = [cans.field(n, device, fdt) for _ in range(3)]
            t32 = lambda a: torch.tensor(a, dtype=torch.float32, device=device)
            self.dzci32, self.dzfi32 = t32(self.dzci_h), t32(self.dzfi_h)
            self.gvr_c32, self.gvr_f32 = t32(gvr_c), t32(gvr_f)
            self.rk_work = cans.rk_f32_work(n, False, device)
        self.time, self.istep, self.dt, self.dti = 0., 0, 0., 0.
        self.divtot = self.divmax = 0.
        self.dpdl = np.zeros(3)
        self._init_scalars(case, device)

    def _init_scalars(self, case, device):
        """src/scal.f90:321-360 (initialize_scalars) and src/param.f90:277-317."""
        import torch
        n = self.n
        nscal = max(0, int(case.get("nscal", 0)))
        self.gacc = [float(x) for x in case.get("gacc", [0.] * 3)]
        self.beta = float(case.get("beta", 0.))
        self.is_buoyancy = bool(case.get("is_boussinesq_buoyancy", False))
        if self.is_buoyancy and nscal == 0:
            raise ValueError("is_boussinesq_buoyancy requires nscal > 0")
        self.scalars = []
        for i in range(nscal):
            cbc = case["cbcscal"][i]
            bc = list(case.get("bcscal", [[0.] * 6] * nscal)[i])
            sc = {"alpha": 1. / float(case["alphai"][i]), "cbc": cbc, "bc": bc,
                  "source": float(case.get("ssource", [0.] * nscal)[i]),
                  "is_forced": int(case.get("is_sforced", [0] * nscal)[i]),
                  "scalf": float(case.get("scalf", [0.] * nscal)[i]),
                  "val": cans.field(n, device),
                  "dsdtrko": torch.zeros((n[2], n[1], n[0]), dtype=torch.float64, device=device),
                  "work": cans.rk_scal_work(n, self.is_impdiff, device), "f": 0.}
            if self.is_impdiff:
                sc["plan"] = cans.Plan(n, self.dli, self.dzci_h, self.dzfi_h, cbc, bc, "ccc")
            self.scalars.append(sc)
        self.fs = np.zeros(nscal)
        # alpha_max: the largest diffusivity, for the time-step restriction
        self.alpha_max = max([sc["alpha"] for sc in self.scalars], default=1. / DBL_MAX)

    # ------------------------------------------------------------------ initial conditions
    def set_fields(self, u=None, v=None, w=None, p=None, scalars=()):
        """Fortran-indexed host arrays (n1+2, n2+2, n3+2) -> device fields."""
        for name, a in (("u", u), ("v", v), ("w", w), ("p", p)):
            if a is not None:
                fld = getattr(self, name)
                fld.copy_(cans.to_device(a, self.device, fld.dtype))
        for sc, a in zip(self.scalars, scalars):
            if a is not None:
                sc["val"].copy_(cans.to_device(a, self.device))

    def _io_vars(self):
        """(file stem, field) of every checkpointed variable, src/main.f90:360-368."""
        out = [(name, getattr(self, name)) for name in ("u", "v", "w", "p")]
        return out + [(f"s_{i + 1:03d}", sc["val"]) for i, sc in enumerate(self.scalars)]

    def start(self, restart_dir=None):
        """src/main.f90:372-418: the initial fields (or, with restart_dir, the checkpoint
        fld_u/v/w/p.bin there), their BCs and the first dt."""
        n = self.n
        restart = restart_dir is not None
        self.istep, self.time = 0, 0.
        if restart:
            import os
            for name, fld in self._io_vars():
                tmp = fld if fld.dtype == self.pp.dtype else cans.field(n, self.device)
                self.time, self.istep = cans.load_field(os.path.join(restart_dir, f"fld_{name}.bin"), n, tmp)
                if tmp is not fld:
                    fld.copy_(tmp)
        elif self.case.get("inivel"):
            self._initflow()
        bounduvw = cans.bounduvw_f32 if self.fp32 else cans.bounduvw
        boundp = cans.boundp_f32 if self.fp32 else cans.boundp
        bounduvw(self.cbcvel, n, self.bcvel, self.is_bound, self.dl, self.dzc, self.dzf, self.u, self.v, self.w,
                 restart)
        boundp(self.cbcpre, n, self.bcpre, self.is_bound, self.dl, self.dzc, self.p, cans.HALO_UPPER)
        for sc in self.scalars:
            cans.boundp(sc["cbc"], n, sc["bc"], self.is_bound, self.dl, self.dzc, sc["val"])
        self._new_dt()

    def _initflow(self):
        """initflow (src/initflow.f90:16-259, src/main.f90:375) from the case's inivel and
        is_wallturb keys, on the device (FP64, rounded into the fields of the FP32 run)."""
        n = self.n
        flds = [cans.field(n, self.device) for _ in range(4)] if self.fp32 else [self.u, self.v, self.w, self.p]
        cans.initflow(self.case["inivel"], self.bcvel, n, self.l, self.dl, self.zc, self.zf, self.dzc, self.dzf,
                      self.visc, self.is_forced, self.velf, self.bforce, bool(self.case.get("is_wallturb", False)),
                      *flds)
        if self.fp32:
            for dst, src in zip((self.u, self.v, self.w, self.p), flds):
                dst[1:-1, 1:-1, 1:-1] = src[1:-1, 1:-1, 1:-1]

    def save(self, datadir):
        """Checkpoint (src/main.f90:578-616 with is_overwrite_save): fld_u/v/w/p.bin and
        fld_s_001.bin ... for the scalars."""
        import os
        for name, fld in self._io_vars():
            # the FP32 run writes the reference's FP64 file layout (values widened exactly)
            cans.save_field(os.path.join(datadir, f"fld_{name}.bin"), self.n, fld.double(), self.time, self.istep)

    # ------------------------------------------------------------------ text output
    def out0d(self, datadir):
        """The 0d logs of src/main.f90:515-552: time.out, forcing.out and forcing_s_NNN.out."""
        import os
        output.out0d(os.path.join(datadir, "time.out"), [1. * self.istep, self.dt, self.time])
        if any(self.is_forced) or any(abs(b) > 0. for b in self.bforce):
            mean = [0., 0., 0.]
            for d, (fld, gvr) in enumerate(((self.u, self.gvr_f), (self.v, self.gvr_f), (self.w, self.gvr_c))):
                if self.is_forced[d] or abs(self.bforce[d]) > 0.:
                    mean[d] = cans.bulk_mean(self.n, gvr, fld.double())
            dpdl = list(self.dpdl) if any(self.is_forced) else [-b for b in self.bforce]
            output.out0d(os.path.join(datadir, "forcing.out"), [self.time] + dpdl + mean)
        for i, sc in enumerate(self.scalars):
            if sc["is_forced"] or abs(sc["source"]) > 0.:
                ms = cans.bulk_mean(self.n, self.gvr_f, sc["val"])
                fs = self.fs[i] if sc["is_forced"] else sc["source"]
                output.out0d(os.path.join(datadir, f"forcing_s_{i + 1:03d}.out"), [self.time, fs, ms])

    def out1d(self, datadir, velstats=False):
        """The profiles of src/out1d.h90: umean_z, vmean_z, wmean_z (and scal_01_mean with a
        scalar) for step istep; velstats=True adds out1d_chan's velstats file."""
        import os
        import torch
        n, fld = self.n, f"{self.istep:07d}"
        dzf, dzc = (torch.tensor(a, dtype=torch.float64, device=self.u.device) for a in (self.dzf, self.dzc))
        path = lambda name: os.path.join(datadir, f"{name}_fld_{fld}.out")
        items = [("umean_z", self.zc, dzf, self.u), ("vmean_z", self.zc, dzf, self.v),
                 ("wmean_z", self.zf, dzc, self.w)]
        if self.scalars:
            items.append(("scal_01_mean", self.zc, dzc, self.scalars[0]["val"]))
        for name, z_g, dz, f in items:
            p1d = cans.out1d(n, self.l, self.dl, 3, dz, f.double()).cpu().numpy()
            output.write_out1d(path(name), 3, n, self.dl, z_g, p1d)
        if velstats:
            st = cans.out1d_chan(n, self.l, self.dl, self.u.double(), self.v.double(), self.w.double()).cpu().numpy()
            output.write_out1d_chan(path("velstats"), n, self.zc, st)
        torch.cuda.synchronize()

    def _new_dt(self):
        if self.fp32:
            dt_cfl = cans.chkdt_f32(self.n, self.dl, self.dzci32, self.dzfi32, self.visc, self.alpha_max, 0, 0,
                                    self.u, self.v, self.w)
        else:
            dt_cfl = cans.chkdt(self.n, self.dl, self.dzci, self.dzfi, self.visc, self.alpha_max, self.is_impdiff,
                                0, self.u, self.v, self.w)
        self.dt = self.dt_f if self.dt_f > 0. else min(self.cfl * dt_cfl, self.dtmax)
        self.dti = 1. / self.dt
        return dt_cfl

    def _substep_fp32(self, irk):
        """One RK3 substep of the FP32 run, in the order of substep(): rk writes the new
        velocity into the second buffer and the two buffers are swapped (the reference updates
        u, v, w in place; every later call reads the new velocity, so the results agree)."""
        n = self.n
        dtrk = (RKCOEFF[irk][0] + RKCOEFF[irk][1]) * self.dt
        dtrki = 1. / dtrk
        f = cans.rk_f32(RKCOEFF[irk], n, self.dli, self.dzci32, self.dzfi32, self.gvr_c32, self.gvr_f32, self.dt,
                        self.visc, self.p, self.is_forced, self.velf, self.bforce, self.dudtrko, self.dvdtrko,
                        self.dwdtrko, self.u, self.v, self.w, self.unew, self.vnew, self.wnew, self.rk_work)
        self.u, self.unew = self.unew, self.u
        self.v, self.vnew = self.vnew, self.v
        self.w, self.wnew = self.wnew, self.w
        self.dpdl += f
        cans.bounduvw_f32(self.cbcvel, n, self.bcvel, self.is_bound, self.dl, self.dzc, self.dzf, self.u, self.v,
                          self.w, False, cans.HALO_LOWER)
        cans.fillps_f32(n, self.dli, self.dzfi32, dtrki, self.u, self.v, self.w, self.pp)
        cans.updt_rhs_b("ccc", self.cbcpre, n, self.is_bound, self.plan_p.rhsb, self.pp)
        it, _ = self.plan_p.solve_refined(self.pp, self.dli, self.dzci, self.dzfi,
                                          rtol=self.p_refine.get("rtol", 0.), max_iter=self.p_refine["max_iter"])
        self.p_refine_iters = max(self.p_refine_iters, it)
        cans.boundp(self.cbcpre, n, self.bcpre, self.is_bound, self.dl, self.dzc, self.pp)
        # correc and updatep in one pass over pp (they write disjoint fields), then the two
        # boundary calls of src/main.f90:470,472
        cans.correc_updatep_f32(n, self.dli, self.dzci32, dtrk, self.pp, self.u, self.v, self.w, self.p)
        cans.bounduvw_f32(self.cbcvel, n, self.bcvel, self.is_bound, self.dl, self.dzc, self.dzf, self.u, self.v,
                          self.w, True, cans.HALO_UPPER, cans.HALO_NONE)
        cans.boundp_f32(self.cbcpre, n, self.bcpre, self.is_bound, self.dl, self.dzc, self.p, cans.HALO_UPPER)

    def substep(self, irk):
        if self.fp32:
            return self._substep_fp32(irk)
        n = self.n
        dtrk = (RKCOEFF[irk][0] + RKCOEFF[irk][1]) * self.dt
        dtrki = 1. / dtrk
        for i, sc in enumerate(self.scalars):
            sc["f"] = cans.rk_scal(RKCOEFF[irk], n, self.dli, self.dzci, self.dzfi, self.gvr_f, sc["alpha"], self.dt,
                                   self.u, self.v, self.w, sc["is_forced"], sc["scalf"], sc["source"],
                                   self.is_impdiff, sc["dsdtrko"], sc["val"], sc["work"])
            cans.bulk_forcing_s(n, sc["is_forced"], sc["f"], sc["val"])
            self.fs[i] += sc["f"]
            if self.is_impdiff:
                sc["plan"].solve_helmholtz(-.5 * sc["alpha"] * dtrk, self.is_bound, sc["val"])
            cans.boundp(sc["cbc"], n, sc["bc"], self.is_bound, self.dl, self.dzc, sc["val"])
        rk_args = (RKCOEFF[irk], n, self.dli, self.dzci, self.dzfi, self.gvr_c, self.gvr_f, self.dt, self.visc,
                   self.p, self.is_forced, self.velf, self.bforce, self.is_impdiff)
        fields = (self.dudtrko, self.dvdtrko, self.dwdtrko, self.u, self.v, self.w)
        if self.is_buoyancy:
            f = cans.rk_buoy(*rk_args, self.gacc, self.beta, self.scalars[0]["val"], *fields)
        else:
            f = cans.rk(*rk_args, *fields)
        self.dpdl += f
        alpha = 0.
        if self.is_impdiff:
            alpha = -.5 * self.visc * dtrk
            for c, fld in enumerate((self.u, self.v, self.w)):
                self.plans_v[c].solve_helmholtz(alpha, self.is_bound, fld)
        cans.bounduvw(self.cbcvel, n, self.bcvel, self.is_bound, self.dl, self.dzc, self.dzf, self.u, self.v,
                      self.w, False, cans.HALO_LOWER)
        cans.fillps(n, self.dli, self.dzfi, dtrki, self.u, self.v, self.w, self.pp)
        cans.updt_rhs_b("ccc", self.cbcpre, n, self.is_bound, self.plan_p.rhsb, self.pp)
        if self.p_refine:
            it, _ = self.plan_p.solve_refined(self.pp, self.dli, self.dzci, self.dzfi,
                                              rtol=self.p_refine.get("rtol", 0.), max_iter=self.p_refine["max_iter"])
            self.p_refine_iters = max(self.p_refine_iters, it)
        else:
            self.plan_p.solve(self.pp)
        cans.boundp(self.cbcpre, n, self.bcpre, self.is_bound, self.dl, self.dzc, self.pp)
        cans.correc(n, self.dli, self.dzci, dtrk, self.pp, self.u, self.v, self.w)
        cans.bounduvw(self.cbcvel, n, self.bcvel, self.is_bound, self.dl, self.dzc, self.dzf, self.u, self.v,
                      self.w, True, cans.HALO_UPPER, cans.HALO_NONE)
        cans.updatep(n, self.dli, self.dzci, self.dzfi, alpha, self.is_impdiff, self.pp, self.p)
        cans.boundp(self.cbcpre, n, self.bcpre, self.is_bound, self.dl, self.dzc, self.p, cans.HALO_UPPER)

    def _abort(self, why):
        self.kill = True
        raise SimulationAborted(f"step {self.istep}: {why}; aborting (src/main.f90:489-510)")

    def check(self):
        """The stability checks of src/main.f90:489-510: new dt from chkdt (abort when dt_cfl <
        small), then chkdiv (abort when divmax > small or divtot is NaN, unless
        is_mask_divergence_check)."""
        dt_cfl = self._new_dt()
        if dt_cfl < self.small:
            self._abort(f"time step is too small (dt_cfl = {dt_cfl:.3e})")
        if self.fp32:
            self.divtot, self.divmax = cans.chkdiv_f32(self.n, self.l, self.dli, self.dzfi32, self.u, self.v, self.w,
                                                       allow_nonfinite=True)
        else:
            self.divtot, self.divmax = cans.chkdiv(self.n, self.l, self.dli, self.dzfi, self.u, self.v, self.w,
                                                   allow_nonfinite=True)
        if not self.is_mask_divergence_check and (self.divmax > self.small or np.isnan(self.divtot)):
            self._abort(f"maximum divergence is too large (divtot = {self.divtot:.3e}, "
                        f"divmax = {self.divmax:.3e})")
        # the library's own record of the pressure solves (no counterpart in the reference)
        if not self.plan_p.check():
            self._abort("the pressure solve met a non-finite right-hand side")

    def step(self, nsteps=1):
        if self.kill:
            raise SimulationAborted("the run was stopped by a failed stability check")
        for _ in range(nsteps):
            self.istep += 1
            self.time += self.dt
            self.dpdl[:] = 0.
            self.fs[:] = 0.
            for irk in range(3):
                self.substep(irk)
            self.dpdl = -self.dpdl * self.dti
            self.fs = self.fs * self.dti
            if self.icheck > 0 and self.istep % self.icheck == 0:
                self.check()


class Boxes:
    """Many independent boxes advanced together (cans_boxes_*): the batched form of
    `Simulation` for closed boxes with a fixed time step and implicit diffusion.

    `cases`: list of dicts with the `Simulation` keys ng, l, gtype, gr, visci, dt_f, cbcvel,
    bcvel, cbcpre, bcpre (and bforce).  Every box runs the call sequence of
    `Simulation.substep` and evolves bit-identically to it; one stage of a substep is one
    persistent launch over all boxes, and `step(use_graph=True)` replays one CUDA graph per
    time step.  The boxes run on their own CUDA stream (`self.stream`)."""

    def __init__(self, cases, is_impdiff=1, autotune=False, device="cuda"):
        import torch
        self.device = device
        self.stream = torch.cuda.Stream(device=device)
        self.boxes = []
        self._keep = []
        structs = (cans.CBox * len(cases))()
        for b, case in enumerate(cases):
            n = [int(x) for x in case["ng"]]
            l = [float(x) for x in case["l"]]
            zper = case["cbcpre"][4:6] == "PP"
            dzc, dzf, zc, zf = initgrid(case.get("gtype", 1), n[2], case.get("gr", 0.), l[2], zper)
            t = lambda a: torch.tensor(a, dtype=torch.float64, device=device)
            box = dict(n=n, l=l, dzc=dzc, dzf=dzf, dzci=t(1. / dzc), dzfi=t(1. / dzf),
                       u=cans.field(n, device), v=cans.field(n, device), w=cans.field(n, device),
                       p=cans.field(n, device), pp=cans.field(n, device),
                       dudtrko=torch.zeros((n[2], n[1], n[0]), dtype=torch.float64, device=device),
                       dvdtrko=torch.zeros((n[2], n[1], n[0]), dtype=torch.float64, device=device),
                       dwdtrko=torch.zeros((n[2], n[1], n[0]), dtype=torch.float64, device=device))
            s = structs[b]
            s.n[:] = n
            s.l[:] = l
            s.visc = 1. / case["visci"]
            s.dt = float(case["dt_f"])
            s.cbcvel = case["cbcvel"].encode()
            s.cbcpre = case["cbcpre"].encode()
            s.bcvel[:] = list(case.get("bcvel", [0.] * 18))
            s.bcpre[:] = list(case.get("bcpre", [0.] * 6))
            s.bforce[:] = list(case.get("bforce", [0.] * 3))
            s.dzc_g = dzc.ctypes.data_as(cans._D)
            s.dzf_g = dzf.ctypes.data_as(cans._D)
            for name in ("dzci", "dzfi", "u", "v", "w", "p", "pp", "dudtrko", "dvdtrko", "dwdtrko"):
                setattr(s, name, box[name].data_ptr())
            self.boxes.append(box)
        h = C.c_void_p()
        rc = cans.lib().cans_boxes_create(len(cases), structs, int(is_impdiff), int(bool(autotune)),
                                          C.c_void_p(self.stream.cuda_stream), C.byref(h))
        if rc != 0:
            raise cans.CansError(rc, "cans_boxes_create")
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and cans._lib is not None:
            cans._lib.cans_boxes_destroy(h)
            self._h = None

    def _call(self, name, *args):
        rc = getattr(cans.lib(), name)(self._h, *args)
        if rc != 0:
            raise cans.CansError(rc, name)

    def start(self):
        import torch
        torch.cuda.synchronize()
        self._call("cans_boxes_start")

    def substep(self, irk):
        self._call("cans_boxes_substep", int(irk))

    def step(self, nsteps=1, use_graph=False):
        for _ in range(nsteps):
            self._call("cans_boxes_step", int(bool(use_graph)))

    @property
    def graph_nodes(self):
        return cans.lib().cans_boxes_graph_nodes(self._h)

    def synchronize(self):
        self.stream.synchronize()
