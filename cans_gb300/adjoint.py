"""Reverse-mode gradients of a CaNS run through the library's hand-written adjoint kernels.

`AdjointRun(case)` wraps `driver.Simulation` for explicit or implicit diffusion
(`is_impdiff`: the three velocity Helmholtz solves of src/main.f90:455-463 and updatep's
alpha lap(pp) term are reversed too), a fixed time step (`dt_f`) and no flow-rate forcing.  `forward(u0, v0, w0, bforce, nsteps)` runs the model
from the given interior initial velocity and uniform body force and returns

    J = 1/2 sum over interior cells of (u^2 dx dy dzf + v^2 dx dy dzf + w^2 dx dy dzc),

the volume-integrated kinetic energy after `nsteps` steps, keeping the state (u, v, w, p)
every `ckpt_every` steps.  `backward()` returns dJ/d(u0, v0, w0) (interior arrays) and
dJ/d(bforce): it walks the segments between checkpoints backwards, recomputes each
segment's substep inputs from its checkpoint, and applies the adjoint of every substep
(src/main.f90:452-472 in reverse: boundp, updatep, bounduvw, correc, boundp, solver,
fillps, bounduvw, the Helmholtz solves when diffusion is implicit, rk) and finally that of
the initial boundary fills
(src/main.f90:388-418).  Device memory: one checkpoint per `ckpt_every` steps plus
3 x 3 x ckpt_every velocity fields of the segment being reversed.
"""
import numpy as np

from . import cans
from .driver import RKCOEFF, Simulation


class AdjointRun:
    def __init__(self, case, device="cuda", ckpt_every=10):
        if any(int(x) for x in case.get("is_forced", [0, 0, 0])):
            raise ValueError("adjoint: no flow-rate forcing")
        if not case.get("dt_f", -1.) > 0.:
            raise ValueError("adjoint: fixed time step (dt_f > 0) required")
        self.case = dict(case)
        self.case["icheck"] = 0
        self.device = device
        self.ckpt_every = int(ckpt_every)
        self.sim = Simulation(self.case, device=device)
        self.work = cans.rk_adjoint_work(self.sim.n, device)

    # ------------------------------------------------------------------ forward
    def _set_initial(self, u0, v0, w0, bforce):
        import torch
        s = self.sim
        for f, a in ((s.u, u0), (s.v, v0), (s.w, w0), (s.p, None)):
            f.zero_()
            if a is not None:
                f[1:-1, 1:-1, 1:-1] = a
        for d in (s.dudtrko, s.dvdtrko, s.dwdtrko, s.pp):
            d.zero_()
        s.bforce = [float(x) for x in bforce]
        s.dpdl[:] = 0.
        s.start()
        torch.cuda.synchronize()

    def _weights(self):
        import torch
        s = self.sim
        dxdy = s.dl[0] * s.dl[1]
        wf = torch.tensor(s.dzf[1:-1] * dxdy, dtype=torch.float64, device=self.device).view(-1, 1, 1)
        wc = torch.tensor(s.dzc[1:-1] * dxdy, dtype=torch.float64, device=self.device).view(-1, 1, 1)
        return wf, wc

    def energy(self):
        s = self.sim
        wf, wc = self._weights()
        i = (slice(1, -1),) * 3
        return float(0.5 * ((s.u[i] ** 2 * wf).sum() + (s.v[i] ** 2 * wf).sum() + (s.w[i] ** 2 * wc).sum()))

    def _state(self):
        s = self.sim
        return tuple(t.clone() for t in (s.u, s.v, s.w, s.p))

    def _restore(self, st):
        s = self.sim
        for f, a in zip((s.u, s.v, s.w, s.p), st):
            f.copy_(a)

    def forward(self, u0, v0, w0, bforce, nsteps):
        """u0, v0, w0: interior initial velocity, device tensors (n3, n2, n1)."""
        self.nsteps = int(nsteps)
        self.bforce = [float(x) for x in bforce]
        self._set_initial(u0, v0, w0, bforce)
        self.ckpts = {}
        for step in range(self.nsteps):
            if step % self.ckpt_every == 0:
                self.ckpts[step] = self._state()
            self.sim.step(1)
        return self.energy()

    # ------------------------------------------------------------------ reverse
    def _adjoint_substep(self, irk, u_in, g):
        """g: dict of adjoints (gu, gv, gw, gp haloed; gdu, gdv, gdw flat) at the substep's
        output; updated in place to the adjoints at its input."""
        import torch
        s = self.sim
        n = s.n
        dtrk = (RKCOEFF[irk][0] + RKCOEFF[irk][1]) * s.dt
        alpha = -.5 * s.visc * dtrk if s.is_impdiff else 0.
        gu, gv, gw, gp = g["gu"], g["gv"], g["gw"], g["gp"]
        cans.boundp_adjoint(s.cbcpre, n, s.bcpre, s.is_bound, s.dl, s.dzc, gp, cans.HALO_UPPER)
        gpp = torch.zeros_like(gp)
        cans.updatep_adjoint(n, s.is_impdiff, gp, gpp, s.dli, s.dzci, s.dzfi, alpha)
        cans.bounduvw_adjoint(s.cbcvel, n, s.bcvel, s.is_bound, s.dl, s.dzc, s.dzf, gu, gv, gw, True, cans.HALO_UPPER,
                              cans.HALO_NONE)
        cans.correc_adjoint(n, s.dli, s.dzci, dtrk, gu, gv, gw, gpp)
        cans.boundp_adjoint(s.cbcpre, n, s.bcpre, s.is_bound, s.dl, s.dzc, gpp)
        s.plan_p.solve_adjoint(gpp)
        cans.fillps_adjoint(n, s.dli, s.dzfi, 1. / dtrk, gpp, gu, gv, gw)
        cans.bounduvw_adjoint(s.cbcvel, n, s.bcvel, s.is_bound, s.dl, s.dzc, s.dzf, gu, gv, gw, False,
                              cans.HALO_LOWER)
        if s.is_impdiff:  # the velocity Helmholtz solves (their boundary terms are constants)
            for c, gf in enumerate((gu, gv, gw)):
                s.plans_v[c].solve_helmholtz_adjoint(alpha, gf)
        gbf = cans.rk_adjoint(RKCOEFF[irk], n, s.dli, s.dzci, s.dzfi, s.dt, s.visc, u_in[0], u_in[1], u_in[2], gu, gv,
                              gw, g["gdu"], g["gdv"], g["gdw"], gp, self.work, is_impdiff=s.is_impdiff)
        g["gbf"] += gbf

    def backward(self):
        """returns (du0, dv0, dw0, dbforce): dJ w.r.t. the interior initial velocity and the
        body force"""
        import torch
        s = self.sim
        n = s.n
        wf, wc = self._weights()
        i = (slice(1, -1),) * 3
        # final state: dJ/du = u dx dy dzf (interior) ...
        self._restore_final = None
        g = {"gu": torch.zeros_like(s.u), "gv": torch.zeros_like(s.v), "gw": torch.zeros_like(s.w),
             "gp": torch.zeros_like(s.p), "gdu": torch.zeros_like(s.dudtrko), "gdv": torch.zeros_like(s.dvdtrko),
             "gdw": torch.zeros_like(s.dwdtrko), "gbf": np.zeros(3)}
        g["gu"][i] = s.u[i] * wf
        g["gv"][i] = s.v[i] * wf
        g["gw"][i] = s.w[i] * wc
        starts = sorted(self.ckpts)
        for seg, st in reversed(list(enumerate(starts))):
            end = starts[seg + 1] if seg + 1 < len(starts) else self.nsteps
            # recompute the segment, keeping every substep's input velocity
            self._restore(self.ckpts[st])
            inputs = []
            for _ in range(st, end):
                for irk in range(3):
                    inputs.append((s.u.clone(), s.v.clone(), s.w.clone()))
                    s.substep(irk)
            for e in reversed(range(len(inputs))):
                self._adjoint_substep(e % 3, inputs[e], g)
            del inputs
        # the initial boundary fills of start(): bounduvw (both halos) and boundp (upper)
        cans.boundp_adjoint(s.cbcpre, n, s.bcpre, s.is_bound, s.dl, s.dzc, g["gp"], cans.HALO_UPPER)
        cans.bounduvw_adjoint(s.cbcvel, n, s.bcvel, s.is_bound, s.dl, s.dzc, s.dzf, g["gu"], g["gv"], g["gw"], False)
        torch.cuda.synchronize()
        return g["gu"][i].clone(), g["gv"][i].clone(), g["gw"][i].clone(), g["gbf"].copy()
