"""Host-side step driver over libtsph, in the reference's kick-drift-kick
order (msrTopStepKDK, master.c:8242-8465):

    forces(t=0)                              (main.c:363-387, msrInitSph)
    repeat:  kick_open(dt/2); drift(dt/2); drift(dt/2); forces(); kick_close(dt/2)

where forces() = gravity (pkdGravAll) and, for the gas particles, the
density pass (SMX_DENDVDX), gas pressure and the pressure pass
(SMX_SPHPRESSURETERMS).  `top_step` runs the same with adaptive rungs
(tsph_top_step_kdk).
"""
import time

import numpy as np

from . import Context, FP32, FP64, SMX_DENDVDX, SMX_SPHPRESSURETERMS, grav_params, sph_params


class Simulation:
    def __init__(self, pos, vel, mass, soft, ngas=0, u=None, periodic=False, L=1.0,
                 theta=0.7, nBucket=8, nSmooth=32, precision=FP32, sph_precision=FP64,
                 gravity=True, device=0, ctx=None):
        self.ctx = ctx or Context(device)
        self.ctx.set_particles(pos, mass, soft)
        self.ctx.set_velocities(vel, ngas=ngas, u=u if u is not None else np.zeros(0))
        self.ngas = ngas
        self.gravity = gravity
        self.periodic = periodic
        self.L = L
        self.gp = grav_params(nBucket=nBucket, periodic=periodic, L=L, theta=theta,
                              precision=precision)
        self.sp = sph_params(nSmooth=nSmooth, periodic=periodic, L=L, precision=sph_precision)
        self.learned_h = False
        self.step_count = 0
        self.log = []

    def forces(self):
        t0 = time.perf_counter()
        rec = {}
        if self.gravity:
            rec["grav"] = self.ctx.grav_all(self.gp)
            tg = self.ctx.timings()
            rec["t_grav_ms"] = tg["total"]
        if self.ngas > 0:
            self.sp.bLearnedH = int(self.learned_h)
            rec["density"] = self.ctx.smooth(SMX_DENDVDX, self.sp)
            rec["pressure"] = self.ctx.smooth(SMX_SPHPRESSURETERMS, self.sp)
            t = self.ctx.timings()
            rec["t_knn_tree_ms"] = t["knn"]
            rec["t_knn_density_ms"] = t["density"]
            rec["t_pressure_ms"] = t["pressure"]
        rec["wall_s"] = time.perf_counter() - t0
        return rec

    def step(self, dt):
        self.ctx.kick_rung(-1, 0.5 * dt, close=False)
        self.ctx.drift(0.5 * dt, self.periodic, self.L)
        self.ctx.drift(0.5 * dt, self.periodic, self.L)
        rec = self.forces()
        self.ctx.kick_rung(-1, 0.5 * dt, close=True)
        self.step_count += 1
        rec["step"] = self.step_count
        self.log.append(rec)
        return rec

    def top_step(self, dt, st, t=0.0):
        """One base step dt with adaptive rungs (msrTopStepKDK with rungs)."""
        t0 = time.perf_counter()
        sp = self.sp if self.ngas > 0 else None
        rec = self.ctx.top_step_kdk(t, dt, self.gp, sp, st)
        rec["wall_s"] = time.perf_counter() - t0
        self.step_count += 1
        rec["step"] = self.step_count
        self.log.append(rec)
        return rec

    def state(self):
        return self.ctx.get_state()
