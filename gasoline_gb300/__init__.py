"""gasoline_gb300: GB300-native TreeSPH force path (gravity tree walk with
Ewald, SPH density and pressure gathers, kick-drift-kick) behind the C ABI
declared in include/tsph.h.

This module is a thin ctypes binding of libtsph for tests, the benchmark
and Python callers.  It mirrors the reference's per-rank entry points:
``Context.grav_all`` is pkdGravAll (pkd.c:2869) including the tree build it
needs, ``Context.smooth`` is smInitialize+smSmooth/smReSmooth+smFinish
(smooth.c:54-1749) for SMX_DENDVDX and SMX_SPHPRESSURETERMS.

There is no CPU fallback: if libtsph is missing or no GPU is present the
calls raise.
"""
import ctypes
import os

import numpy as np

from . import ics  # noqa: F401  (re-exported workload generators)

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "_lib", "libtsph.so")

FP64 = 0
FP32 = 1
SMX_DENSITY = 1
SMX_SPHPRESSURETERMS = 22
SMX_DENDVDX = 23

_P = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_UP = ctypes.POINTER(ctypes.c_ulonglong)


class GravParams(ctypes.Structure):
    """tsph_grav_params (include/tsph.h)."""
    _fields_ = [("nBucket", ctypes.c_int), ("iOrder", ctypes.c_int),
                ("bPeriodic", ctypes.c_int), ("bEwald", ctypes.c_int),
                ("iEwOrder", ctypes.c_int), ("nReps", ctypes.c_int),
                ("dTheta", ctypes.c_double), ("dPeriod", ctypes.c_double),
                ("fEwCut", ctypes.c_double), ("fEwhCut", ctypes.c_double),
                ("precision", ctypes.c_int), ("reserved", ctypes.c_int)]


class GravOut(ctypes.Structure):
    _fields_ = [("nActive", ctypes.c_int), ("nBuckets", ctypes.c_int),
                ("dPartSum", ctypes.c_double), ("dCellSum", ctypes.c_double),
                ("dSoftSum", ctypes.c_double), ("dFlop", ctypes.c_double),
                ("dFlopEwald", ctypes.c_double), ("dExactFrac", ctypes.c_double),
                ("dTests", ctypes.c_double), ("dVisits", ctypes.c_double)]


class SphParams(ctypes.Structure):
    _fields_ = [("nSmooth", ctypes.c_int), ("bPeriodic", ctypes.c_int),
                ("dPeriod", ctypes.c_double), ("alpha", ctypes.c_double),
                ("beta", ctypes.c_double), ("gamma", ctypes.c_double),
                ("dEtaCourant", ctypes.c_double),
                ("iViscosityLimiter", ctypes.c_int), ("precision", ctypes.c_int),
                ("bLearnedH", ctypes.c_int), ("reserved", ctypes.c_int)]


class SmoothOut(ctypes.Structure):
    _fields_ = [("nSmoothed", ctypes.c_int), ("nFallback", ctypes.c_int),
                ("dPairs", ctypes.c_double), ("dCandidates", ctypes.c_double),
                ("bSeeded", ctypes.c_int), ("reserved", ctypes.c_int)]


def grav_params(nBucket=8, iOrder=2, periodic=False, ewald=True, iEwOrder=4,
                nReps=1, theta=0.7, L=1.0, fEwCut=2.6, fEwhCut=2.8,
                precision=FP64):
    return GravParams(nBucket, iOrder, int(periodic), int(ewald), iEwOrder,
                      nReps, theta, L, fEwCut, fEwhCut, precision, 0)


def sph_params(nSmooth=32, periodic=False, L=1.0, alpha=1.0, beta=2.0,
               gamma=5.0 / 3.0, dEtaCourant=0.4, limiter=1, precision=FP64,
               learned_h=False):
    return SphParams(nSmooth, int(periodic), L, alpha, beta, gamma,
                     dEtaCourant, limiter, precision, int(learned_h), 0)


class Tuning(ctypes.Structure):
    """tsph_tuning (include/tsph.h): launch-shape knobs, result-neutral."""
    _fields_ = [("taskSize", ctypes.c_int), ("walkBlocksPerSM", ctypes.c_int),
                ("walkGroup", ctypes.c_int), ("walkLists", ctypes.c_int),
                ("reserved", ctypes.c_int * 4)]


STORE_INT_FIELDS = ("r", "fMass", "fSoft", "v", "vPred", "u", "uPred", "a", "fPot", "dtGrav",
                    "fBall2", "fDensity", "divv", "curlv", "dvds", "BalsaraSwitch", "diff",
                    "PoverRho2", "c", "uDotPdV", "uDotAV", "mumax", "dtNew", "iActive")


class StoreLayout(ctypes.Structure):
    """tsph_store_layout (include/tsph.h): stride and byte offsets of the
    fields of a particle store laid out as the reference's PARTICLE."""
    _fields_ = ([("stride", ctypes.c_longlong)] + [(k, ctypes.c_int) for k in STORE_INT_FIELDS] +
                [("activeBit", ctypes.c_uint), ("reserved", ctypes.c_int * 6)])


def store_layout(offsets):
    """A StoreLayout from a dict of offsets (missing fields: -1)."""
    L = StoreLayout()
    L.stride = int(offsets["stride"])
    for k in STORE_INT_FIELDS:
        setattr(L, k, int(offsets.get(k, -1)))
    L.activeBit = int(offsets.get("activeBit", 1))
    return L


class StepParams(ctypes.Structure):
    """tsph_step_params: adaptive-timestep criteria (the reference's defaults,
    master.c:572-623)."""
    _fields_ = [("iMaxRung", ctypes.c_int), ("dEta", ctypes.c_double),
                ("bGravStep", ctypes.c_int), ("bEpsAccStep", ctypes.c_int),
                ("bSqrtPhiStep", ctypes.c_int), ("dEtauDot", ctypes.c_double),
                ("duMinDt", ctypes.c_double)]


def step_params(iMaxRung=4, dEta=0.1, bGravStep=0, bEpsAccStep=1, bSqrtPhiStep=0,
                dEtauDot=0.25, duMinDt=0.0):
    return StepParams(iMaxRung, dEta, bGravStep, bEpsAccStep, bSqrtPhiStep, dEtauDot, duMinDt)


class StepOut(ctypes.Structure):
    _fields_ = [("iCurrMaxRung", ctypes.c_int), ("nForcePasses", ctypes.c_int),
                ("nActiveSum", ctypes.c_longlong), ("nEmergency", ctypes.c_int)]


class RenderParams(ctypes.Structure):
    """tsph_render_params: a TSC frame (dfRenderParticleTSC)."""
    _fields_ = [("nxPix", ctypes.c_int), ("nyPix", ctypes.c_int),
                ("r", ctypes.c_double * 3), ("x", ctypes.c_double * 3),
                ("y", ctypes.c_double * 3), ("z", ctypes.c_double * 3),
                ("zEye", ctypes.c_double), ("zClipNear", ctypes.c_double),
                ("zClipFar", ctypes.c_double), ("iProject", ctypes.c_int),
                ("dGasSoftMul", ctypes.c_double), ("dDarkSoftMul", ctypes.c_double),
                ("dStarSoftMul", ctypes.c_double), ("bGasSph", ctypes.c_int),
                ("dMassGasMin", ctypes.c_double), ("dMassGasMax", ctypes.c_double),
                ("dMassDarkMin", ctypes.c_double), ("dMassDarkMax", ctypes.c_double),
                ("dMassStarMin", ctypes.c_double), ("dMassStarMax", ctypes.c_double),
                ("bColMassWeight", ctypes.c_int), ("bColLogInterp", ctypes.c_int),
                ("nColGas", ctypes.c_int), ("nColDark", ctypes.c_int), ("nColStar", ctypes.c_int),
                ("dColGas", ctypes.c_float * 10), ("dColDark", ctypes.c_float * 10),
                ("dColStar", ctypes.c_float * 10),
                ("colGas", (ctypes.c_float * 3) * 10), ("colDark", (ctypes.c_float * 3) * 10),
                ("colStar", (ctypes.c_float * 3) * 10)]


def render_params(nx=320, ny=240, centre=(0.0, 0.0, 0.0), width=2.0, perspective=False,
                  zEye=0.0, zClip=(-1e30, 1e30), gas_col=((1.0, 0.5, 0.2),), gas_levels=(),
                  dark_col=((0.3, 0.4, 1.0),), star_col=((1.0, 1.0, 1.0),), bGasSph=1,
                  soft_mul=(1.0, 1.0, 1.0), log_interp=0, mass_weight=0):
    """A face-on frame of `width` length units across, looking down z."""
    p = RenderParams()
    p.nxPix, p.nyPix = nx, ny
    s = nx / width
    p.r[:] = centre
    p.x[:] = (s, 0.0, 0.0)
    p.y[:] = (0.0, s, 0.0)
    p.z[:] = (0.0, 0.0, 1.0)
    p.zEye = zEye
    p.zClipNear, p.zClipFar = zClip
    p.iProject = 2 if perspective else 1
    p.dGasSoftMul, p.dDarkSoftMul, p.dStarSoftMul = soft_mul
    p.bGasSph = bGasSph
    big = 1e300
    p.dMassGasMin = p.dMassDarkMin = p.dMassStarMin = 0.0
    p.dMassGasMax = p.dMassDarkMax = p.dMassStarMax = big
    p.bColMassWeight, p.bColLogInterp = mass_weight, log_interp
    for cols, levels, cname, lname, nname in ((gas_col, gas_levels, "colGas", "dColGas", "nColGas"),
                                              (dark_col, (), "colDark", "dColDark", "nColDark"),
                                              (star_col, (), "colStar", "dColStar", "nColStar")):
        for k, c in enumerate(cols):
            getattr(p, cname)[k][:] = c
        for k, v in enumerate(levels):
            getattr(p, lname)[k] = v
        setattr(p, nname, len(levels))
    return p


class TipsyHeader(ctypes.Structure):
    """tsph_tipsy_header: the Tipsy file header (tipsydefs.h struct dump)."""
    _fields_ = [("time", ctypes.c_double), ("nbodies", ctypes.c_int), ("ndim", ctypes.c_int),
                ("nsph", ctypes.c_int), ("ndark", ctypes.c_int), ("nstar", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


def tipsy_header(path, standard=True):
    """The header of a Tipsy snapshot, as a dict."""
    h = TipsyHeader()
    rc = load().tsph_tipsy_read_header(os.fsencode(path), int(standard), ctypes.byref(h))
    if rc:
        raise TsphError(rc, load().tsph_error_string(rc).decode())
    return h.as_dict()


class TsphError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libtsph error {code}: {msg}")
        self.code = code


_lib = None


def load():
    """Load libtsph; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise RuntimeError(
            f"{LIBPATH} not built: run `python -m gasoline_gb300.build`")
    lib = ctypes.CDLL(LIBPATH)
    lib.tsph_error_string.restype = ctypes.c_char_p
    lib.tsph_last_cuda_error.restype = ctypes.c_char_p
    lib.tsph_launch_count.restype = ctypes.c_longlong
    for name in ("tsph_create", "tsph_set_particles", "tsph_set_velocities",
                 "tsph_grav_all", "tsph_get_gravity", "tsph_get_tree",
                 "tsph_get_lists", "tsph_smooth", "tsph_get_sph",
                 "tsph_get_neighbour_hash", "tsph_kick", "tsph_drift",
                 "tsph_get_state", "tsph_get_timings", "tsph_fma_peak",
                 "tsph_hnet_init", "tsph_hnet_set_params", "tsph_hnet_get_params",
                 "tsph_hnet_loss_grad", "tsph_hnet_mode", "tsph_hnet_train",
                 "tsph_hnet_info", "tsph_hnet_num_params", "tsph_set_tuning",
                 "tsph_get_tuning", "tsph_set_systems", "tsph_step",
                 "tsph_step_status", "tsph_tipsy_read_header", "tsph_read_tipsy",
                 "tsph_write_tipsy", "tsph_get_snapshot_fields",
                 "tsph_set_snapshot_fields", "tsph_kick_rung", "tsph_top_step_kdk",
                 "tsph_set_active_rung", "tsph_set_rungs", "tsph_get_rungs", "tsph_render_tsc",
                 "tsph_update_particles", "tsph_store_register", "tsph_store_unregister",
                 "tsph_store_load", "tsph_store_put_gravity", "tsph_store_put_sph"):
        getattr(lib, name).restype = ctypes.c_int
    lib.tsph_destroy.restype = None
    _lib = lib
    return lib


def _d(a):
    return a.ctypes.data_as(_P)


def _c64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


class Context:
    """One libtsph context (one GPU, one stream)."""

    def __init__(self, device=0, stream=None):
        self.lib = load()
        self._ctx = ctypes.c_void_p()
        s = ctypes.c_void_p(stream) if stream else None
        self._check(self.lib.tsph_create(ctypes.byref(self._ctx), device, s))
        self.n = 0
        self.ngas = 0

    def close(self):
        if self._ctx:
            self.lib.tsph_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            msg = self.lib.tsph_error_string(rc).decode()
            if self._ctx:
                cu = self.lib.tsph_last_cuda_error(self._ctx).decode()
                if cu:
                    msg += f" ({cu})"
            raise TsphError(rc, msg)

    # ---- particles ------------------------------------------------------
    def set_particles(self, pos, mass, soft):
        pos = _c64(pos, (-1, 3))
        mass = _c64(mass)
        soft = _c64(soft)
        self.n = len(mass)
        self._check(self.lib.tsph_set_particles(
            self._ctx, self.n, _d(pos), _d(mass), _d(soft)))

    def set_particles_ptr(self, n, pos_ptr, mass_ptr, soft_ptr):
        """Same as set_particles from raw host pointers (e.g. pinned)."""
        self.n = n
        self._check(self.lib.tsph_set_particles(
            self._ctx, n, ctypes.cast(pos_ptr, _P), ctypes.cast(mass_ptr, _P),
            ctypes.cast(soft_ptr, _P)))

    def update_particles_ptr(self, n, pos_ptr, mass_ptr, soft_ptr):
        """tsph_update_particles from raw host pointers: new values for the
        particles already loaded, their order kept."""
        self.n = n
        self._check(self.lib.tsph_update_particles(
            self._ctx, n, ctypes.cast(pos_ptr, _P), ctypes.cast(mass_ptr, _P),
            ctypes.cast(soft_ptr, _P)))

    def update_particles(self, pos, mass, soft):
        pos = _c64(pos, (-1, 3))
        mass = _c64(mass)
        soft = _c64(soft)
        self.n = len(mass)
        self._check(self.lib.tsph_update_particles(self._ctx, self.n, _d(pos), _d(mass), _d(soft)))

    def set_velocities(self, vel, ngas=0, u=None):
        vel = _c64(vel, (-1, 3))
        self.ngas = ngas
        up = _d(_c64(u)) if u is not None else None
        if u is not None:
            self._u_keep = _c64(u)
            up = _d(self._u_keep)
        self._check(self.lib.tsph_set_velocities(self._ctx, _d(vel), ngas, up))

    # ---- gravity ----------------------------------------------------------
    def grav_all(self, gp):
        out = GravOut()
        self._check(self.lib.tsph_grav_all(self._ctx, ctypes.byref(gp),
                                           ctypes.byref(out)))
        return {f: getattr(out, f) for f, _ in GravOut._fields_}

    def get_gravity(self):
        acc = np.zeros((self.n, 3))
        pot = np.zeros(self.n)
        dtg = np.zeros(self.n)
        self._check(self.lib.tsph_get_gravity(self._ctx, _d(acc), _d(pot),
                                              _d(dtg)))
        return dict(acc=acc, pot=pot, dtGrav=dtg)

    def get_gravity_ptr(self, acc_ptr):
        self._check(self.lib.tsph_get_gravity(
            self._ctx, ctypes.cast(acc_ptr, _P), None, None))

    def get_tree(self):
        nn = ctypes.c_int()
        self._check(self.lib.tsph_get_tree(self._ctx, ctypes.byref(nn), None,
                                           None, None))
        inode = np.zeros((nn.value, 6), dtype=np.int32)
        dnode = np.zeros((nn.value, 16))
        perm = np.zeros(self.n, dtype=np.int32)
        self._check(self.lib.tsph_get_tree(
            self._ctx, ctypes.byref(nn), inode.ctypes.data_as(_IP), _d(dnode),
            perm.ctypes.data_as(_IP)))
        return inode, dnode, perm

    def get_lists(self):
        nb = ctypes.c_int()
        self._check(self.lib.tsph_get_lists(self._ctx, ctypes.byref(nb), None))
        bl = np.zeros((nb.value, 4), dtype=np.int32)
        self._check(self.lib.tsph_get_lists(self._ctx, ctypes.byref(nb),
                                            bl.ctypes.data_as(_IP)))
        return bl

    # ---- SPH ----------------------------------------------------------------
    def smooth(self, smx_type, sp):
        out = SmoothOut()
        self._check(self.lib.tsph_smooth(self._ctx, smx_type, ctypes.byref(sp),
                                         ctypes.byref(out)))
        return {f: getattr(out, f) for f, _ in SmoothOut._fields_}

    def get_sph(self):
        out = np.zeros((self.ngas, 16))
        dtn = np.zeros(self.ngas)
        mum = np.zeros(self.ngas)
        self._check(self.lib.tsph_get_sph(self._ctx, _d(out), _d(dtn), _d(mum)))
        names = ["fBall2", "fDensity", "divv", "curlv_x", "curlv_y",
                 "curlv_z", "dvds", "BalsaraSwitch", "diff", "PoverRho2", "c",
                 "ax", "ay", "az", "uDotPdV", "uDotAV"]
        res = {k: out[:, i].copy() for i, k in enumerate(names)}
        res["dtNew"] = dtn
        res["mumax"] = mum
        return res

    def get_neighbour_hash(self):
        cnt = np.zeros(self.ngas, dtype=np.int32)
        hsh = np.zeros(self.ngas, dtype=np.uint64)
        self._check(self.lib.tsph_get_neighbour_hash(
            self._ctx, cnt.ctypes.data_as(_IP), hsh.ctypes.data_as(_UP)))
        return cnt, hsh

    # ---- KDK ----------------------------------------------------------------
    def kick(self, dt):
        self._check(self.lib.tsph_kick(self._ctx, ctypes.c_double(dt)))

    def drift(self, dt, periodic=False, L=1.0):
        self._check(self.lib.tsph_drift(self._ctx, ctypes.c_double(dt),
                                        int(periodic), ctypes.c_double(L)))

    def kick_rung(self, iRung, dt, close=True):
        """pkdKick on rung iRung (all particles when iRung < 0); close=False
        is the opening kick of a KDK step."""
        self._check(self.lib.tsph_kick_rung(self._ctx, int(iRung), ctypes.c_double(dt),
                                            int(close)))

    # ---- frames ---------------------------------------------------------------
    def render_tsc(self, rp, nstar=0):
        """A TSC frame of the loaded particles: float32 (nyPix, nxPix, 3)."""
        img = np.zeros((rp.nyPix, rp.nxPix, 3), dtype=np.float32)
        self._check(self.lib.tsph_render_tsc(self._ctx, ctypes.byref(rp), int(nstar),
                                             img.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return img

    # ---- adaptive timesteps ------------------------------------------------
    def top_step_kdk(self, t, dt, gp, sp, st):
        """One base step dt with rungs (tsph_top_step_kdk); returns its
        counters."""
        out = StepOut()
        self._check(self.lib.tsph_top_step_kdk(self._ctx, ctypes.c_double(t), ctypes.c_double(dt),
                                               ctypes.byref(gp),
                                               ctypes.byref(sp) if sp is not None else None,
                                               ctypes.byref(st), ctypes.byref(out)))
        return {f: getattr(out, f) for f, _ in StepOut._fields_}

    def set_active_rung(self, iRung):
        self._check(self.lib.tsph_set_active_rung(self._ctx, int(iRung)))

    def set_rungs(self, rung):
        r = np.ascontiguousarray(rung, dtype=np.int32)
        self._check(self.lib.tsph_set_rungs(self._ctx, r.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))

    def get_rungs(self):
        """rung (int32), dt, dtNew, mumax of every particle (caller order)."""
        n = self.n
        r = np.zeros(n, dtype=np.int32)
        dt, dtn, mu = np.zeros(n), np.zeros(n), np.zeros(n)
        self._check(self.lib.tsph_get_rungs(self._ctx, r.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                            _d(dt), _d(dtn), _d(mu)))
        return dict(rung=r, dt=dt, dtNew=dtn, mumax=mu)

    def get_state(self):
        pos = np.zeros((self.n, 3))
        vel = np.zeros((self.n, 3))
        u = np.zeros(max(self.ngas, 1))
        self._check(self.lib.tsph_get_state(self._ctx, _d(pos), _d(vel), _d(u)))
        return pos, vel, u[:self.ngas]

    # ---- Tipsy snapshots -------------------------------------------------------
    def read_tipsy(self, path, standard=True, dvFac=1.0, dTuFac=1.0):
        """Load a Tipsy snapshot (pkdReadTipsy pkd.c:297): replaces the
        particles, the first nsph of them gas.  Returns the header."""
        h = TipsyHeader()
        self._check(self.lib.tsph_read_tipsy(self._ctx, os.fsencode(path), int(standard),
                                             ctypes.c_double(dvFac), ctypes.c_double(dTuFac),
                                             ctypes.byref(h)))
        self.n = h.nbodies
        self.ngas = h.nsph
        self.nstar = h.nstar
        return h.as_dict()

    def write_tipsy(self, path, time, standard=True, dvFac=1.0, duTFac=1.0, nstar=None):
        """Write the particles as a Tipsy snapshot (pkdWriteTipsy pkd.c:1628);
        the last `nstar` particles are stars (default: as read in, else 0)."""
        if nstar is None:
            nstar = getattr(self, "nstar", 0)
        self._check(self.lib.tsph_write_tipsy(self._ctx, os.fsencode(path), int(standard),
                                              ctypes.c_double(time), int(nstar),
                                              ctypes.c_double(dvFac), ctypes.c_double(duTFac)))

    def get_snapshot_fields(self):
        """mass, soft, pot (float64) and the snapshot's rho, metals, tform
        (float32), in caller order."""
        n = self.n
        mass, soft, pot = np.zeros(n), np.zeros(n), np.zeros(n)
        rho, met, tf = (np.zeros(n, dtype=np.float32) for _ in range(3))
        fp = ctypes.POINTER(ctypes.c_float)
        self._check(self.lib.tsph_get_snapshot_fields(
            self._ctx, _d(mass), _d(soft), _d(pot), rho.ctypes.data_as(fp),
            met.ctypes.data_as(fp), tf.ctypes.data_as(fp)))
        return dict(mass=mass, soft=soft, pot=pot, rho=rho, metals=met, tform=tf)

    def set_snapshot_fields(self, pot=None, rho=None, metals=None, tform=None):
        """Set the potential (float64) and the snapshot's rho, metals, tform
        (stored as float32) of the loaded particles; None keeps a field."""
        fp = ctypes.POINTER(ctypes.c_float)
        keep = []

        def f32(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float32)
            keep.append(a)
            return a.ctypes.data_as(fp)
        potp = None
        if pot is not None:
            pot = _c64(pot)
            keep.append(pot)
            potp = _d(pot)
        self._check(self.lib.tsph_set_snapshot_fields(self._ctx, potp, f32(rho), f32(metals),
                                                      f32(tform)))

    # ---- learned smoothing length ---------------------------------------------
    def hnet_init(self, seed=1):
        self._check(self.lib.tsph_hnet_init(self._ctx, ctypes.c_ulonglong(seed)))

    def hnet_params(self):
        n = self.lib.tsph_hnet_num_params()
        w = np.zeros(n, dtype=np.float32)
        self._check(self.lib.tsph_hnet_get_params(
            self._ctx, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), n))
        return w

    def hnet_set_params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._check(self.lib.tsph_hnet_set_params(
            self._ctx, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(w)))

    def hnet_loss_grad(self, x, y):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        n = self.lib.tsph_hnet_num_params()
        g = np.zeros(n, dtype=np.float32)
        loss = ctypes.c_double()
        fp = ctypes.POINTER(ctypes.c_float)
        self._check(self.lib.tsph_hnet_loss_grad(
            self._ctx, len(y), x.ctypes.data_as(fp), y.ctypes.data_as(fp),
            g.ctypes.data_as(fp), ctypes.byref(loss)))
        return loss.value, g

    def hnet_mode(self, collect=False, predict=False, margin=0.05):
        self._check(self.lib.tsph_hnet_mode(self._ctx, int(collect), int(predict),
                                            ctypes.c_double(margin)))

    def hnet_train(self, steps=2000, batch=8192, lr=3e-3):
        loss = ctypes.c_double()
        self._check(self.lib.tsph_hnet_train(self._ctx, steps, batch,
                                             ctypes.c_double(lr), ctypes.byref(loss)))
        return loss.value

    def hnet_info(self):
        n = ctypes.c_longlong()
        st = (ctypes.c_float * 8)()
        self._check(self.lib.tsph_hnet_info(self._ctx, ctypes.byref(n), st))
        return int(n.value), list(st)

    def timings(self):
        t = (ctypes.c_float * 8)()
        self._check(self.lib.tsph_get_timings(self._ctx, t))
        keys = ["build", "moments", "walk", "ewald", "knn", "density",
                "pressure", "total"]
        return {k: float(t[i]) for i, k in enumerate(keys)}

    def launches(self):
        return int(self.lib.tsph_launch_count(self._ctx))

    def set_systems(self, sys_of, nsys=None):
        """Independent systems (tsph_set_systems): sys_of[i] is the system
        of caller particle i."""
        so = np.ascontiguousarray(sys_of, dtype=np.int32)
        if nsys is None:
            nsys = int(so.max()) + 1 if len(so) else 1
        self._check(self.lib.tsph_set_systems(self._ctx, int(nsys), so.ctypes.data_as(_IP)))

    def step(self, dt, gp, sp=None, graph=False):
        """One kick-drift-kick step (tsph_step); with graph=True the step is
        captured once as a CUDA graph and replayed.  Queued only: call
        step_status() to wait and collect errors."""
        self._check(self.lib.tsph_step(self._ctx, ctypes.c_double(dt), ctypes.byref(gp),
                                       ctypes.byref(sp) if sp is not None else None,
                                       1 if graph else 0))

    def step_status(self):
        """Wait for queued steps; raise on the first error they raised."""
        self._check(self.lib.tsph_step_status(self._ctx))

    # --- a particle store in the reference's PARTICLE layout (numpy
    # structured arrays here) ---
    def store_register(self, store):
        self._check(self.lib.tsph_store_register(self._ctx, ctypes.c_void_p(store.ctypes.data),
                                                 ctypes.c_size_t(store.nbytes)))

    def store_unregister(self, store):
        self._check(self.lib.tsph_store_unregister(self._ctx, ctypes.c_void_p(store.ctypes.data)))

    @staticmethod
    def _order(order):
        if order is None:
            return None, None
        o = np.ascontiguousarray(order, dtype=np.int32)
        return o, o.ctypes.data_as(ctypes.POINTER(ctypes.c_int))

    def store_load(self, store, layout, order=None, ngas=0):
        o, op = self._order(order)
        self._check(self.lib.tsph_store_load(self._ctx, len(store), ctypes.c_void_p(store.ctypes.data),
                                             ctypes.byref(layout), op, int(ngas)))

    def store_put_gravity(self, store, layout, order=None):
        o, op = self._order(order)
        self._check(self.lib.tsph_store_put_gravity(self._ctx, ctypes.c_void_p(store.ctypes.data),
                                                    ctypes.byref(layout), op))

    def store_put_sph(self, which, store, layout, order=None):
        o, op = self._order(order)
        self._check(self.lib.tsph_store_put_sph(self._ctx, int(which), ctypes.c_void_p(store.ctypes.data),
                                                ctypes.byref(layout), op))

    def set_tuning(self, taskSize=0, walkBlocksPerSM=0, walkGroup=0, walkLists=0):
        t = Tuning(taskSize, walkBlocksPerSM, walkGroup, walkLists)
        self._check(self.lib.tsph_set_tuning(self._ctx, ctypes.byref(t)))

    def get_tuning(self):
        t = Tuning()
        self._check(self.lib.tsph_get_tuning(self._ctx, ctypes.byref(t)))
        return {"taskSize": t.taskSize, "walkBlocksPerSM": t.walkBlocksPerSM,
                "walkGroup": t.walkGroup, "walkLists": t.walkLists}
