"""CPU oracle for the TreeSPH force path (test infrastructure only).

Loads oracle/_build/liboracle.so (the C restatement of the reference's
algorithm in tsph_oracle.c) and, where it has been built in this checkout,
oracle/_ref/libgasref.so (the reference's own sources compiled by
build_ref.sh).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg use this package, as the checker; the product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(HERE, "_build", "liboracle.so")
_REF = os.path.join(HERE, "_ref", "libgasref.so")

_P = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_UP = ctypes.POINTER(ctypes.c_ulonglong)


class GravParams(ctypes.Structure):
    """Same field order as orc_grav_params / the reference harness."""
    _fields_ = [("nBucket", ctypes.c_int), ("iOrder", ctypes.c_int),
                ("bPeriodic", ctypes.c_int), ("bEwald", ctypes.c_int),
                ("iEwOrder", ctypes.c_int), ("nReps", ctypes.c_int),
                ("dTheta", ctypes.c_double), ("dPeriod", ctypes.c_double),
                ("fEwCut", ctypes.c_double), ("fEwhCut", ctypes.c_double)]


class SphParams(ctypes.Structure):
    _fields_ = [("nSmooth", ctypes.c_int), ("bPeriodic", ctypes.c_int),
                ("dPeriod", ctypes.c_double), ("alpha", ctypes.c_double),
                ("beta", ctypes.c_double), ("gamma", ctypes.c_double),
                ("dEtaCourant", ctypes.c_double), ("nBucket", ctypes.c_int),
                ("iViscosityLimiter", ctypes.c_int)]


class StepParams(ctypes.Structure):
    """Adaptive-timestep parameters (ref_step_params / the library's
    tsph_step_params), the reference's defaults (master.c:572-623)."""
    _fields_ = [("nSteps", ctypes.c_int), ("iMaxRung", ctypes.c_int),
                ("dDelta", ctypes.c_double), ("dEta", ctypes.c_double),
                ("bGravStep", ctypes.c_int), ("bEpsAccStep", ctypes.c_int),
                ("bSqrtPhiStep", ctypes.c_int), ("dEtauDot", ctypes.c_double),
                ("duMinDt", ctypes.c_double)]


def step_params(nSteps=1, iMaxRung=4, dDelta=0.01, dEta=0.1, bGravStep=0, bEpsAccStep=1,
                bSqrtPhiStep=0, dEtauDot=0.25, duMinDt=0.0):
    return StepParams(nSteps, iMaxRung, dDelta, dEta, bGravStep, bEpsAccStep, bSqrtPhiStep,
                      dEtauDot, duMinDt)


MULTISTEP_FIELDS = ("u", "uPred", "fPot", "dtGrav", "dt", "dtNew", "mumax", "fDensity",
                    "fBall2", "uDotPdV", "uDotAV", "rung")


def grav_params(nBucket=8, iOrder=2, periodic=False, ewald=True, iEwOrder=4,
                nReps=1, theta=0.7, L=1.0, fEwCut=2.6, fEwhCut=2.8):
    return GravParams(nBucket, iOrder, int(periodic), int(ewald), iEwOrder,
                      nReps, theta, L, fEwCut, fEwhCut)


def sph_params(nSmooth=32, periodic=False, L=1.0, alpha=1.0, beta=2.0,
               gamma=5.0 / 3.0, dEtaCourant=0.4, nBucket=8, limiter=1):
    return SphParams(nSmooth, int(periodic), L, alpha, beta, gamma,
                     dEtaCourant, nBucket, limiter)


SPH_FIELDS = ["fBall2", "fDensity", "divv", "curlv_x", "curlv_y", "curlv_z",
              "dvds", "BalsaraSwitch", "diff", "PoverRho2", "c", "ax", "ay",
              "az", "uDotPdV", "uDotAV"]


def build():
    subprocess.check_call(["sh", os.path.join(HERE, "build_oracle.sh")])


def reference_available():
    return os.path.exists(_REF)


def build_reference(refdir=None):
    """Compile the reference's own sources into oracle/_ref (build_ref.sh;
    refdir defaults to the recipe's: $GASOLINE_REFERENCE or its checkout)."""
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")] + ([refdir] if refdir else []))


def _d(a):
    return a.ctypes.data_as(_P)


def _c64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


class _Impl:
    def __init__(self, path, prefix):
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix
        self.lib[prefix + "grav"].restype = ctypes.c_int
        self.lib[prefix + "tree"].restype = ctypes.c_int
        self.lib[prefix + "lists"].restype = ctypes.c_int
        self.lib[prefix + "sph"].restype = ctypes.c_int

    def grav(self, pos, mass, soft, gp, nthreads=1):
        pos = _c64(pos, (-1, 3)); mass = _c64(mass); soft = _c64(soft)
        n = len(mass)
        acc = np.zeros((n, 3)); pot = np.zeros(n); dtg = np.zeros(n)
        cnt = np.zeros(5)
        f = self.lib[self.prefix + "grav"]
        if self.prefix == "orc_":
            f(n, _d(pos), _d(mass), _d(soft), ctypes.byref(gp), _d(acc), _d(pot),
              _d(dtg), _d(cnt), ctypes.c_int(nthreads))
        else:
            f(n, _d(pos), _d(mass), _d(soft), ctypes.byref(gp), _d(acc), _d(pot),
              _d(dtg), _d(cnt))
        return dict(acc=acc, pot=pot, dtGrav=dtg, counters=cnt)

    def tree(self, pos, mass, soft, gp):
        pos = _c64(pos, (-1, 3)); mass = _c64(mass); soft = _c64(soft)
        n = len(mass)
        f = self.lib[self.prefix + "tree"]
        nn = f(n, _d(pos), _d(mass), _d(soft), ctypes.byref(gp), None, None, None)
        inode = np.zeros((nn, 6), dtype=np.int32)
        dnode = np.zeros((nn, 16))
        perm = np.zeros(n, dtype=np.int32)
        f(n, _d(pos), _d(mass), _d(soft), ctypes.byref(gp),
          inode.ctypes.data_as(_IP), _d(dnode), perm.ctypes.data_as(_IP))
        return inode, dnode, perm

    def lists(self, pos, mass, soft, gp):
        pos = _c64(pos, (-1, 3)); mass = _c64(mass); soft = _c64(soft)
        n = len(mass)
        f = self.lib[self.prefix + "lists"]
        nb = f(n, _d(pos), _d(mass), _d(soft), ctypes.byref(gp), None)
        bl = np.zeros((nb, 4), dtype=np.int32)
        f(n, _d(pos), _d(mass), _d(soft), ctypes.byref(gp), bl.ctypes.data_as(_IP))
        return bl

    def sph(self, pos, vel, mass, soft, u, sp, nthreads=1):
        pos = _c64(pos, (-1, 3)); vel = _c64(vel, (-1, 3)); mass = _c64(mass)
        soft = _c64(soft); u = _c64(u)
        n = len(mass)
        out = np.zeros((n, 16)); dtn = np.zeros(n); mum = np.zeros(n)
        f = self.lib[self.prefix + "sph"]
        res = dict()
        if self.prefix == "orc_":
            cnt = np.zeros(n, dtype=np.int32)
            hsh = np.zeros(n, dtype=np.uint64)
            f(n, _d(pos), _d(vel), _d(mass), _d(soft), _d(u), ctypes.byref(sp),
              _d(out), _d(dtn), _d(mum), cnt.ctypes.data_as(_IP),
              hsh.ctypes.data_as(_UP), ctypes.c_int(nthreads))
            res["nbr_count"] = cnt
            res["nbr_hash"] = hsh
        else:
            f(n, _d(pos), _d(vel), _d(mass), _d(soft), _d(u), ctypes.byref(sp),
              _d(out), _d(dtn), _d(mum))
        for k, name in enumerate(SPH_FIELDS):
            res[name] = out[:, k].copy()
        res["dtNew"] = dtn
        res["mumax"] = mum
        return res


_oracle = None
_ref = None


def oracle():
    """The C restatement (always available once built)."""
    global _oracle
    if _oracle is None:
        if not os.path.exists(_LIB):
            build()
        _oracle = _Impl(_LIB, "orc_")
        _oracle.lib.orc_knn.restype = ctypes.c_int
    return _oracle


_ADAPT = os.path.join(HERE, "_ref", "libgasadapt.so")
_adapt = None


def adapter():
    """The reference harness with its gravity and SPH calls made through the
    reference-side binding of libtsph (gasoline_gb300/pkd/tsph_pkd.c) and a
    CPU stand-in of libtsph whose arithmetic is the oracle's
    (adapter_fake_tsph.c); None where the reference was not built."""
    global _adapt
    if _adapt is None and os.path.exists(_ADAPT):
        _adapt = _Impl(_ADAPT, "ref_")
    return _adapt


def reference():
    """The reference's own code, or None where it was not built."""
    global _ref
    if _ref is None and os.path.exists(_REF):
        _ref = _Impl(_REF, "ref_")
    return _ref


def reference_tipsy_write(path, standard, time, ngas, ndark, nstar, pos, vel, f,
                          dvFac=1.0, duTFac=1.0):
    """The reference's pkdWriteTipsy (after msrWriteTipsy's header) on these
    particles; f is (n, 9): mass, soft, u, rho, metals, tform, phi, 0, 0."""
    lib = reference().lib
    pos = _c64(pos, (-1, 3)); vel = _c64(vel, (-1, 3)); f = _c64(f, (-1, 9))
    rc = lib.ref_tipsy_write(os.fsencode(path), int(standard), ctypes.c_double(time), ngas,
                             ndark, nstar, ctypes.c_double(dvFac), ctypes.c_double(duTFac),
                             _d(pos), _d(vel), _d(f))
    if rc:
        raise OSError(f"ref_tipsy_write failed on {path}")


def reference_tipsy_read(path, standard, ngas, ndark, nstar, dvFac=1.0, dTuFac=1.0):
    """The reference's pkdReadTipsy: (pos, vel, f) in file order."""
    lib = reference().lib
    n = ngas + ndark + nstar
    pos = np.zeros((n, 3)); vel = np.zeros((n, 3)); f = np.zeros((n, 9))
    rc = lib.ref_tipsy_read(os.fsencode(path), int(standard), ngas, ndark, nstar,
                            ctypes.c_double(dvFac), ctypes.c_double(dTuFac), _d(pos), _d(vel), _d(f))
    if rc:
        raise OSError(f"ref_tipsy_read failed on {path}")
    return pos, vel, f


def reference_multistep(pos, vel, mass, soft, ngas, u, gp, sp, st):
    """The reference's msrTopStepKDK recursion (ref_multistep in the
    harness) for st.nSteps top steps after the initial forces."""
    lib = reference().lib
    pos = _c64(pos, (-1, 3)); vel = _c64(vel, (-1, 3)); mass = _c64(mass); soft = _c64(soft)
    n = len(mass)
    uu = _c64(u if ngas > 0 else np.zeros(1))
    opos = np.zeros((n, 3)); ovel = np.zeros((n, 3)); ovp = np.zeros((n, 3))
    oacc = np.zeros((n, 3)); f = np.zeros((n, 12))
    mr = np.zeros(max(st.nSteps, 1), dtype=np.int32); cnt = np.zeros(2)
    lib.ref_multistep(n, ngas, _d(pos), _d(vel), _d(mass), _d(soft), _d(uu), ctypes.byref(gp),
                      ctypes.byref(sp), ctypes.byref(st), _d(opos), _d(ovel), _d(ovp), _d(oacc),
                      _d(f), mr.ctypes.data_as(_IP), _d(cnt))
    out = dict(pos=opos, vel=ovel, vPred=ovp, acc=oacc, maxRung=mr[:st.nSteps], counts=cnt)
    for k, name in enumerate(MULTISTEP_FIELDS):
        out[name] = f[:, k].copy()
    out["rung"] = out["rung"].astype(np.int32)
    return out


def reference_grav_active(pos, mass, soft, rung, iRung, gp):
    """The reference's gravity pass over the particles with rung >= iRung."""
    lib = reference().lib
    pos = _c64(pos, (-1, 3)); mass = _c64(mass); soft = _c64(soft)
    r = np.ascontiguousarray(rung, dtype=np.int32)
    n = len(mass)
    acc = np.zeros((n, 3)); pot = np.zeros(n); dtg = np.zeros(n); cnt = np.zeros(5)
    lib.ref_grav_active(n, _d(pos), _d(mass), _d(soft), r.ctypes.data_as(_IP), int(iRung),
                        ctypes.byref(gp), _d(acc), _d(pot), _d(dtg), _d(cnt))
    return dict(acc=acc, pot=pot, dtGrav=dtg, counters=cnt)


def reference_sph_active(pos, vel, mass, soft, u, rung, iRung, sp):
    """The reference's SPH pass (all particles gas) with rung >= iRung active."""
    lib = reference().lib
    pos = _c64(pos, (-1, 3)); vel = _c64(vel, (-1, 3)); mass = _c64(mass)
    soft = _c64(soft); u = _c64(u)
    r = np.ascontiguousarray(rung, dtype=np.int32)
    n = len(mass)
    acc = np.zeros((n, 3)); f = np.zeros((n, 6))
    lib.ref_sph_active(n, _d(pos), _d(vel), _d(mass), _d(soft), _d(u), r.ctypes.data_as(_IP),
                       int(iRung), ctypes.byref(sp), _d(acc), _d(f))
    return dict(acc=acc, uDotPdV=f[:, 0].copy(), uDotAV=f[:, 1].copy(), dtNew=f[:, 2].copy(),
                mumax=f[:, 3].copy(), dt=f[:, 4].copy(), fDensity=f[:, 5].copy())


STORE_FIELDS = ["stride", "r", "fMass", "fSoft", "v", "vPred", "u", "uPred", "a", "fPot", "dtGrav",
                "fBall2", "fDensity", "divv", "curlv", "dvds", "BalsaraSwitch", "diff", "PoverRho2",
                "c", "uDotPdV", "uDotAV", "mumax", "dtNew", "iActive", "activeBit", "iOrder", "gasBit"]


def reference_particle_layout():
    """sizeof(PARTICLE) and the byte offsets of its fields in the reference
    build here (ref_particle_layout), keyed by STORE_FIELDS."""
    o = np.zeros(len(STORE_FIELDS), dtype=np.int64)
    reference().lib.ref_particle_layout(o.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
    return {k: int(v) for k, v in zip(STORE_FIELDS, o)}


def reference_knn_sets(pos, mass, soft, sp):
    """The reference's own smSmooth kNN sets (ref_knn_sets in the harness):
    per particle the nnList size, the order-independent hash of its members'
    input indices (the oracle's and the CUDA path's neighbour hash) and fBall2."""
    lib = reference().lib
    pos = _c64(pos, (-1, 3)); mass = _c64(mass); soft = _c64(soft)
    n = len(mass)
    hsh = np.zeros(n, dtype=np.uint64)
    cnt = np.zeros(n, dtype=np.int32)
    fb = np.zeros(n)
    lib.ref_knn_sets(n, _d(pos), _d(mass), _d(soft), ctypes.byref(sp), hsh.ctypes.data_as(_UP),
                     cnt.ctypes.data_as(_IP), _d(fb))
    return dict(nbr_hash=hsh, nbr_count=cnt, fBall2=fb)


def reference_render_tsc(pos, mass, soft, fBall2, fDensity, ngas, nstar, rp):
    """The reference's dfRenderParticles (TSC) frame: float32 (ny, nx, 3)."""
    lib = reference().lib
    arrs = [_c64(pos, (-1, 3)), _c64(mass), _c64(soft), _c64(fBall2), _c64(fDensity)]
    img = np.zeros((rp.nyPix, rp.nxPix, 3), dtype=np.float32)
    lib.ref_render_tsc(len(arrs[1]), int(ngas), int(nstar), *[_d(a) for a in arrs], ctypes.byref(rp),
                       img.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    return img


def knn_fball2(pos, nsmooth, periodic=False, L=1.0, nthreads=1):
    pos = _c64(pos, (-1, 3))
    n = pos.shape[0]
    out = np.zeros(n)
    oracle().lib.orc_knn(n, _d(pos), nsmooth, int(periodic), ctypes.c_double(L),
                         _d(out), nthreads)
    return out


class exact_rsqrt:
    """Context manager: the oracle takes 1/r as 1.0/sqrt(r2) instead of the
    reference's v_sqrt1 approximation while active."""

    def __enter__(self):
        oracle().lib.orc_set_exact_rsqrt(1)

    def __exit__(self, *a):
        oracle().lib.orc_set_exact_rsqrt(0)


def direct(pos, mass, soft, targets, nthreads=8):
    """FP64 direct-sum accelerations and potentials of the particles
    `targets` (indices) over all particles (orc_direct)."""
    pos = _c64(pos, (-1, 3)); mass = _c64(mass); soft = _c64(soft)
    q = np.ascontiguousarray(targets, dtype=np.int32)
    acc = np.zeros((len(q), 3)); pot = np.zeros(len(q))
    oracle().lib.orc_direct(len(mass), _d(pos), _d(mass), _d(soft), len(q),
                            q.ctypes.data_as(_IP), _d(acc), _d(pot), nthreads)
    return acc, pot


def ewald_direct(pos, mass, soft, targets, L=1.0, nthreads=8):
    """Exact periodic accelerations of `targets` by a pairwise Ewald sum
    (orc_ewald_direct)."""
    pos = _c64(pos, (-1, 3)); mass = _c64(mass); soft = _c64(soft)
    q = np.ascontiguousarray(targets, dtype=np.int32)
    acc = np.zeros((len(q), 3))
    oracle().lib.orc_ewald_direct(len(mass), _d(pos), _d(mass), _d(soft), ctypes.c_double(L),
                                  len(q), q.ctypes.data_as(_IP), _d(acc), nthreads)
    return acc


def v_sqrt1(r2):
    r2 = _c64(r2)
    out = np.zeros_like(r2)
    oracle().lib.orc_v_sqrt1(len(r2), _d(r2), _d(out))
    return out


def kdk(which, dt, pos, vel, acc, ngas=0, u=None, udot=None, periodic=False,
        L=1.0):
    """In-place KDK half step on float64 arrays (see orc_kdk)."""
    n = pos.shape[0]
    vpred = np.zeros_like(vel)
    upred = np.zeros(n) if u is not None else None
    lib = oracle().lib
    nul = ctypes.cast(None, _P)
    lib.orc_kdk(n, which, ctypes.c_double(dt), int(periodic), ctypes.c_double(L),
                _d(pos), _d(vel), _d(acc), ngas,
                _d(u) if u is not None else nul,
                _d(udot) if udot is not None else nul,
                _d(vpred), _d(upred) if upred is not None else nul)
    return vpred, upred
