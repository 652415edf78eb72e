"""Tipsy snapshot format restated in numpy (test infrastructure only).

The CPU checker of the library's snapshot reader and writer.  It restates
the reference's file layout and conversions:
  tipsydefs.h:9-45       record layouts (gas 12, dark 9, star 11 floats)
  master.c:3563-3575     header order (time, nbodies, ndim, nsph, ndark,
                         nstar, pad) -- xdrHeader
  pkd.c:253-285          record offsets (pkdSeek)
  pkd.c:297-686          reading (pkdReadTipsy): float -> double,
                         v = dvFac*vel, u = uPred = dTuFac*temp (gas)
  pkd.c:1628-1798        writing (pkdWriteTipsy): (float)(dvFac*v),
                         (float)(duTFac*u) for the adiabatic gas model
The standard form is big-endian (XDR); the native form is host order.

Arrays use the layout of the reference harness in ref_harness.c:
pos, vel (n, 3) float64 and f (n, 9) float64 with columns
mass, soft, u, rho, metals, tform, phi, 0, 0 -- as the reference's
PARTICLE holds them after pkdReadTipsy (tform of non-star particles is the
reader's initial 1e37, pkd.c:371).
"""
import numpy as np

GAS = ("mass", "x", "y", "z", "vx", "vy", "vz", "rho", "temp", "eps", "metals", "phi")
DARK = ("mass", "x", "y", "z", "vx", "vy", "vz", "eps", "phi")
STAR = ("mass", "x", "y", "z", "vx", "vy", "vz", "metals", "tform", "eps", "phi")
HEADER_BYTES = 32


def _rec(fields, standard):
    return np.dtype([(f, ">f4" if standard else "=f4") for f in fields])


def _hdr(standard):
    if standard:
        return np.dtype([("time", ">f8"), ("nbodies", ">i4"), ("ndim", ">i4"), ("nsph", ">i4"),
                         ("ndark", ">i4"), ("nstar", ">i4"), ("pad", ">i4")])
    return np.dtype([("time", "=f8"), ("nbodies", "=i4"), ("ndim", "=i4"), ("nsph", "=i4"),
                     ("ndark", "=i4"), ("nstar", "=i4"), ("pad", "V4")])


def read_header(path, standard=True):
    h = np.fromfile(path, dtype=_hdr(standard), count=1)[0]
    return {k: (float(h[k]) if k == "time" else int(h[k]))
            for k in ("time", "nbodies", "ndim", "nsph", "ndark", "nstar")}


def read(path, standard=True, dvFac=1.0, dTuFac=1.0):
    """Returns (header, pos, vel, f) as the reference's reader leaves them."""
    h = read_header(path, standard)
    ng, nd, ns = h["nsph"], h["ndark"], h["nstar"]
    n = ng + nd + ns
    raw = np.fromfile(path, dtype=np.uint8)
    off = HEADER_BYTES
    parts = []
    for cnt, fields in ((ng, GAS), (nd, DARK), (ns, STAR)):
        dt = _rec(fields, standard)
        parts.append(np.frombuffer(raw[off:off + cnt * dt.itemsize].tobytes(), dtype=dt, count=cnt))
        off += cnt * dt.itemsize
    pos = np.zeros((n, 3))
    vel = np.zeros((n, 3))
    f = np.zeros((n, 9))
    f[:, 5] = 1e37
    lo = 0
    for kind, rec in enumerate(parts):
        hi = lo + len(rec)
        d = lambda k: rec[k].astype(np.float64)   # noqa: E731
        pos[lo:hi] = np.stack([d("x"), d("y"), d("z")], axis=1)
        vel[lo:hi] = dvFac * np.stack([d("vx"), d("vy"), d("vz")], axis=1)
        f[lo:hi, 0] = d("mass")
        f[lo:hi, 1] = d("eps")
        f[lo:hi, 6] = d("phi")
        if kind == 0:
            f[lo:hi, 2] = dTuFac * d("temp")
            f[lo:hi, 3] = d("rho")
            f[lo:hi, 4] = d("metals")
        elif kind == 2:
            f[lo:hi, 4] = d("metals")
            f[lo:hi, 5] = d("tform")
        lo = hi
    return h, pos, vel, f


def write(path, time, ngas, ndark, nstar, pos, vel, f, standard=True, dvFac=1.0, duTFac=1.0):
    """Writes the file pkdWriteTipsy would write for these particles."""
    n = ngas + ndark + nstar
    h = np.zeros(1, dtype=_hdr(standard))
    h["time"] = time
    h["nbodies"], h["ndim"], h["nsph"], h["ndark"], h["nstar"] = n, 3, ngas, ndark, nstar
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    vel = np.asarray(vel, dtype=np.float64).reshape(-1, 3)
    f = np.asarray(f, dtype=np.float64).reshape(-1, 9)
    out = [h.tobytes()]
    lo = 0
    for kind, (cnt, fields) in enumerate(((ngas, GAS), (ndark, DARK), (nstar, STAR))):
        hi = lo + cnt
        rec = np.zeros(cnt, dtype=_rec(fields, standard))
        rec["mass"] = f[lo:hi, 0]
        for j, k in enumerate("xyz"):
            rec[k] = pos[lo:hi, j]
            rec["v" + k] = dvFac * vel[lo:hi, j]
        rec["eps"] = f[lo:hi, 1]
        rec["phi"] = f[lo:hi, 6]
        if kind == 0:
            rec["rho"] = f[lo:hi, 3]
            rec["temp"] = duTFac * f[lo:hi, 2]
            rec["metals"] = f[lo:hi, 4]
        elif kind == 2:
            rec["metals"] = f[lo:hi, 4]
            rec["tform"] = f[lo:hi, 5]
        out.append(rec.tobytes())
        lo = hi
    with open(path, "wb") as fh:
        for b in out:
            fh.write(b)
