"""Loading helpers for the golden fixtures in tests/golden/."""
import os

import numpy as np

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GRAV_CASES = ["grav_plummer_2k", "grav_box_8", "grav_cube_soft",
              # octopole (iOrder 3) and hexadecapole (iOrder 4, the reference's default) cells
              "grav_plummer_2k_o3", "grav_plummer_2k_o4", "grav_box_8_o4"]


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def grav_params_of(d, mod):
    p = d["params"]
    return mod.grav_params(nBucket=int(p[0]), iOrder=int(p[1]),
                           periodic=bool(p[2]), ewald=bool(p[3]),
                           iEwOrder=int(p[4]), nReps=int(p[5]), theta=p[6],
                           L=p[7], fEwCut=p[8], fEwhCut=p[9])


def sph_params_of(d, mod, **kw):
    p = d["params"]
    args = dict(nSmooth=int(p[0]), periodic=bool(p[1]), L=p[2], alpha=p[3],
                beta=p[4], gamma=p[5], dEtaCourant=p[6])
    args.update(kw)
    return mod.sph_params(**args)


def rel_err(a, b):
    """Per-particle |a-b|/|b| for vectors (n,3) or scalars (n,)."""
    a = np.asarray(a); b = np.asarray(b)
    if a.ndim == 2:
        num = np.linalg.norm(a - b, axis=1)
        den = np.linalg.norm(b, axis=1)
    else:
        num = np.abs(a - b)
        den = np.abs(b)
    return num / np.maximum(den, 1e-300)


def render_frames():
    """The frame parameters of the rendering fixture (gasoline_gb300's
    render_params): orthographic with log density colours and mass
    weighting, and perspective."""
    import gasoline_gb300 as g
    return [g.render_params(nx=160, ny=120, width=3.0, gas_levels=(-1.0, 1.0),
                            gas_col=((1.0, 0.2, 0.1), (0.2, 0.4, 1.0)), log_interp=1, mass_weight=1,
                            soft_mul=(1.0, 2.0, 4.0)),
            g.render_params(nx=160, ny=120, width=3.0 / 4.0, perspective=True, zEye=4.0,
                            zClip=(0.5, 100.0), gas_levels=(0.5, 5.0),
                            gas_col=((1.0, 0.0, 0.0), (0.0, 1.0, 0.0)))]


# Periodic SPH against the reference (sph_box_16).  The reference re-centres
# a neighbour queue it inherits from the previous particle (smRecentrePQ,
# smooth.c:1307-1335) by forming a kept neighbour's offset as (x - r_j) + ax,
# ax being an earlier (x' +- L) - x'; a fresh search forms (x +- L) - r_j.
# Without periodic images ax = 0 and the two agree bit for bit; through a
# face of the box they round differently, so the reference's fBall2 (the
# k-th key of its queue) carries the rounding of its processing order.  The
# neighbour SETS are unaffected and must be identical; fBall2 agrees to a
# few ulps (15 at most on this fixture).  Where the reference's fBall2 sits
# below the k-th neighbour's fresh distance, its pressure gather (which
# recomputes distances) leaves that edge neighbour out, as its cpStart
# gather can without images: the pair has zero kernel weight, so only the
# Courant and viscosity bounds dtNew and mumax of its two particles move,
# dtNew only down and mumax only up on this side.
PSPH_FBALL2_REL = 1e-14
PSPH_DTNEW_REL = 1e-13


def check_periodic_sph_vs_golden(r, d, fields, field_rel, hashes):
    """r: fields of an evaluation of the sph_box_16 input (oracle or CUDA),
    d: the fixture, hashes: the evaluation's neighbour-set hashes."""
    import numpy as np
    assert np.array_equal(hashes, d["knn_hash"]), int((hashes != d["knn_hash"]).sum())
    assert (d["knn_count"] == 32).all()
    fb = d["out"][:, 0]
    assert np.max(np.abs(r["fBall2"] - fb) / fb) <= PSPH_FBALL2_REL
    for k, name in enumerate(fields):
        if name == "fBall2":
            continue
        ref = d["out"][:, k]
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(r[name] - ref)) <= field_rel * scale, name
    rel = np.abs(r["dtNew"] - d["dtNew"]) / d["dtNew"]
    edge = rel > PSPH_DTNEW_REL
    assert (r["dtNew"][edge] < d["dtNew"][edge]).all()
    assert edge.sum() <= 0.005 * len(fb), int(edge.sum())
    murel = np.abs(r["mumax"] - d["mumax"]) / np.maximum(np.abs(d["mumax"]), 1e-300)
    mu = murel > PSPH_DTNEW_REL
    assert (r["mumax"][mu] >= d["mumax"][mu]).all()
    assert mu.sum() <= 0.005 * len(fb), int(mu.sum())
    return int(edge.sum())
