"""Loading helpers for the golden fixtures in tests/golden/."""
import os

import numpy as np

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GRAV_CASES = ["grav_plummer_2k", "grav_box_8", "grav_cube_soft"]


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
