"""GPU tests of the TSC frame (tsph_render_tsc) against the reference's own
dfRenderParticles (golden frames from tests/golden/make_golden.py).

Bar: every pixel within 1e-5 of the frame's brightest (the reference adds
float contributions in particle order, this path in FP64 in any order);
identical frames run to run.
"""
import numpy as np
import pytest

import gasoline_gb300 as g
from golden_io import load, render_frames

pytestmark = pytest.mark.gpu


def test_render_tsc_vs_reference(ctx):
    d = load("render_tsc")
    n, ngas, nstar = len(d["mass"]), int(d["ngas"]), int(d["nstar"])
    ctx.set_particles(d["pos"], d["mass"], d["soft"])
    ctx.set_velocities(np.zeros((n, 3)), ngas=ngas, u=d["u"])
    ctx.smooth(g.SMX_DENDVDX, g.sph_params(nSmooth=32))
    for k, rp in enumerate(render_frames()):
        img = ctx.render_tsc(rp, nstar=nstar)
        ref = d[f"img{k}"]
        assert img.shape == ref.shape
        scale = float(ref.max())
        assert scale > 0
        assert np.max(np.abs(img - ref)) <= 1e-5 * scale, k
        assert np.array_equal(img > 0, ref > 0), k
        assert np.array_equal(img, ctx.render_tsc(rp, nstar=nstar)), k
