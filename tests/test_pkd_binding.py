"""CPU tests of the reference-side binding (gasoline_gb300/pkd/tsph_pkd.c).

The binding is compiled against the reference's own pkd.h, smooth.h and
smoothfcn.h, as an integrator would compile it, and the reference harness
is built a second time with its pkdBuildBinary / pkdGravAll / smSmooth /
smReSmooth calls replaced by the binding's (oracle/_ref/libgasadapt.so).
libtsph is stood in for by a CPU implementation of the same calls whose
arithmetic is the oracle's, which restates the reference bit for bit; so
the harness run through the binding must reproduce the reference's golden
outputs exactly.  What this pins is the binding itself: the PARTICLE
layout it reads and writes (offsetof in the reference's own headers), the
caller-index mapping through iOrder after the reference's tree build has
permuted the store, pkdGravAll's accumulation into a[], fPot and dtGrav,
the SMF parameters it hands over, and the counters it returns.  The GPU
side of the same calls (the store entry points on a PARTICLE-layout
store) is tested in tests/test_store_gpu.py.
"""
import numpy as np
import pytest

import oracle
from golden_io import grav_params_of, load, sph_params_of

pytestmark = pytest.mark.skipif(oracle.adapter() is None,
                                reason="reference sources not built here")


@pytest.mark.parametrize("name", ["grav_plummer_2k", "grav_cube_soft"])
def test_binding_gravity_reproduces_reference(name):
    d = load(name)
    gp = grav_params_of(d, oracle)
    r = oracle.adapter().grav(d["pos"], d["mass"], d["soft"], gp)
    assert np.array_equal(r["acc"], d["acc"])
    assert np.array_equal(r["pot"], d["pot"])
    assert np.array_equal(r["dtGrav"], d["dtGrav"])
    assert np.array_equal(r["counters"], d["counters"])


def test_binding_sph_reproduces_reference():
    d = load("sph_sphere_2k")
    sp = sph_params_of(d, oracle)
    r = oracle.adapter().sph(d["pos"], d["vel"], d["mass"], d["soft"], d["u"], sp)
    for k, name in enumerate(oracle.SPH_FIELDS):
        ref = d["out"][:, k]
        if name in ("fBall2", "c"):
            assert np.array_equal(r[name], ref), name
        else:
            assert np.max(np.abs(r[name] - ref)) <= 1e-12 * np.max(np.abs(ref)), name
    assert np.array_equal(r["dtNew"], d["dtNew"])
    assert np.array_equal(r["mumax"], d["mumax"])


def test_particle_layout_fixture_matches_the_reference_build():
    """The PARTICLE layout the GPU store tests use (tests/golden/
    particle_layout.json, where the reference's headers are absent) is the
    layout of the reference build here."""
    import json
    import os
    fx = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "particle_layout.json")))
    assert fx == oracle.reference_particle_layout()
