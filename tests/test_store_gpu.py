"""GPU tests of the particle-store entry points (tsph_store_*) on a store
laid out exactly as the reference's PARTICLE (tests/golden/
particle_layout.json, the layout of the reference build the fixtures came
from; tests/test_pkd_binding.py pins the fixture to that build and the
reference-side binding that calls these entry points to the reference).

The store is permuted against the caller order, as the reference's tree
build leaves its particle store, and is used registered (the GPU reads and
writes it in place) and unregistered (block copy in, host write-back).
Bar: the results written into the store equal, bit for bit, those of the
plain SoA entry points on the same particles, combined with what the store
held as the reference combines them (a[], fPot += ; dtGrav max; dtNew
min); fields outside the ones named stay untouched; inactive particles
keep their values.  Against the reference's golden outputs: the gravity
and SPH bars of the other GPU tests.
"""
import json
import os

import numpy as np
import pytest

import gasoline_gb300 as g
from golden_io import grav_params_of, load, rel_err, sph_params_of

pytestmark = pytest.mark.gpu

LAYOUT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "particle_layout.json")))
FIELDS3 = ("r", "v", "vPred", "a", "curlv")
FIELDS1 = ("fMass", "fSoft", "u", "uPred", "fPot", "dtGrav", "fBall2", "fDensity", "divv", "dvds",
           "BalsaraSwitch", "diff", "PoverRho2", "c", "uDotPdV", "uDotAV", "mumax", "dtNew")


def particle_dtype():
    names, formats, offsets = [], [], []
    for k in FIELDS3:
        names.append(k); formats.append(("<f8", (3,))); offsets.append(LAYOUT[k])
    for k in FIELDS1:
        names.append(k); formats.append("<f8"); offsets.append(LAYOUT[k])
    for k in ("iOrder", "iActive"):
        names.append(k); formats.append("<u4" if k == "iActive" else "<i4"); offsets.append(LAYOUT[k])
    return np.dtype({"names": names, "formats": formats, "offsets": offsets,
                     "itemsize": LAYOUT["stride"]})


def make_store(pos, mass, soft, rng, vel=None, u=None):
    """A PARTICLE-layout store holding the particles in a shuffled order:
    store entry order[i] is caller particle i.  Every byte starts as
    garbage so untouched fields can be checked."""
    n = len(mass)
    order = rng.permutation(n).astype(np.int32)
    raw = np.frombuffer(rng.bytes(n * LAYOUT["stride"]), dtype=np.uint8).copy()
    st = raw.view(particle_dtype())
    for k in FIELDS1 + FIELDS3:   # finite garbage in every double field
        st[k] = rng.uniform(-1.0, 1.0, st[k].shape)
    st["r"][order] = pos
    st["fMass"][order] = mass
    st["fSoft"][order] = soft
    st["iOrder"][order] = np.arange(n)
    st["iActive"] = LAYOUT["activeBit"] | (LAYOUT["gasBit"] if u is not None else 0)
    if vel is not None:
        st["v"][order] = vel
        st["vPred"][order] = vel
    if u is not None:
        st["u"][order] = u
        st["uPred"][order] = u
    return st, order


LAY = g.store_layout(LAYOUT)


@pytest.fixture
def ctx():
    """A context of its own: a store load sets the active rung from the
    store's activity words."""
    c = g.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("registered", [True, False])
def test_store_gravity_equals_soa_path(ctx, registered):
    d = load("grav_plummer_2k")
    gp = grav_params_of(d, g)
    rng = np.random.default_rng(51)
    n = len(d["mass"])
    st, order = make_store(d["pos"], d["mass"], d["soft"], rng)
    inactive = rng.random(n) < 0.25
    st["iActive"][order[inactive]] = 0
    before = st.copy()
    before_raw = st.view(np.uint8).copy()   # every byte, gaps between fields included
    # the SoA path on the same particles, all active: the reference's bar
    ctx.set_particles(d["pos"], d["mass"], d["soft"])
    out_all = ctx.grav_all(gp)
    assert np.percentile(rel_err(ctx.get_gravity()["acc"], d["acc"]), 99) < 1e-9
    # and with the same particles active (each bucket walks with the box of
    # its active particles, as pkdGravAll does)
    ctx.set_rungs(np.where(inactive, 0, 1).astype(np.int32))
    ctx.set_active_rung(1)
    out_soa = ctx.grav_all(gp)
    soa = ctx.get_gravity()
    if registered:
        ctx.store_register(st)
    try:
        ctx.store_load(st, LAY, order)
        out = ctx.grav_all(gp)
        ctx.store_put_gravity(st, LAY, order)
    finally:
        if registered:
            ctx.store_unregister(st)
    act = ~inactive
    e = order[act]
    # the counters sum over the active particles only
    assert out == out_soa and out["nActive"] == act.sum() < out_all["nActive"]
    np.testing.assert_array_equal(st["a"][e], before["a"][e] + soa["acc"][act])
    np.testing.assert_array_equal(st["fPot"][e], before["fPot"][e] + soa["pot"][act])
    np.testing.assert_array_equal(st["dtGrav"][e], np.maximum(before["dtGrav"][e], soa["dtGrav"][act]))
    # inactive particles and every other byte untouched
    ei = order[inactive]
    for k in ("a", "fPot", "dtGrav"):
        np.testing.assert_array_equal(st[k][ei], before[k][ei])
    mask = np.ones(LAYOUT["stride"], dtype=bool)
    for k, w in (("a", 24), ("fPot", 8), ("dtGrav", 8)):
        mask[LAYOUT[k]:LAYOUT[k] + w] = False
    rawa = st.view(np.uint8).reshape(n, -1)
    rawb = before_raw.reshape(n, -1)
    diff = np.nonzero((rawa != rawb).any(axis=0) & mask)[0]
    assert diff.size == 0, f"bytes changed at offsets {diff.tolist()[:16]}"


def test_store_reload_after_permutation_keeps_results(ctx):
    """A second load of the same store after the reference permuted it (a
    new order, the same particles) is an update: results are unchanged."""
    d = load("grav_plummer_2k")
    gp = grav_params_of(d, g)
    rng = np.random.default_rng(52)
    st, order = make_store(d["pos"], d["mass"], d["soft"], rng)
    ctx.store_register(st)
    try:
        st["a"] = 0.0
        ctx.store_load(st, LAY, order)
        ctx.grav_all(gp)
        ctx.store_put_gravity(st, LAY, order)
        a1 = st["a"][order].copy()
        perm = rng.permutation(len(st))         # the store reshuffled in place
        st2 = st[perm].copy()
        st[:] = st2
        order2 = np.argsort(perm)[order].astype(np.int32)
        st["a"] = 0.0
        ctx.store_load(st, LAY, order2)
        ctx.grav_all(gp)
        ctx.store_put_gravity(st, LAY, order2)
        np.testing.assert_array_equal(st["a"][order2], a1)
    finally:
        ctx.store_unregister(st)


@pytest.mark.parametrize("registered", [True, False])
def test_store_sph_equals_soa_path(ctx, registered):
    d = load("sph_sphere_2k")
    sp = sph_params_of(d, g)
    rng = np.random.default_rng(53)
    n = len(d["mass"])
    ctx.set_particles(d["pos"], d["mass"], d["soft"])
    ctx.set_velocities(d["vel"], ngas=n, u=d["u"])
    ctx.smooth(g.SMX_DENDVDX, sp)
    ctx.smooth(g.SMX_SPHPRESSURETERMS, sp)
    soa = ctx.get_sph()
    st, order = make_store(d["pos"], d["mass"], d["soft"], rng, vel=d["vel"], u=d["u"])
    st["dtNew"] = np.finfo(np.float32).max   # as initSphPressureTermsParticle leaves it
    before = st.copy()
    if registered:
        ctx.store_register(st)
    try:
        ctx.store_load(st, LAY, order, ngas=n)
        ctx.smooth(g.SMX_DENDVDX, sp)
        ctx.store_put_sph(g.SMX_DENDVDX, st, LAY, order)
        ctx.smooth(g.SMX_SPHPRESSURETERMS, sp)
        ctx.store_put_sph(g.SMX_SPHPRESSURETERMS, st, LAY, order)
    finally:
        if registered:
            ctx.store_unregister(st)
    for k in ("fBall2", "fDensity", "divv", "dvds", "BalsaraSwitch", "diff", "PoverRho2", "c",
              "uDotPdV", "uDotAV", "mumax", "dtNew"):
        np.testing.assert_array_equal(st[k][order], soa[k], err_msg=k)
    np.testing.assert_array_equal(st["curlv"][order],
                                  np.stack([soa["curlv_x"], soa["curlv_y"], soa["curlv_z"]], 1))
    np.testing.assert_array_equal(st["a"][order], before["a"][order] +
                                  np.stack([soa["ax"], soa["ay"], soa["az"]], 1))
    # and the SoA path itself is the reference's (golden) result
    np.testing.assert_array_equal(soa["fBall2"], d["out"][:, 0])
