"""GPU tests of adaptive timesteps (rungs): force passes over an active
subset and whole msrTopStepKDK runs, against the reference's own code
(golden vectors written by tests/golden/make_golden.py through the
reference build).

Bars: the active set, the per-bucket interaction-list sums and every
rung bit-exact; FP64 forces on the active particles within the same 1e-9
rms of the reference as the all-active path (its v_sqrt1 is an
approximate 1/sqrt); SPH rates within 1e-10 of scale; the timestep dt
within 1e-12, and dtNew and mumax too except for the few particles whose
extreme comes from a ball's boundary pair (see test_active_sph); a
three-step run with up to four rungs within 1e-8 of scale in positions,
velocities and energies.
"""
import numpy as np
import pytest

import gasoline_gb300 as g
from golden_io import load, rel_err

pytestmark = pytest.mark.gpu


def _scale_err(a, b):
    s = np.max(np.abs(b))
    return np.max(np.abs(a - b)) / s if s > 0 else np.max(np.abs(a))


@pytest.mark.parametrize("grp", [0, 32])
@pytest.mark.parametrize("prec,tol", [(g.FP64, 1e-9), (g.FP32, 1e-4)])
def test_active_gravity_vs_reference(ctx, prec, tol, grp):
    """Also with walk groups of 32 particles, whose shared walk uses the
    group's whole box while each bucket walks with its active box."""
    d = load("ms_active_grav")
    act = d["rung"] >= int(d["iRung"])
    ctx.set_particles(d["pos"], d["mass"], d["soft"])
    ctx.set_rungs(d["rung"])
    ctx.set_active_rung(int(d["iRung"]))
    ctx.set_tuning(walkGroup=grp)
    try:
        out = ctx.grav_all(g.grav_params(periodic=False, precision=prec))
    finally:
        ctx.set_active_rung(0)
        ctx.set_tuning()
    r = ctx.get_gravity()
    e = rel_err(r["acc"][act], d["acc"][act])
    if prec == g.FP64:
        assert np.sqrt(np.mean(e ** 2)) <= tol
    else:
        assert np.percentile(e, 99) <= tol
    # inactive particles keep what they had (zero after loading)
    assert np.all(r["acc"][~act] == 0.0) and np.all(r["pot"][~act] == 0.0)
    c = d["counters"]
    assert out["nActive"] == int(c[0]) == int(act.sum())
    assert out["dPartSum"] == c[1] and out["dCellSum"] == c[2] and out["dSoftSum"] == c[3]


def test_active_gravity_all_rungs_equals_plain(ctx):
    """An active rung every particle is on gives the plain evaluation."""
    d = load("ms_active_grav")
    gp = g.grav_params(periodic=False, precision=g.FP32)
    ctx.set_particles(d["pos"], d["mass"], d["soft"])
    ctx.grav_all(gp)
    a = ctx.get_gravity()
    ctx.set_particles(d["pos"], d["mass"], d["soft"])
    ctx.set_rungs(d["rung"])
    ctx.set_active_rung(0)
    ctx.grav_all(gp)
    b = ctx.get_gravity()
    for k in ("acc", "pot", "dtGrav"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("iRung", [1, 2])
def test_active_sph_vs_reference(ctx, iRung):
    """Two thirds of the gas active (a density pass over all gas) and one
    third (a pass over the particles the active ones need only)."""
    d = load("ms_active_sph")
    d = dict(d, **{k[:-3]: v for k, v in d.items() if k.endswith(f"_r{iRung}")})
    act = d["rung"] >= iRung
    n = len(d["mass"])
    ctx.set_particles(d["pos"], d["mass"], d["soft"])
    ctx.set_velocities(d["vel"], ngas=n, u=d["u"])
    ctx.set_rungs(d["rung"])
    ctx.set_active_rung(iRung)
    sp = g.sph_params(nSmooth=32)
    try:
        ctx.smooth(g.SMX_DENDVDX, sp)
        ctx.smooth(g.SMX_SPHPRESSURETERMS, sp)
    finally:
        ctx.set_active_rung(0)
    r = ctx.get_sph()
    rr = ctx.get_rungs()
    # particles the pass did not need keep their state; the rest match
    done = np.abs(r["fDensity"] - d["fDensity"]) <= 1e-10 * np.max(d["fDensity"])
    assert np.all(done[act])
    if iRung == 1:
        assert np.all(done)
    for k, j in (("ax", 0), ("ay", 1), ("az", 2)):
        assert _scale_err(r[k][act], d["acc"][act, j]) <= 1e-10, k
    for k in ("uDotPdV", "uDotAV"):
        assert _scale_err(r[k][act], d[k][act]) <= 1e-10, k
    # the timestep dt of every gas particle the pass computed drops to its
    # Courant time (a particle it did not need takes its last ball's)
    e = np.abs(rr["dt"] - d["dt"]) / d["dt"]
    assert e[done].max() <= 1e-12
    # dtNew and mumax change for every particle with an active partner.
    # The reference's pressure pass gathers each ball from the cell its kNN
    # search ended in (smResmoothParticle's cpStart, smooth.c:1120-1131),
    # which can leave out the k-th neighbour, a pair of zero kernel weight:
    # such a pair moves no force or energy but its Courant and viscosity
    # terms can set dtNew and mumax.  This path gathers the whole ball, so
    # where the two differ it can only have the lower dtNew or the higher
    # mumax, and that for a few particles.
    for name, got, sign in (("dtNew", rr["dtNew"], -1), ("mumax", rr["mumax"], 1)):
        ref = d[name]
        big = ref > 1e30
        assert np.array_equal(big, got > 1e30), name
        e = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
        e[big] = 0.0
        off = e > 1e-12
        assert off.sum() <= max(2, n // 500), (name, off.sum())
        assert np.all(sign * (got[off] - ref[off]) > 0), name
    assert np.array_equal(rr["dtNew"], r["dtNew"])


def _run(ctx, d, prec=g.FP64, sph_prec=g.FP64):
    n = len(d["mass"])
    ngas = int(d["ngas"])
    ctx.set_particles(d["pos0"], d["mass"], d["soft"])
    ctx.set_velocities(d["vel0"], ngas=ngas, u=d["u0"])
    gp = g.grav_params(periodic=False, precision=prec)
    sp = g.sph_params(nSmooth=32, precision=sph_prec)
    ctx.grav_all(gp)
    ctx.smooth(g.SMX_DENDVDX, sp)
    ctx.smooth(g.SMX_SPHPRESSURETERMS, sp)
    nSteps, iMaxRung = (int(x) for x in d["steps"])
    st = g.step_params(iMaxRung=iMaxRung)
    dt = float(d["dDelta"])
    outs = [ctx.top_step_kdk(k * dt, dt, gp, sp, st) for k in range(nSteps)]
    pos, vel, u = ctx.get_state()
    return outs, pos, vel, u, ctx.get_rungs(), n, ngas


def test_multistep_run_vs_reference(ctx):
    d = load("ms_run")
    outs, pos, vel, u, rr, n, ngas = _run(ctx, d)
    assert [o["iCurrMaxRung"] for o in outs] == list(d["maxRung"])
    assert np.array_equal(rr["rung"], d["rung"])
    assert 1 + sum(o["nForcePasses"] for o in outs) == int(d["counts"][0])
    assert n + sum(o["nActiveSum"] for o in outs) == int(d["counts"][1])
    assert _scale_err(pos, d["pos"]) <= 1e-8
    assert _scale_err(vel, d["vel"]) <= 1e-8
    assert _scale_err(u, d["u"][:ngas]) <= 1e-8
    e = np.abs(rr["dt"] - d["dt"]) / np.abs(d["dt"])
    assert e.max() <= 1e-8


def test_multistep_fp32_keeps_rungs(ctx):
    """The FP32 gravity and SPH paths step the same run; their rungs agree
    with the reference's for all but a few particles near a rung boundary."""
    d = load("ms_run")
    outs, pos, vel, u, rr, n, ngas = _run(ctx, d, g.FP32, g.FP32)
    assert np.mean(rr["rung"] == d["rung"]) >= 0.99
    assert _scale_err(pos, d["pos"]) <= 1e-3


def test_single_rung_top_step_equals_step(ctx):
    """With one rung a top step is the plain kick-drift-kick step."""
    d = load("ms_run")
    ngas = int(d["ngas"])
    gp = g.grav_params(periodic=False)
    sp = g.sph_params(nSmooth=32)
    res = []
    for multi in (False, True):
        ctx.set_particles(d["pos0"], d["mass"], d["soft"])
        ctx.set_velocities(d["vel0"], ngas=ngas, u=d["u0"])
        ctx.grav_all(gp)
        ctx.smooth(g.SMX_DENDVDX, sp)
        ctx.smooth(g.SMX_SPHPRESSURETERMS, sp)
        for k in range(2):
            if multi:
                out = ctx.top_step_kdk(0.0, 0.01, gp, sp, g.step_params(iMaxRung=1))
                assert out["iCurrMaxRung"] == 0 and out["nForcePasses"] == 1
            else:
                ctx.step(0.01, gp, sp)
                ctx.step_status()
        res.append(ctx.get_state())
    for k in range(3):
        assert np.array_equal(res[0][k], res[1][k]), k
