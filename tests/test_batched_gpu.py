"""GPU tests of independent systems in one context (tsph_set_systems).

Each system of the batch gets its own gravity tree and gas tree inside one
launch of every kernel.  The bar: every system's forces, SPH rates and
neighbour sets are bit-identical to those of the same system loaded alone
(the batch changes the launch, never a result), and the batch's FP32
forces stay within the tree method's error of the FP64 direct sum.
"""
import numpy as np
import pytest

import gasoline_gb300 as g
import oracle

pytestmark = pytest.mark.gpu


def _batch(k=6, seed=11, nmin=600, nmax=6000):
    systems = g.ics.batched_systems(nsys=k, seed=seed, nmin=nmin, nmax=nmax, gas_frac=0.2)
    return systems, g.ics.pack_systems(systems)


def _hash(idx):
    """The library's order-free neighbour-set hash: the wrapping sum of a
    64-bit mix of (caller index + 1) over the set."""
    with np.errstate(over="ignore"):
        h = np.asarray(idx, dtype=np.uint64) + np.uint64(1)
        h = h * np.uint64(0x9E3779B97F4A7C15)
        h ^= h >> np.uint64(29)
        h = h * np.uint64(0xBF58476D1CE4E5B9)
        h ^= h >> np.uint64(32)
        return np.uint64(np.sum(h, dtype=np.uint64))


@pytest.fixture(scope="module")
def pair():
    a, b = g.Context(0), g.Context(0)
    yield a, b
    a.close()
    b.close()


@pytest.mark.parametrize("grp", [0, 64])
@pytest.mark.parametrize("prec", [g.FP32, g.FP64])
def test_batch_gravity_equals_each_system_alone(pair, prec, grp):
    """Also with walk groups of 64 particles: a group never spans two
    systems, so each system's groups are those it has alone."""
    c, c1 = pair
    systems, (pos, vel, m, soft, ngas, u, so, index) = _batch()
    c.set_tuning(walkGroup=grp)
    c1.set_tuning(walkGroup=grp)
    try:
        c.set_particles(pos, m, soft)
        c.set_velocities(vel, ngas, u)
        c.set_systems(so)
        gp = g.grav_params(periodic=False, precision=prec)
        out = c.grav_all(gp)
        r = c.get_gravity()
        part = cell = 0.0
        for s, d in enumerate(systems):
            c1.set_particles(d["pos"], d["mass"], d["soft"])
            o1 = c1.grav_all(gp)
            r1 = c1.get_gravity()
            for k in ("acc", "pot", "dtGrav"):
                assert np.array_equal(r[k][index[s]], r1[k]), (s, k)
            part += o1["dPartSum"]
            cell += o1["dCellSum"]
        assert out["dPartSum"] == part
        assert out["dCellSum"] == cell
        assert out["nActive"] == len(m)
    finally:
        c.set_tuning()
        c1.set_tuning()


def test_batch_sph_equals_each_system_alone(pair):
    c, c1 = pair
    systems, (pos, vel, m, soft, ngas, u, so, index) = _batch(seed=12)
    sp = g.sph_params(nSmooth=32)
    c.set_particles(pos, m, soft)
    c.set_velocities(vel, ngas, u)
    c.set_systems(so)
    c.smooth(g.SMX_DENDVDX, sp)
    c.smooth(g.SMX_SPHPRESSURETERMS, sp)
    s_all = c.get_sph()
    h_all = c.get_neighbour_hash()          # (count, hash) per gas particle
    nsph = 0
    for s, d in enumerate(systems):
        if d["ngas"] == 0:
            continue
        nsph += 1
        c1.set_particles(d["pos"], d["mass"], d["soft"])
        c1.set_velocities(d["vel"], d["ngas"], np.full(d["ngas"], 0.05))
        c1.smooth(g.SMX_DENDVDX, sp)
        c1.smooth(g.SMX_SPHPRESSURETERMS, sp)
        s1 = c1.get_sph()
        h1 = c1.get_neighbour_hash()
        gi = index[s][: d["ngas"]]
        for k in ("fBall2", "fDensity", "divv", "PoverRho2", "ax", "ay", "az", "uDotPdV",
                  "uDotAV", "dtNew"):
            assert np.array_equal(s_all[k][gi], s1[k]), (s, k)
        # neighbour counts equal; the hashes key on caller indices, which
        # differ between the batch and the lone system, so both are checked
        # against the set {j : d2 <= fBall2} recomputed here
        assert np.array_equal(h_all[0][gi], h1[0]), s
        gp_ = d["pos"][: d["ngas"]]
        for i in range(0, d["ngas"], 97):
            d2 = np.sum((gp_ - gp_[i]) ** 2, axis=1)
            nb = np.nonzero(d2 <= s1["fBall2"][i])[0]
            assert len(nb) == h1[0][i]
            assert _hash(nb) == h1[1][i]
            assert _hash(gi[nb]) == h_all[1][gi[i]]
    assert nsph >= 2


def test_batch_fp32_vs_direct_sum(pair):
    """Per-system error of the FP32 batched forces against an FP64 direct
    sum on a sample of each system's particles."""
    c, _ = pair
    systems, (pos, vel, m, soft, ngas, u, so, index) = _batch(k=8, seed=13, nmax=8000)
    c.set_particles(pos, m, soft)
    c.set_systems(so)
    c.grav_all(g.grav_params(periodic=False, precision=g.FP32))
    acc = c.get_gravity()["acc"]
    worst = 0.0
    for s, d in enumerate(systems):
        q = np.arange(0, len(d["mass"]), 37)
        ad, _ = oracle.direct(d["pos"], d["mass"], d["soft"], q)
        e = np.linalg.norm(acc[index[s][q]] - ad, axis=1) / np.linalg.norm(ad, axis=1)
        worst = max(worst, float(np.sqrt(np.mean(e ** 2))))
    # theta = 0.7 with quadrupoles: the tree method's own error is ~5e-3 rms
    assert worst < 1.5e-2, worst


def test_batch_rejects_periodic_and_small_gas_systems(pair):
    c, _ = pair
    systems, (pos, vel, m, soft, ngas, u, so, index) = _batch(seed=14)
    c.set_particles(pos, m, soft)
    c.set_velocities(vel, ngas, u)
    c.set_systems(so)
    with pytest.raises(g.TsphError) as e:
        c.grav_all(g.grav_params(periodic=True, L=200.0))
    assert e.value.code == 7
    small = min(d["ngas"] for d in systems if d["ngas"] > 0)
    with pytest.raises(g.TsphError) as e:
        c.smooth(g.SMX_DENDVDX, g.sph_params(nSmooth=small + 1))
    assert e.value.code == 1
    # the context stays usable
    c.grav_all(g.grav_params(periodic=False, precision=g.FP32))


def test_graph_step_equals_direct_steps():
    """Three kick-drift-kick steps replayed from one captured CUDA graph give
    bit-identical states to three directly issued steps."""
    systems, (pos, vel, m, soft, ngas, u, so, index) = _batch(k=5, seed=15)
    gp = g.grav_params(periodic=False, precision=g.FP32)
    sp = g.sph_params(nSmooth=32)
    states = []
    for graph in (False, True):
        c = g.Context(0)
        try:
            c.set_particles(pos, m, soft)
            c.set_velocities(vel, ngas, u)
            c.set_systems(so)
            c.grav_all(gp)
            c.smooth(g.SMX_DENDVDX, sp)
            c.smooth(g.SMX_SPHPRESSURETERMS, sp)
            c.step(1e-3, gp, sp, graph=graph)       # captures in graph mode
            n0 = c.launches()
            for _ in range(2):
                c.step(1e-3, gp, sp, graph=graph)
            c.step_status()
            states.append((c.get_state(), c.launches() - n0))
        finally:
            c.close()
    (sa, la), (sb, lb) = states
    for k in range(3):
        assert np.array_equal(sa[k], sb[k]), k
    # a replay counts the kernels it runs (the captured build's fixed top
    # levels included, some of them empty)
    assert lb > 0 and la > 0


def test_graph_step_with_two_task_sizes():
    """The gravity tree (900k particles) and the gas tree (700k) pick
    different subtree task sizes on a 152-SM GPU; one captured step holds
    both builds and replays bit-identically to direct steps."""
    pg, vg, mg, u = g.ics.gas_sphere(700_000, seed=21)
    pd, vd, md = g.ics.plummer(200_000, seed=22)
    pos = np.concatenate([pg, pd])
    vel = np.concatenate([vg, vd])
    m = np.concatenate([0.2 * mg, 0.8 * md])
    soft = np.full(len(m), 0.01)
    gp = g.grav_params(periodic=False, precision=g.FP32)
    sp = g.sph_params(nSmooth=32)
    states = []
    for graph in (False, True):
        c = g.Context(0)
        try:
            c.set_particles(pos, m, soft)
            c.set_velocities(vel, len(mg), u)
            c.grav_all(gp)                       # the opening kick's forces
            c.smooth(g.SMX_DENDVDX, sp)
            c.smooth(g.SMX_SPHPRESSURETERMS, sp)
            for _ in range(2):
                c.step(1e-4, gp, sp, graph=graph)
            c.step_status()
            states.append(c.get_state())
        finally:
            c.close()
    for k in range(3):
        assert np.array_equal(states[0][k], states[1][k]), k


def _direct_and_graph_states(setup, dt, gp, sp, nsteps=3):
    """Run `nsteps` KDK steps on two fresh contexts prepared by setup(c):
    directly, then as one captured graph replayed; returns both states."""
    states = []
    for graph in (False, True):
        c = g.Context(0)
        try:
            setup(c)
            for _ in range(nsteps):
                c.step(dt, gp, sp, graph=graph)
            c.step_status()
            states.append(c.get_state())
        finally:
            c.close()
    return states


def test_graph_step_recaptures_on_a_tuning_change():
    """A launch shape changed between graph steps is captured anew (the
    knobs are part of the graph): the step after the change runs the
    preparation and the capture besides the replay, the next one replays
    only, and the states equal direct steps with the same change."""
    pos, vel, m = g.ics.plummer(20000, seed=9)
    soft = np.full(len(m), 0.01)
    gp = g.grav_params(periodic=False, precision=g.FP32)

    def run(graph):
        c = g.Context(0)
        try:
            c.set_particles(pos, m, soft)
            c.set_velocities(vel)
            c.grav_all(gp)
            for _ in range(2):
                c.step(1e-3, gp, None, graph=graph)
            c.set_tuning(walkBlocksPerSM=2)
            l0 = c.launches()
            c.step(1e-3, gp, None, graph=graph)
            l1 = c.launches()
            c.step(1e-3, gp, None, graph=graph)
            l2 = c.launches()
            c.step_status()
            return c.get_state(), l1 - l0, l2 - l1
        finally:
            c.close()

    sa, _, _ = run(False)
    sb, first, replay = run(True)
    for k in range(3):
        assert np.array_equal(sa[k], sb[k]), k
    assert first > replay > 0


def test_graph_step_periodic_ewald_equals_direct_steps():
    """A periodic box with Ewald (FP32 gravity, periodic FP32 SPH): the
    Ewald constants are rebuilt on the device from each step's root
    moments, so the step captures; replays equal direct steps bit for bit."""
    pos, vel, m, ngas, u = g.ics.mixed_box(ng=24, seed=31, nclump=8)
    soft = np.full(len(m), 0.2 / 24)
    gp = g.grav_params(periodic=True, L=1.0, precision=g.FP32)
    sp = g.sph_params(nSmooth=32, periodic=True, L=1.0, precision=g.FP32)

    def setup(c):
        c.set_particles(pos, m, soft)
        c.set_velocities(vel, ngas, u)
        c.grav_all(gp)
        c.smooth(g.SMX_DENDVDX, sp)
        c.smooth(g.SMX_SPHPRESSURETERMS, sp)

    sa, sb = _direct_and_graph_states(setup, 2e-3, gp, sp)
    for k in range(3):
        assert np.array_equal(sa[k], sb[k]), k
    # the particles moved and stayed in the box
    assert not np.array_equal(sa[0], pos)
    assert np.all(np.abs(sa[0]) <= 0.5)


def test_graph_step_learned_h_equals_direct_steps():
    """A gas sphere whose kNN is seeded by a trained h-network: the seeding
    (features, prediction) is captured with the step; replays equal direct
    steps bit for bit, and collecting samples under capture is refused."""
    n = 20000
    pos, vel, m, u = g.ics.gas_sphere(n, seed=43)
    soft = np.full(n, 0.01)
    gp = g.grav_params(periodic=False, precision=g.FP32)
    sp = g.sph_params(nSmooth=32, precision=g.FP32)
    sp_l = g.sph_params(nSmooth=32, precision=g.FP32, learned_h=True)
    dt = 0.01

    def setup(c):
        c.set_particles(pos, m, soft)
        c.set_velocities(vel, n, u)
        c.hnet_init(seed=5)
        c.hnet_mode(collect=True)
        c.grav_all(gp)
        c.smooth(g.SMX_DENDVDX, sp)
        c.smooth(g.SMX_SPHPRESSURETERMS, sp)
        for _ in range(3):
            c.step(dt, gp, sp)
        c.hnet_train(steps=200, batch=4096, lr=3e-3)
        c.hnet_mode(collect=False, predict=True, margin=0.08)

    sa, sb = _direct_and_graph_states(setup, dt, gp, sp_l)
    for k in range(3):
        assert np.array_equal(sa[k], sb[k]), k
    c = g.Context(0)
    try:
        c.set_particles(pos, m, soft)
        c.set_velocities(vel, n, u)
        c.hnet_init(seed=5)
        c.hnet_mode(collect=True)
        with pytest.raises(g.TsphError) as e:
            c.step(dt, gp, sp_l, graph=True)
        assert e.value.code == 7
    finally:
        c.close()


def test_graph_step_takes_any_dt():
    """A captured step reads dt from device memory: one graph replays steps
    of different dt, negative included, and the states equal those of
    direct steps with the same dt sequence bit for bit.  Gravity alone is
    time-reversible under the leapfrog: steps of dt1, dt2, -dt2, -dt1 bring
    the particles back to where they started, up to rounding."""
    pos, vel, m = g.ics.plummer(20000, seed=17)
    soft = np.full(len(m), 0.01)
    gp = g.grav_params(periodic=False, precision=g.FP32)
    seq = (1e-3, 2e-3, -2e-3, -1e-3)
    states = []
    for graph in (False, True):
        c = g.Context(0)
        try:
            c.set_particles(pos, m, soft)
            c.set_velocities(vel)
            c.grav_all(gp)
            for dt in seq:
                c.step(dt, gp, None, graph=graph)
            c.step_status()
            states.append(c.get_state())
        finally:
            c.close()
    for k in range(2):
        assert np.array_equal(states[0][k], states[1][k]), k
    scale = np.abs(pos).max()
    assert np.abs(states[1][0] - pos).max() <= 1e-12 * scale
    assert np.abs(states[1][1] - vel).max() <= 1e-9 * np.abs(vel).max()
