"""GPU tests of Tipsy snapshot I/O (tsph_read_tipsy / tsph_write_tipsy).

Bar: bit-exact.  Values read equal the reference's pkdReadTipsy output
(golden vectors) and the oracle's; files written are byte-identical to the
reference's pkdWriteTipsy output or to the oracle's writer; a snapshot
loaded from a file gives bit-identical forces to the same particles loaded
through tsph_set_particles / tsph_set_velocities.
"""
import os

import numpy as np
import pytest

import gasoline_gb300 as g
from oracle import tipsy
from golden_io import GOLD, load

pytestmark = pytest.mark.gpu


def _golden():
    d = load("tipsy_mixed")
    ng, nd, ns = (int(x) for x in d["counts"])
    return d, ng, nd, ns, d["factors"]


def _read_all(ctx):
    pos, vel, u = ctx.get_state()
    return pos, vel, u, ctx.get_snapshot_fields()


@pytest.mark.parametrize("tag,std", [("std", True), ("nat", False)])
def test_read_equals_reference_reader(ctx, tag, std):
    d, ng, nd, ns, (dvFac, duTFac, rvFac, rTuFac) = _golden()
    h = ctx.read_tipsy(os.path.join(GOLD, f"tipsy_mixed.{tag}"), standard=std, dvFac=rvFac,
                       dTuFac=rTuFac)
    assert (h["nsph"], h["ndark"], h["nstar"], h["time"]) == (ng, nd, ns, float(d["time"]))
    pos, vel, u, s = _read_all(ctx)
    f = d[f"f_{tag}"]
    assert np.array_equal(pos, d[f"pos_{tag}"])
    assert np.array_equal(vel, d[f"vel_{tag}"])
    assert np.array_equal(u, f[:ng, 2])
    assert np.array_equal(s["mass"], f[:, 0])
    assert np.array_equal(s["soft"], f[:, 1])
    assert np.array_equal(s["pot"], f[:, 6])
    assert np.array_equal(s["rho"][:ng].astype(np.float64), f[:ng, 3])
    assert np.array_equal(s["metals"][:ng].astype(np.float64), f[:ng, 4])
    assert np.array_equal(s["metals"][ng + nd:].astype(np.float64), f[ng + nd:, 4])
    assert np.array_equal(s["tform"][ng + nd:].astype(np.float64), f[ng + nd:, 5])


@pytest.mark.parametrize("tag,std", [("std", True), ("nat", False)])
def test_write_equals_reference_writer(ctx, scratch, tag, std):
    """The particles the reference wrote (double precision) loaded directly
    and written with the same unit factors give its file byte for byte."""
    d, ng, nd, ns, (dvFac, duTFac, _, _) = _golden()
    f = d["f"]
    ctx.set_particles(d["pos"], f[:, 0], f[:, 1])
    ctx.set_velocities(d["vel"], ngas=ng, u=f[:ng, 2])
    ctx.set_snapshot_fields(pot=f[:, 6], rho=f[:, 3], metals=f[:, 4], tform=f[:, 5])
    out = os.path.join(scratch, "w.bin")
    ctx.write_tipsy(out, float(d["time"]), standard=std, dvFac=dvFac, duTFac=duTFac, nstar=ns)
    with open(out, "rb") as a, open(os.path.join(GOLD, f"tipsy_mixed.{tag}"), "rb") as b:
        assert a.read() == b.read()


@pytest.mark.parametrize("tag,std", [("std", True), ("nat", False)])
def test_round_trip_is_byte_identical(ctx, scratch, tag, std):
    gold = os.path.join(GOLD, f"tipsy_mixed.{tag}")
    h = ctx.read_tipsy(gold, standard=std)
    out = os.path.join(scratch, "rt.bin")
    ctx.write_tipsy(out, h["time"], standard=std)
    with open(out, "rb") as a, open(gold, "rb") as b:
        assert a.read() == b.read()


def test_large_file_chunked_round_trip(ctx, scratch):
    """3.2M particles (several pipeline chunks, type boundaries inside
    chunks): read equals the oracle's reader, write(read(file)) == file."""
    ng, nd, ns = 1_100_003, 1_700_001, 400_007
    n = ng + nd + ns
    rng = np.random.default_rng(77)
    pos = rng.normal(size=(n, 3)); vel = rng.normal(size=(n, 3))
    f = np.zeros((n, 9))
    f[:, 0] = rng.uniform(0.5, 1.0, n); f[:, 1] = rng.uniform(0.001, 0.01, n)
    f[:, 6] = rng.normal(size=n)
    f[:ng, 2:5] = rng.uniform(0.0, 1.0, (ng, 3))
    f[ng + nd:, 4:6] = rng.uniform(0.0, 1.0, (ns, 2))
    src = os.path.join(scratch, "big.std")
    tipsy.write(src, 0.75, ng, nd, ns, pos, vel, f, standard=True)
    ctx.read_tipsy(src, standard=True, dvFac=2.0, dTuFac=3.0)
    _, p_o, v_o, f_o = tipsy.read(src, standard=True, dvFac=2.0, dTuFac=3.0)
    p, v, u, s = _read_all(ctx)
    assert np.array_equal(p, p_o) and np.array_equal(v, v_o)
    assert np.array_equal(u, f_o[:ng, 2]) and np.array_equal(s["mass"], f_o[:, 0])
    assert np.array_equal(s["pot"], f_o[:, 6])
    out = os.path.join(scratch, "big2.std")
    ctx.write_tipsy(out, 0.75, standard=True, dvFac=0.5, duTFac=1.0 / 3.0)
    back = os.path.join(scratch, "big3.std")
    tipsy.write(back, 0.75, ng, nd, ns, p, v, np.column_stack(
        [s["mass"], s["soft"], np.concatenate([u, np.zeros(n - ng)]), s["rho"], s["metals"],
         s["tform"], s["pot"], np.zeros(n), np.zeros(n)]), standard=True, dvFac=0.5,
        duTFac=1.0 / 3.0)
    with open(out, "rb") as a, open(back, "rb") as b:
        assert a.read() == b.read()


def test_forces_from_snapshot_equal_direct_load(ctx, scratch):
    """A gas + dark snapshot read from a file gives the same gravity and SPH
    results, bit for bit, as the same values set directly."""
    pg, vg, mg, u = g.ics.gas_sphere(6000, seed=61)
    pd, vd, md = g.ics.plummer(4000, seed=62)
    pos = np.concatenate([pg, pd]); vel = np.concatenate([vg, vd])
    n, ng = 10000, 6000
    f = np.zeros((n, 9))
    f[:, 0] = np.concatenate([0.3 * mg, 0.7 * md]); f[:, 1] = 0.01; f[:ng, 2] = u
    src = os.path.join(scratch, "s.std")
    tipsy.write(src, 0.0, ng, n - ng, 0, pos, vel, f, standard=True)
    _, p_o, v_o, f_o = tipsy.read(src, standard=True)
    gp = g.grav_params(periodic=False)
    sp = g.sph_params(nSmooth=32)
    res = []
    for via_file in (True, False):
        if via_file:
            ctx.read_tipsy(src, standard=True)
        else:
            ctx.set_particles(p_o, f_o[:, 0], f_o[:, 1])
            ctx.set_velocities(v_o, ngas=ng, u=f_o[:ng, 2])
        ctx.grav_all(gp)
        ctx.smooth(g.SMX_DENDVDX, sp)
        ctx.smooth(g.SMX_SPHPRESSURETERMS, sp)
        res.append((ctx.get_gravity(), ctx.get_sph()))
    (ga, sa), (gb, sb) = res
    for k in ("acc", "pot", "dtGrav"):
        assert np.array_equal(ga[k], gb[k]), k
    for k in ("fBall2", "fDensity", "ax", "uDotPdV", "uDotAV"):
        assert np.array_equal(sa[k], sb[k]), k


def test_write_after_forces_carries_density_and_potential(ctx, scratch):
    pos, vel, m, u = g.ics.gas_sphere(3000, seed=63)
    soft = np.full(3000, 0.01)
    ctx.set_particles(pos, m, soft)
    ctx.set_velocities(vel, ngas=3000, u=u)
    ctx.grav_all(g.grav_params(periodic=False))
    ctx.smooth(g.SMX_DENDVDX, g.sph_params(nSmooth=32))
    out = os.path.join(scratch, "f.std")
    ctx.write_tipsy(out, 0.1, standard=True, nstar=0)
    h, p, v, f = tipsy.read(out, standard=True)
    assert h["nsph"] == 3000 and h["ndark"] == 0
    rho = ctx.get_sph()["fDensity"]
    pot = ctx.get_gravity()["pot"]
    assert np.array_equal(f[:, 3], rho.astype(np.float32).astype(np.float64))
    assert np.array_equal(f[:, 6], pot.astype(np.float32).astype(np.float64))
    assert np.array_equal(f[:, 4], np.zeros(3000))      # no metals: not read from a file
    assert np.array_equal(p, pos.astype(np.float32).astype(np.float64))


def test_read_errors_leave_no_particles(ctx, scratch):
    d, ng, nd, ns, _ = _golden()
    gold = os.path.join(GOLD, "tipsy_mixed.std")
    with open(gold, "rb") as fh:
        data = fh.read()
    short = os.path.join(scratch, "short.std")
    with open(short, "wb") as fh:
        fh.write(data[:-10])
    with pytest.raises(g.TsphError) as ei:
        ctx.read_tipsy(short)
    assert ei.value.code == 12
    with pytest.raises(g.TsphError) as ei:
        ctx.grav_all(g.grav_params(periodic=False))
    assert ei.value.code == 8
    # a gas particle of zero mass (the reference's reader asserts > 0)
    bad = bytearray(data)
    bad[32:36] = b"\0\0\0\0"
    badp = os.path.join(scratch, "bad.std")
    with open(badp, "wb") as fh:
        fh.write(bytes(bad))
    with pytest.raises(g.TsphError) as ei:
        ctx.read_tipsy(badp)
    assert ei.value.code == 12
    with pytest.raises(g.TsphError) as ei:
        ctx.read_tipsy(os.path.join(scratch, "missing.std"))
    assert ei.value.code == 12
    # the context recovers with the next good load
    ctx.read_tipsy(gold)
    ctx.grav_all(g.grav_params(periodic=False))


def test_empty_snapshot(ctx, scratch):
    p = os.path.join(scratch, "empty.std")
    tipsy.write(p, 1.0, 0, 0, 0, np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 9)))
    h = ctx.read_tipsy(p)
    assert h["nbodies"] == 0
    out = os.path.join(scratch, "empty2.std")
    ctx.write_tipsy(out, 1.0)
    with open(out, "rb") as a, open(p, "rb") as b:
        assert a.read() == b.read()
