"""Tipsy snapshot format on the CPU: the oracle's restatement pinned to the
reference's own writer and reader (golden files written by pkdWriteTipsy,
values read back by pkdReadTipsy), and the library's header parser.

Bar: byte-identical files and bit-identical values (integer/byte work)."""
import os

import numpy as np
import pytest

import oracle
from oracle import tipsy
from golden_io import GOLD, load


def _golden():
    d = load("tipsy_mixed")
    ng, nd, ns = (int(x) for x in d["counts"])
    dvFac, duTFac, rvFac, rTuFac = d["factors"]
    return d, ng, nd, ns, dvFac, duTFac, rvFac, rTuFac


@pytest.mark.parametrize("tag,std", [("std", True), ("nat", False)])
def test_oracle_writer_matches_reference_file(scratch, tag, std):
    d, ng, nd, ns, dvFac, duTFac, _, _ = _golden()
    out = os.path.join(scratch, "o.bin")
    tipsy.write(out, float(d["time"]), ng, nd, ns, d["pos"], d["vel"], d["f"], standard=std,
                dvFac=dvFac, duTFac=duTFac)
    with open(out, "rb") as a, open(os.path.join(GOLD, f"tipsy_mixed.{tag}"), "rb") as b:
        assert a.read() == b.read()


@pytest.mark.parametrize("tag,std", [("std", True), ("nat", False)])
def test_oracle_reader_matches_reference_values(tag, std):
    d, ng, nd, ns, _, _, rvFac, rTuFac = _golden()
    h, pos, vel, f = tipsy.read(os.path.join(GOLD, f"tipsy_mixed.{tag}"), standard=std,
                                dvFac=rvFac, dTuFac=rTuFac)
    assert (h["nsph"], h["ndark"], h["nstar"], h["nbodies"], h["ndim"]) == (ng, nd, ns, ng + nd + ns, 3)
    assert h["time"] == float(d["time"])
    assert np.array_equal(pos, d[f"pos_{tag}"])
    assert np.array_equal(vel, d[f"vel_{tag}"])
    assert np.array_equal(f, d[f"f_{tag}"])


@pytest.mark.skipif(not oracle.reference_available(), reason="reference not built here")
@pytest.mark.parametrize("counts", [(0, 40, 0), (0, 0, 17), (25, 0, 0), (0, 0, 0), (7, 9, 3)])
@pytest.mark.parametrize("std", [True, False])
def test_oracle_vs_reference_edge_counts(scratch, counts, std):
    """Files with missing particle types (and an empty file) from the live
    reference build: identical bytes written, identical values read."""
    ng, nd, ns = counts
    rng = np.random.default_rng(sum(counts) + std)
    n = ng + nd + ns
    pos = rng.normal(size=(n, 3)); vel = rng.normal(size=(n, 3))
    f = np.zeros((n, 9))
    f[:, 0] = rng.uniform(0.5, 1.0, n); f[:, 1] = 0.01; f[:, 6] = -1.0
    f[:ng, 2:5] = rng.uniform(0.0, 1.0, (ng, 3))
    f[ng + nd:, 4:6] = rng.uniform(0.0, 1.0, (ns, 2))
    a, b = os.path.join(scratch, "a"), os.path.join(scratch, "b")
    oracle.reference_tipsy_write(a, std, 3.5, ng, nd, ns, pos, vel, f, dvFac=2.0, duTFac=0.5)
    tipsy.write(b, 3.5, ng, nd, ns, pos, vel, f, standard=std, dvFac=2.0, duTFac=0.5)
    with open(a, "rb") as fa, open(b, "rb") as fb:
        assert fa.read() == fb.read()
    p1, v1, f1 = oracle.reference_tipsy_read(a, std, ng, nd, ns, dvFac=0.5, dTuFac=3.0)
    _, p2, v2, f2 = tipsy.read(a, standard=std, dvFac=0.5, dTuFac=3.0)
    assert np.array_equal(p1, p2) and np.array_equal(v1, v2) and np.array_equal(f1, f2)


@pytest.mark.parametrize("tag,std", [("std", True), ("nat", False)])
def test_library_header_parser(tag, std):
    """tsph_tipsy_read_header is host code: it runs without a GPU."""
    import gasoline_gb300 as g
    h = g.tipsy_header(os.path.join(GOLD, f"tipsy_mixed.{tag}"), standard=std)
    assert h == tipsy.read_header(os.path.join(GOLD, f"tipsy_mixed.{tag}"), standard=std)


def test_library_header_errors(scratch):
    import gasoline_gb300 as g
    with pytest.raises(g.TsphError) as ei:
        g.tipsy_header(os.path.join(scratch, "missing"))
    assert ei.value.code == 12
    short = os.path.join(scratch, "short")
    with open(short, "wb") as fh:
        fh.write(b"\0" * 20)
    with pytest.raises(g.TsphError) as ei:
        g.tipsy_header(short)
    assert ei.value.code == 12
    # nbodies != nsph + ndark + nstar (the reference asserts it, master.c:3633)
    bad = os.path.join(scratch, "bad")
    h = np.zeros(1, dtype=[("time", ">f8"), ("nbodies", ">i4"), ("ndim", ">i4"), ("nsph", ">i4"),
                           ("ndark", ">i4"), ("nstar", ">i4"), ("pad", ">i4")])
    h["nbodies"], h["ndim"], h["nsph"], h["ndark"], h["nstar"] = 10, 3, 2, 3, 4
    h.tofile(bad)
    with pytest.raises(g.TsphError) as ei:
        g.tipsy_header(bad)
    assert ei.value.code == 12
