"""bigWig output of the 1D LEF occupancy track (modlefork_gb300/bigwig.py).

libBigWig, which the reference writes the track with, is not available here, so the files are
checked by parsing them back: chromosome list, fixed-step intervals and float32 values, the
index trees (one and several levels), the zoom summaries against a direct computation, and the
values the reference computes from the counters (simulation.cpp:245-255).
"""

import struct

import numpy as np
import pytest

from modlefork_gb300 import bigwig as bw
from modlefork_gb300 import engine
from modlefork_gb300.simulate import ChromResult, occupancy_values, write_lef_occupancy_bigwig


def _roundtrip(tmp_path, chroms, tracks, **kw):
    p = tmp_path / "t.bw"
    bw.write_bigwig(str(p), chroms, tracks, **kw)
    return p, bw.read_bigwig(str(p))


def _expected_intervals(t):
    return [(t.start + k * t.step, t.start + k * t.step + t.span, float(v)) for k, v in enumerate(t.values)]


def test_roundtrip_values_and_chromosomes(tmp_path):
    rng = np.random.default_rng(1)
    chroms = [("chr2", 50_000), ("chr10", 120_345), ("chrX", 999), ("chr1", 77_001)]
    tracks = [bw.Track("chr10", 345, 1000, 1000, rng.random(120).astype(np.float32)),
              bw.Track("chr1", 0, 500, 500, rng.random(155).astype(np.float32)),
              bw.Track("chr2", 7, 250, 250, np.zeros(200, np.float32))]
    p, d = _roundtrip(tmp_path, chroms, tracks)
    # ids follow the byte-wise name order; every chromosome is listed, with or without data
    assert d["chroms"] == sorted(chroms, key=lambda c: c[0].encode())
    for t in tracks:
        assert d["intervals"][t.chrom] == _expected_intervals(t)
    assert d["intervals"]["chrX"] == []
    raw = p.read_bytes()
    magic, version = struct.unpack_from("<IH", raw, 0)
    assert magic == bw.BIGWIG_MAGIC and version == 4
    covered, vmin, vmax, vsum, vsq = d["summary"]
    allv = np.concatenate([t.values for t in tracks]).astype(np.float64)
    assert covered == sum(t.values.size * t.span for t in tracks)
    assert vmin == allv.min() and vmax == allv.max()
    assert np.isclose(vsum, sum(float((t.values.astype(np.float64) * t.span).sum()) for t in tracks))


def test_multilevel_trees(tmp_path):
    """More chromosomes and sections than one node holds: both trees get inner levels."""
    rng = np.random.default_rng(2)
    chroms = [(f"c{k:04d}", 10_000 + k) for k in range(600)]
    tracks = [bw.Track(f"c{k:04d}", 0, 100, 100, rng.random(100).astype(np.float32)) for k in range(0, 600, 2)]
    tracks.append(bw.Track("c0001", 0, 10, 10, rng.random(1000).astype(np.float32)))
    _, d = _roundtrip(tmp_path, chroms, tracks, items_per_slot=8)
    assert len(d["chroms"]) == 600 and d["chroms"] == chroms
    for t in tracks:
        assert d["intervals"][t.chrom] == _expected_intervals(t)


def _brute_zoom(track, size, reduction):
    out = []
    items = [(s, min(e, size), v) for s, e, v in _expected_intervals(track) if min(e, size) > s]
    w = items[0][0] // reduction
    while w * reduction < items[-1][1]:
        lo, hi = w * reduction, min((w + 1) * reduction, size)
        cov, mn, mx, sm, sq = 0, np.inf, -np.inf, 0.0, 0.0
        for s, e, v in items:
            o = min(e, hi) - max(s, lo)
            if o > 0:
                cov += o
                mn, mx = min(mn, v), max(mx, v)
                sm += v * o
                sq += v * v * o
        if cov:
            out.append((lo, hi, cov, mn, mx, sm, sq))
        w += 1
    return out


def test_zoom_summaries_match_a_direct_computation(tmp_path):
    rng = np.random.default_rng(3)
    size = 98_765  # the last item runs past the chromosome end, as the reference writes it
    t = bw.Track("chrA", 1_234, 1000, 1000, rng.random(98).astype(np.float32))
    _, d = _roundtrip(tmp_path, [("chrA", size)], [t])
    assert [r for r, _ in d["zooms"]] == [4000, 16000, 64000]
    for red, recs in d["zooms"]:
        want = _brute_zoom(t, size, red)
        assert len(recs) == len(want)
        for (cid, lo, hi, cov, mn, mx, sm, sq), (wlo, whi, wcov, wmn, wmx, wsm, wsq) in zip(recs, want):
            assert (cid, lo, hi, cov) == (0, wlo, whi, wcov)
            assert mn == np.float32(wmn) and mx == np.float32(wmx)
            assert np.isclose(sm, wsm, rtol=1e-6) and np.isclose(sq, wsq, rtol=1e-6)


def test_rejects_unknown_chromosome(tmp_path):
    with pytest.raises(ValueError):
        bw.write_bigwig(str(tmp_path / "x.bw"), [("chr1", 100)], [bw.Track("chr2", 0, 10, 10, [1.0])])


def test_occupancy_values_follow_the_reference():
    occ = np.array([0, 3, 7, 7, 1], dtype=np.uint64)
    v = occupancy_values(occ)
    assert v.dtype == np.float32
    assert np.array_equal(v, (occ.astype(np.float64) / 7.0).astype(np.float32))
    assert np.isnan(occupancy_values(np.zeros(3, np.uint64))).all()  # 0.0 / 0.0, as there


def test_occupancy_bigwig_file(tmp_path):
    cfg = engine.config_defaults(bin_size=5000)
    chroms = [engine.Chromosome("chr1", 1_000_000, 100_000, 900_000), engine.Chromosome("chr2", 400_000)]
    nb = -(-chroms[0].size // 5000)
    occ = np.random.default_rng(4).integers(0, 50, nb).astype(np.uint64)
    res = [ChromResult(chroms[0], 10, None, 0, [], occupancy=occ)]
    p = tmp_path / "occ.bw"
    write_lef_occupancy_bigwig(str(p), cfg, res, chroms)
    d = bw.read_bigwig(str(p))
    assert d["chroms"] == [("chr1", 1_000_000), ("chr2", 400_000)]
    got = d["intervals"]["chr1"]
    vals = occupancy_values(occ)
    assert got == [(100_000 + k * 5000, 100_000 + (k + 1) * 5000, float(vals[k])) for k in range(nb)]
    assert d["intervals"]["chr2"] == []
