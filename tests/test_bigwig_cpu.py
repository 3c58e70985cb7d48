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


def test_file_layout_byte_by_byte(tmp_path):
    """Decode a written file at the byte offsets of the published bigWig layout (Kent et al.,
    Bioinformatics 26:2204, supplementary tables), without the module's reader or structs:
    the 64-byte header, the 24-byte zoom headers, the 40-byte total summary, the chromosome
    B+ tree (32-byte header, 4-byte node headers, key + id + size leaves), the 64-bit section
    count at the data offset, the 24-byte section headers, and the R-tree index (48-byte
    header whose end-of-data field equals the index offset, 32-byte leaf items)."""
    import zlib

    chroms = [("chrB", 40_000), ("chrA10", 90_001)]
    tracks = [bw.Track("chrA10", 1, 1000, 1000, np.arange(90, dtype=np.float32)),
              bw.Track("chrB", 0, 500, 500, np.full(80, 0.5, np.float32))]
    p = tmp_path / "layout.bw"
    bw.write_bigwig(str(p), chroms, tracks, items_per_slot=64)
    buf = open(p, "rb").read()
    u16 = lambda o: struct.unpack_from("<H", buf, o)[0]  # noqa: E731
    u32 = lambda o: struct.unpack_from("<I", buf, o)[0]  # noqa: E731
    u64 = lambda o: struct.unpack_from("<Q", buf, o)[0]  # noqa: E731
    # header
    assert u32(0) == 0x888FFC26 and u16(4) == 4
    nz = u16(6)
    tree_off, data_off, index_off = u64(8), u64(16), u64(24)
    assert u16(32) == 0 and u16(34) == 0 and u64(36) == 0  # fieldCount, definedFieldCount, autoSql
    summary_off, max_raw = u64(44), u32(52)
    assert u64(56) == 0
    assert summary_off == 64 + 24 * nz and tree_off == summary_off + 40 and nz >= 1
    # total summary: bases covered, min, max, sum, sum of squares
    covered, vmin, vmax, vsum, vsq = struct.unpack_from("<Qdddd", buf, summary_off)
    assert covered == 90 * 1000 + 80 * 500 and vmin == 0.0 and vmax == 89.0
    assert vsum == pytest.approx(1000 * sum(range(90)) + 500 * 0.5 * 80)
    # chromosome B+ tree
    assert u32(tree_off) == 0x78CA8C91
    block, key_size, val_size, count = u32(tree_off + 4), u32(tree_off + 8), u32(tree_off + 12), u64(tree_off + 16)
    assert key_size == len("chrA10") and val_size == 8 and count == 2 and block >= 2
    node = tree_off + 32
    assert buf[node] == 1 and u16(node + 2) == 2  # one leaf with both chromosomes
    leaf = []
    for k in range(2):
        it = node + 4 + k * (key_size + 8)
        leaf.append((buf[it:it + key_size].rstrip(b"\0").decode(), u32(it + key_size), u32(it + key_size + 4)))
    assert leaf == [("chrA10", 0, 90_001), ("chrB", 1, 40_000)]  # byte order of the names
    # data: a 64-bit section count, then zlib sections with 24-byte headers (type 3 = fixed step)
    nsec = u64(data_off)
    assert nsec == 2 + 2  # 90 values -> 2 sections of <= 64, 80 values -> 2
    # R-tree index of the sections
    assert u32(index_off) == 0x2468ACE0
    assert u64(index_off + 8) == nsec and u64(index_off + 32) == index_off and u32(index_off + 40) == 64
    node = index_off + 48
    assert buf[node] == 1 and u16(node + 2) == nsec
    seen = 0
    for k in range(nsec):
        it = node + 4 + 32 * k
        sc, sb, ec, eb, off, size = struct.unpack_from("<IIIIQQ", buf, it)
        raw = zlib.decompress(buf[off:off + size])
        assert len(raw) <= max_raw
        cid, s, e, step, span, typ, _, n = struct.unpack_from("<IIIIIBBH", raw, 0)
        assert (cid, s, e) == (sc, sb, eb) and sc == ec and typ == 3 and len(raw) == 24 + 4 * n
        seen += n
        assert data_off + 8 <= off < index_off
    assert seen == 170
    # zoom headers: reduction level, reserved, data offset (32-bit record count), index offset
    for z in range(nz):
        red, res, zdata, zindex = struct.unpack_from("<IIQQ", buf, 64 + 24 * z)
        assert res == 0 and zdata < zindex <= len(buf) - 48 and u32(zindex) == 0x2468ACE0
        assert u64(zindex + 32) == zindex  # its data ends where its index starts
        assert red == 1000 * 4 ** (z + 1)
