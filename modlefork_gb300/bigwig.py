"""bigWig files for the 1D LEF occupancy track.

The reference writes the track with libBigWig (io::bigwig::Writer, src/libmodle_io/bigwig.cpp;
write_range, bigwig_impl.hpp:72-97; called from Simulation::write_1d_lef_occupancy_to_disk,
simulation.cpp:214-262): the genome's chromosome list, then for every chromosome with a track
one run of float32 values with span = step = bin size from the chromosome's start
(bwAddIntervalSpanSteps), 10 zoom levels.  libBigWig is not available here, so this module
writes the same data from the published bigWig layout (Kent et al., Bioinformatics 2010, and
the UCSC bigWig/bigBed format description):

* a 64-byte header, the zoom headers and a 40-byte total summary;
* the chromosome B+ tree (names sorted byte-wise, ids in that order);
* the data: a section count, then zlib-compressed fixedStep sections of up to ITEMS_PER_SLOT
  values each;
* an R-tree over the sections (BLOCK_SIZE children per node, root first);
* per zoom level, summary records (valid bases, min, max, sum, sum of squares over windows of
  `reduction` bases, aligned at multiples of it) in compressed blocks, with their own R-tree.

The files are not byte-identical to libBigWig's (its zoom reductions and block packing are its
own), but hold the same chromosomes, intervals and float32 values.  read_bigwig parses the
same layout back.
"""

import struct
import zlib

import numpy as np

BIGWIG_MAGIC = 0x888FFC26
BPT_MAGIC = 0x78CA8C91
CIRTREE_MAGIC = 0x2468ACE0
VERSION = 4
BLOCK_SIZE = 256
ITEMS_PER_SLOT = 1024
ZOOM_LEVELS = 10
ZOOM_FACTOR = 4

_HDR = struct.Struct("<IHHQQQHHQQIQ")       # 64 bytes
_ZOOM_HDR = struct.Struct("<IIQQ")          # 24 bytes
_SUMMARY = struct.Struct("<Qdddd")          # 40 bytes
_BPT_HDR = struct.Struct("<IIIIQQ")         # 32 bytes
_NODE_HDR = struct.Struct("<BBH")           # 4 bytes
_CIR_HDR = struct.Struct("<IIQIIIIQII")     # 48 bytes
_CIR_LEAF = struct.Struct("<IIIIQQ")        # 32 bytes
_CIR_INNER = struct.Struct("<IIIIQ")        # 24 bytes
_SECTION = struct.Struct("<IIIIIBBH")       # 24 bytes
_ZOOM_REC = struct.Struct("<IIIIffff")      # 32 bytes

assert _HDR.size == 64 and _CIR_HDR.size == 48 and _SECTION.size == 24 and _ZOOM_REC.size == 32


class Track:
    """One fixed-step run of values: item k covers [start + k*step, start + k*step + span)."""

    def __init__(self, chrom, start, span, step, values):
        self.chrom = str(chrom)
        self.start = int(start)
        self.span = int(span)
        self.step = int(step)
        self.values = np.ascontiguousarray(values, dtype=np.float32)
        if self.span <= 0 or self.step <= 0:
            raise ValueError("span and step must be positive")


def _levels(items, block_size):
    """Bottom-up tree levels: level 0 holds chunks of `items`, level k chunks of level k - 1's
    nodes, up to a single root node."""
    levels = [[items[i:i + block_size] for i in range(0, len(items), block_size)] or [[]]]
    while len(levels[-1]) > 1:
        prev = levels[-1]
        levels.append([prev[i:i + block_size] for i in range(0, len(prev), block_size)])
    return levels


def _node_offsets(levels, base, leaf_bytes, inner_bytes):
    """File offsets of every node, root level first, each node padded to its full size."""
    offs, pos = {}, base
    for lv in range(len(levels) - 1, -1, -1):
        for k in range(len(levels[lv])):
            offs[(lv, k)] = pos
            pos += leaf_bytes if lv == 0 else inner_bytes
    return offs


def _cir_index(entries, base, items_per_slot, block_size=BLOCK_SIZE):
    """R-tree over leaf entries (chrom_id, start, chrom_id_end, end, offset, size) with its
    header at file offset `base`."""
    if entries:
        s0, b0, s1, b1 = entries[0][0], entries[0][1], entries[-1][2], entries[-1][3]
    else:
        s0 = b0 = s1 = b1 = 0
    hdr = _CIR_HDR.pack(CIRTREE_MAGIC, block_size, len(entries), s0, b0, s1, b1, base, items_per_slot, 0)
    levels = _levels(list(entries), block_size)
    leaf_bytes = _NODE_HDR.size + block_size * _CIR_LEAF.size
    inner_bytes = _NODE_HDR.size + block_size * _CIR_INNER.size
    offs = _node_offsets(levels, base + _CIR_HDR.size, leaf_bytes, inner_bytes)
    # range of every node: (first chrom, first start, last chrom, last end)
    rng = {}
    for k, node in enumerate(levels[0]):
        rng[(0, k)] = (node[0][0], node[0][1], node[-1][2], node[-1][3]) if node else (0, 0, 0, 0)
    for lv in range(1, len(levels)):
        first = 0
        for k, node in enumerate(levels[lv]):
            lo, hi = rng[(lv - 1, first)], rng[(lv - 1, first + len(node) - 1)]
            rng[(lv, k)] = (lo[0], lo[1], hi[2], hi[3])
            first += len(node)
    body = bytearray()
    for lv in range(len(levels) - 1, -1, -1):
        first = 0
        for node in levels[lv]:
            body += _NODE_HDR.pack(1 if lv == 0 else 0, 0, len(node))
            if lv == 0:
                for e in node:
                    body += _CIR_LEAF.pack(*e)
                body += bytes((block_size - len(node)) * _CIR_LEAF.size)
            else:
                for j in range(len(node)):
                    body += _CIR_INNER.pack(*rng[(lv - 1, first + j)], offs[(lv - 1, first + j)])
                body += bytes((block_size - len(node)) * _CIR_INNER.size)
            first += len(node)
    return hdr + bytes(body)


def _chrom_tree(chroms, base, block_size=BLOCK_SIZE):
    """B+ tree of the chromosomes with its header at file offset `base`: names sorted byte-wise,
    ids in that order; returns (bytes, {name: id})."""
    names = sorted(chroms, key=lambda c: c[0].encode())
    key_size = max(1, max((len(n.encode()) for n, _ in names), default=1))
    bs = max(1, min(block_size, len(names)))
    items = [(n.encode().ljust(key_size, b"\0"), i, int(sz)) for i, (n, sz) in enumerate(names)]
    hdr = _BPT_HDR.pack(BPT_MAGIC, bs, key_size, 8, len(items), 0)
    levels = _levels(items, bs)
    node_bytes = _NODE_HDR.size + bs * (key_size + 8)
    offs = _node_offsets(levels, base + _BPT_HDR.size, node_bytes, node_bytes)
    first_key = {}
    for k, node in enumerate(levels[0]):
        first_key[(0, k)] = node[0][0] if node else b"\0" * key_size
    for lv in range(1, len(levels)):
        first = 0
        for k, node in enumerate(levels[lv]):
            first_key[(lv, k)] = first_key[(lv - 1, first)]
            first += len(node)
    body = bytearray()
    for lv in range(len(levels) - 1, -1, -1):
        first = 0
        for node in levels[lv]:
            body += _NODE_HDR.pack(1 if lv == 0 else 0, 0, len(node))
            for j, it in enumerate(node):
                if lv == 0:
                    body += it[0] + struct.pack("<II", it[1], it[2])
                else:
                    body += first_key[(lv - 1, first + j)] + struct.pack("<Q", offs[(lv - 1, first + j)])
            body += bytes((bs - len(node)) * (key_size + 8))
            first += len(node)
    return hdr + bytes(body), {n: i for i, (n, _) in enumerate(names)}


def _zoom_records(tracks, ids, sizes, reduction):
    """Summary records of one zoom level: windows of `reduction` bases aligned at multiples of
    it and clipped to the chromosome, over every track's items (overlap-weighted sums).  An item
    no longer than the window overlaps at most two windows, so each item is split in two pieces
    and the windows' sums are accumulated with bincount."""
    recs = []
    for t in sorted(tracks, key=lambda t: (ids[t.chrom], t.start)):
        n = t.values.size
        if n == 0:
            continue
        size = sizes[t.chrom]
        starts = t.start + np.arange(n, dtype=np.int64) * t.step
        ends = np.minimum(starts + t.span, size)
        keep = ends > starts
        starts, ends, v = starts[keep], ends[keep], t.values[keep].astype(np.float64)
        if starts.size == 0:
            continue
        if t.span > reduction:
            raise ValueError("zoom windows must be at least one item long")
        w_first = starts // reduction
        w_last = (ends - 1) // reduction
        cut = np.minimum((w_first + 1) * reduction, ends)
        win = np.concatenate([w_first, w_last])
        ov = np.concatenate([cut - starts, np.where(w_last > w_first, ends - cut, 0)])
        vals = np.concatenate([v, v])
        m = ov > 0
        win, ov, vals = win[m], ov[m].astype(np.float64), vals[m]
        w0 = int(win.min())
        idx = win - w0
        nw = int(idx.max()) + 1
        covered = np.bincount(idx, weights=ov, minlength=nw)
        ssum = np.bincount(idx, weights=vals * ov, minlength=nw)
        ssq = np.bincount(idx, weights=vals * vals * ov, minlength=nw)
        vmin = np.full(nw, np.inf)
        vmax = np.full(nw, -np.inf)
        np.minimum.at(vmin, idx, vals)
        np.maximum.at(vmax, idx, vals)
        cid = ids[t.chrom]
        for k in np.nonzero(covered > 0)[0].tolist():
            lo = (w0 + k) * reduction
            recs.append((cid, lo, min(lo + reduction, size), int(covered[k]), float(vmin[k]), float(vmax[k]),
                         float(ssum[k]), float(ssq[k])))
    return recs


def write_bigwig(path, chroms, tracks, zoom_levels=ZOOM_LEVELS, items_per_slot=ITEMS_PER_SLOT):
    """Write `tracks` (Track objects) over the chromosome list `chroms` [(name, size)]."""
    sizes = {n: int(s) for n, s in chroms}
    for t in tracks:
        if t.chrom not in sizes:
            raise ValueError(f"track on unknown chromosome {t.chrom!r}")
    span = max((t.span for t in tracks), default=1)  # every item fits a zoom window
    max_size = max(sizes.values(), default=0)
    reductions = []
    r = span * ZOOM_FACTOR
    while len(reductions) < zoom_levels and r < max_size:
        reductions.append(r)
        r *= ZOOM_FACTOR
    nz = len(reductions)
    chrom_tree_off = _HDR.size + nz * _ZOOM_HDR.size + _SUMMARY.size
    tree, ids = _chrom_tree(chroms, chrom_tree_off)
    data_off = chrom_tree_off + len(tree)
    # sections, in chromosome-id then position order
    sections, max_raw = [], 0
    for t in sorted(tracks, key=lambda t: (ids[t.chrom], t.start)):
        for k0 in range(0, t.values.size, items_per_slot):
            vals = t.values[k0:k0 + items_per_slot]
            s = t.start + k0 * t.step
            e = s + (vals.size - 1) * t.step + t.span
            raw = _SECTION.pack(ids[t.chrom], s, e, t.step, t.span, 3, 0, vals.size) + vals.astype("<f4").tobytes()
            max_raw = max(max_raw, len(raw))
            sections.append((ids[t.chrom], s, e, zlib.compress(raw)))
    body = bytearray(struct.pack("<Q", len(sections)))
    entries = []
    pos = data_off + 8
    for cid, s, e, blob in sections:
        entries.append((cid, s, cid, e, pos, len(blob)))
        body += blob
        pos += len(blob)
    index_off = pos
    index = _cir_index(entries, index_off, items_per_slot)
    pos += len(index)
    # zoom levels
    zoom_hdrs, zoom_bytes = [], bytearray()
    for red in reductions:
        recs = _zoom_records(tracks, ids, sizes, red)
        zdata_off = pos
        blob = bytearray(struct.pack("<I", len(recs)))
        zentries = []
        p = zdata_off + 4
        for k0 in range(0, len(recs), items_per_slot):
            chunk = recs[k0:k0 + items_per_slot]
            raw = b"".join(_ZOOM_REC.pack(*rc) for rc in chunk)
            max_raw = max(max_raw, len(raw))
            c = zlib.compress(raw)
            zentries.append((chunk[0][0], chunk[0][1], chunk[-1][0], chunk[-1][2], p, len(c)))
            blob += c
            p += len(c)
        zindex_off = p
        zindex = _cir_index(zentries, zindex_off, items_per_slot)
        zoom_bytes += blob + zindex
        pos = zindex_off + len(zindex)
        zoom_hdrs.append(_ZOOM_HDR.pack(red, 0, zdata_off, zindex_off))
    # total summary over all items
    covered, vmin, vmax, vsum, vsq = 0, np.inf, -np.inf, 0.0, 0.0
    for t in tracks:
        if t.values.size:
            v = t.values.astype(np.float64)
            covered += t.values.size * t.span
            vmin, vmax = min(vmin, float(v.min())), max(vmax, float(v.max()))
            vsum += float((v * t.span).sum())
            vsq += float((v * v * t.span).sum())
    if covered == 0:
        vmin = vmax = 0.0
    summary_off = _HDR.size + nz * _ZOOM_HDR.size
    hdr = _HDR.pack(BIGWIG_MAGIC, VERSION, nz, chrom_tree_off, data_off, index_off, 0, 0, 0,
                    summary_off, max_raw, 0)
    with open(path, "wb") as f:
        f.write(hdr)
        for z in zoom_hdrs:
            f.write(z)
        f.write(_SUMMARY.pack(covered, vmin, vmax, vsum, vsq))
        f.write(tree)
        f.write(body)
        f.write(index)
        f.write(zoom_bytes)


# ---------------------------------------------------------------------------------------------
# reader

def _read_cir_leaves(buf, off):
    magic, bs, count, *_ = _CIR_HDR.unpack_from(buf, off)
    if magic != CIRTREE_MAGIC:
        raise ValueError("bad R-tree magic")
    out = []

    def walk(node_off):
        is_leaf, _, n = _NODE_HDR.unpack_from(buf, node_off)
        p = node_off + _NODE_HDR.size
        for _ in range(n):
            if is_leaf:
                out.append(_CIR_LEAF.unpack_from(buf, p))
                p += _CIR_LEAF.size
            else:
                walk(_CIR_INNER.unpack_from(buf, p)[4])
                p += _CIR_INNER.size

    walk(off + _CIR_HDR.size)
    if len(out) != count:
        raise ValueError("R-tree item count mismatch")
    return out


def _read_chrom_tree(buf, off):
    magic, bs, key_size, val_size, count, _ = _BPT_HDR.unpack_from(buf, off)
    if magic != BPT_MAGIC or val_size != 8:
        raise ValueError("bad chromosome tree")
    out = []

    def walk(node_off):
        is_leaf, _, n = _NODE_HDR.unpack_from(buf, node_off)
        p = node_off + _NODE_HDR.size
        for _ in range(n):
            key = bytes(buf[p:p + key_size]).rstrip(b"\0").decode()
            if is_leaf:
                cid, size = struct.unpack_from("<II", buf, p + key_size)
                out.append((key, cid, size))
            else:
                walk(struct.unpack_from("<Q", buf, p + key_size)[0])
            p += key_size + 8

    walk(off + _BPT_HDR.size)
    if len(out) != count:
        raise ValueError("chromosome tree item count mismatch")
    return out


def read_bigwig(path):
    """Parse a file written by write_bigwig: returns dict(chroms=[(name, size)] in id order,
    intervals={name: [(start, end, value)]}, zooms=[(reduction, records)], summary=(bases,
    min, max, sum, sum of squares), uncompress_buf_size)."""
    buf = memoryview(open(path, "rb").read())
    (magic, version, nz, ctree, data_off, index_off, _, _, _, summary_off, ubuf, _) = _HDR.unpack_from(buf, 0)
    if magic != BIGWIG_MAGIC or version < 4:
        raise ValueError("not a bigWig file")
    chroms = _read_chrom_tree(buf, ctree)
    by_id = {cid: (name, size) for name, cid, size in chroms}
    intervals = {name: [] for name, _, _ in chroms}
    for cid0, s, cid1, e, off, size in _read_cir_leaves(buf, index_off):
        raw = zlib.decompress(bytes(buf[off:off + size]))
        if len(raw) > ubuf:
            raise ValueError("section larger than the declared buffer")
        cid, start, end, step, span, typ, _, n = _SECTION.unpack_from(raw, 0)
        if typ != 3:
            raise ValueError("only fixedStep sections are written here")
        vals = np.frombuffer(raw, dtype="<f4", count=n, offset=_SECTION.size)
        name = by_id[cid][0]
        for k in range(n):
            intervals[name].append((start + k * step, start + k * step + span, float(vals[k])))
    zooms = []
    for z in range(nz):
        red, _, zdata, zindex = _ZOOM_HDR.unpack_from(buf, _HDR.size + z * _ZOOM_HDR.size)
        recs = []
        for _, _, _, _, off, size in _read_cir_leaves(buf, zindex):
            raw = zlib.decompress(bytes(buf[off:off + size]))
            for k in range(len(raw) // _ZOOM_REC.size):
                recs.append(_ZOOM_REC.unpack_from(raw, k * _ZOOM_REC.size))
        zooms.append((red, recs))
    summary = _SUMMARY.unpack_from(buf, summary_off)
    return dict(chroms=[(by_id[i][0], by_id[i][1]) for i in sorted(by_id)], intervals=intervals,
                zooms=zooms, summary=summary, uncompress_buf_size=ubuf)
