"""Python binding of the GB300 epoch engine (libmgpu_modle.so) through its C ABI.

This mirrors the reference's operator interface for the hot path: ``Engine`` plays the role
of ``modle::Simulation`` (src/libmodle/cpu/simulation.cpp:58-105) holding a transformed
Config, and ``Engine.simulate_cells`` is the batched drop-in for calling
``Simulation::simulate_one_cell`` once per (chromosome, cell) task
(src/libmodle/cpu/scheduler_simulate.cpp:229-256).  Errors surface as ``EngineError`` with
the library's status code and message; there is no CPU fallback: if the compiled library is
missing, loading fails.
"""

import ctypes as C
import os

import numpy as np

from . import _abi as abi

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libmgpu_modle.so")
_lib = None


class EngineError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{abi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(path=LIB_PATH):
    """Load the compiled engine; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run modlefork_gb300.build.build() first")
    lib = C.CDLL(path)
    P = C.POINTER
    u64, i32 = C.c_uint64, C.c_int
    sigs = {
        "mgpu_config_defaults": (None, [P(abi.Config)]),
        "mgpu_config_transform": (i32, [P(abi.Config)]),
        "mgpu_cell_seed": (u64, [C.c_char_p, u64, u64, u64, u64]),
        "mgpu_xxh3_64": (u64, [C.c_void_p, u64, u64]),
        "mgpu_num_lefs": (u64, [P(abi.Config), u64]),
        "mgpu_contacts_per_epoch": (u64, [P(abi.Config), u64]),
        "mgpu_npixels": (u64, [P(abi.Config), u64]),
        "mgpu_band_shape": (None, [P(abi.Config), u64, P(u64), P(u64)]),
        "mgpu_task_targets": (i32, [P(abi.Config), u64, u64, u64, P(u64), P(u64)]),
        "mgpu_barrier_from_bed": (i32, [P(abi.Chrom), u64, u64, C.c_char, C.c_double, C.c_double,
                                        C.c_double, P(abi.Barrier)]),
        "mgpu_sort_barriers": (i32, [P(abi.Barrier), u64]),
        "mgpu_last_error_string": (C.c_char_p, []),
        "mgpu_abi_version": (i32, []),
        "mgpu_create": (i32, [i32, P(abi.Config), P(C.c_void_p)]),
        "mgpu_destroy": (i32, [C.c_void_p]),
        "mgpu_sync": (i32, [C.c_void_p]),
        "mgpu_upload_chrom": (i32, [C.c_void_p, P(abi.Chrom), P(abi.Barrier), u64, P(i32)]),
        "mgpu_upload_window": (i32, [C.c_void_p, P(abi.Chrom), u64, u64, P(abi.Barrier), u64, P(i32)]),
        "mgpu_set_chrom_config": (i32, [C.c_void_p, i32, P(abi.Config)]),
        "mgpu_simulate_cells": (i32, [C.c_void_p, i32, C.c_void_p, C.c_void_p, u64, u64, u64,
                                      C.c_void_p, C.c_void_p, C.c_void_p]),
        "mgpu_simulate_cells_noalloc": (i32, [C.c_void_p, i32, C.c_void_p, C.c_void_p, u64, u64, u64,
                                              C.c_void_p, C.c_void_p, C.c_void_p]),
        "mgpu_simulate_cells_ex": (i32, [C.c_void_p, i32, C.c_void_p, C.c_void_p, u64, u64, u64,
                                         C.c_void_p, C.c_void_p, C.c_void_p, P(abi.ExtraOutputs)]),
        "mgpu_simulate_batch": (i32, [C.c_void_p, P(abi.BatchTask), u64, P(C.c_void_p), u64, C.c_void_p,
                                      C.c_void_p]),
        "mgpu_band_to_pixels": (i32, [C.c_void_p, C.c_void_p, u64, u64, u64, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, u64, P(u64)]),
        "mgpu_trace_cell": (i32, [C.c_void_p, i32, u64, u64, u64, u64, C.c_void_p,
                                  P(abi.CellStats), P(abi.TraceRequest)]),
        "mgpu_state_digest": (u64, [u64] + [P(u64)] * 9),
        "mgpu_run_phase": (i32, [C.c_void_p, i32, i32, P(abi.PhaseIO)]),
        "mgpu_prng_seed": (None, [u64, P(u64)]),
        "mgpu_set_stream": (i32, [C.c_void_p, C.c_void_p]),
        "mgpu_last_kernel_ms": (i32, [C.c_void_p, P(C.c_double)]),
        "mgpu_set_debug_flags": (i32, [C.c_void_p, C.c_uint32, u64]),
        "mgpu_last_profile": (i32, [C.c_void_p, P(u64)]),
        "mgpu_set_launch_table": (i32, [C.c_void_p, P(abi.LaunchSetting), u64]),
        "mgpu_probe_samplers": (i32, [i32, i32, C.c_void_p, u64, u64, C.c_double, C.c_double, C.c_void_p,
                                      C.c_void_p]),
        "mgpu_probe_libm": (i32, [i32, i32, C.c_void_p, C.c_void_p, u64, C.c_double, C.c_double, C.c_double,
                                  C.c_void_p]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _check(rc, what=""):
    if rc != abi.MGPU_OK:
        msg = _lib.mgpu_last_error_string().decode(errors="replace")
        raise EngineError(rc, f"{what}: {msg}" if what else msg)


def config_defaults(**overrides):
    """modle::Config defaults (simulation_config.hpp:24-135) with keyword overrides."""
    lib = load()
    cfg = abi.Config()
    lib.mgpu_config_defaults(C.byref(cfg))
    for k, v in overrides.items():
        if not hasattr(cfg, k):
            raise KeyError(k)
        setattr(cfg, k, v)
    return cfg


def config_transform(cfg):
    """Cli::transform_args (src/modle/cli.cpp:1194-1215), in place."""
    lib = load()
    _check(lib.mgpu_config_transform(C.byref(cfg)), "mgpu_config_transform")
    return cfg


def cell_seed(name, chrom_size, seed, cell_id):
    """Chromosome::hash (src/libmodle/internal/genome.cpp:317-335)."""
    lib = load()
    b = name.encode() if isinstance(name, str) else bytes(name)
    return lib.mgpu_cell_seed(b, len(b), chrom_size, seed, cell_id)


def num_lefs(cfg, size_bp):
    return load().mgpu_num_lefs(C.byref(cfg), size_bp)


def band_shape(cfg, size_bp):
    nr, nc = C.c_uint64(), C.c_uint64()
    load().mgpu_band_shape(C.byref(cfg), size_bp, C.byref(nr), C.byref(nc))
    return nr.value, nc.value


def task_targets(cfg, size_bp, nlefs, ncells):
    t = np.zeros(ncells, dtype=np.uint64)
    e = C.c_uint64()
    _check(load().mgpu_task_targets(C.byref(cfg), size_bp, nlefs, ncells,
                                    t.ctypes.data_as(C.POINTER(C.c_uint64)), C.byref(e)),
           "mgpu_task_targets")
    return t, e.value


def barriers_from_bed(chrom, records, default_stp_active, default_stp_inactive):
    """BED records (start, end, strand, score) -> barrier list (genome.cpp:194-210)."""
    lib = load()
    ch = chrom.as_abi()
    out = []
    b = abi.Barrier()
    for (s, e, strand, score) in records:
        rc = lib.mgpu_barrier_from_bed(C.byref(ch), s, e, strand.encode(), float(score),
                                       default_stp_active, default_stp_inactive, C.byref(b))
        if rc < 0:
            _check(rc, "mgpu_barrier_from_bed")
        if rc == 1:
            out.append(dict(pos=b.pos, stp_active=b.stp_active, stp_inactive=b.stp_inactive,
                            blocking_dir=b.blocking_dir))
    return out


PROBE_NORMAL, PROBE_EXPONENTIAL, PROBE_POISSON, PROBE_BINOMIAL, PROBE_BINOMIAL_DEVICE_POW, PROBE_GEV = range(6)
PROBE_LOG, PROBE_EXP, PROBE_POW, PROBE_GEV_NOISE, PROBE_BELOW_EXP = range(5)


def probe_samplers(kind, seeds, per_stream, a0=0.0, a1=0.0, device=0):
    """The epoch loop's serial samplers on the device (test hook mgpu_probe_samplers):
    (samples[nstreams, per_stream], draws[nstreams])."""
    seeds = np.ascontiguousarray(seeds, dtype=np.uint64)
    out = np.empty((len(seeds), per_stream), dtype=np.float64)
    draws = np.empty(len(seeds), dtype=np.uint64)
    _check(load().mgpu_probe_samplers(device, kind, seeds.ctypes.data, len(seeds), per_stream, a0, a1,
                                      out.ctypes.data, draws.ctypes.data), "mgpu_probe_samplers")
    return out, draws


def probe_libm(kind, x, y=None, mu=0.0, sigma=0.0, xi=0.0, device=0):
    """The device's log / exp / pow / GEV noise / below_exp on arguments (test hook
    mgpu_probe_libm)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    yp = None
    if y is not None:
        y = np.ascontiguousarray(y, dtype=np.float64)
        yp = y.ctypes.data
    out = np.empty_like(x)
    _check(load().mgpu_probe_libm(device, kind, x.ctypes.data, yp, len(x), mu, sigma, xi, out.ctypes.data),
           "mgpu_probe_libm")
    return out


class Chromosome:
    """Simulated range of one chromosome (modle::Chromosome)."""

    def __init__(self, name, size, start=0, end=None):
        self.name = name
        self.size = int(size)
        self.start = int(start)
        self.end = int(size if end is None else end)

    @property
    def simulated_size(self):
        return self.end - self.start

    def as_abi(self):
        ch = abi.Chrom()
        self._name_bytes = self.name.encode()
        ch.name = self._name_bytes
        ch.name_len = len(self._name_bytes)
        ch.size = self.size
        ch.start = self.start
        ch.end = self.end
        return ch


class Engine:
    """A device context bound to one transformed Config (like modle::Simulation)."""

    def __init__(self, cfg, device=0):
        self.lib = load()
        self.cfg = cfg
        h = C.c_void_p()
        _check(self.lib.mgpu_create(device, C.byref(cfg), C.byref(h)), "mgpu_create")
        self.h = h
        self.chroms = {}

    def close(self):
        if self.h:
            self.lib.mgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def upload_chrom(self, chrom, barriers):
        """Upload a chromosome and its barriers (IITree order); returns the handle."""
        ch = chrom.as_abi()
        bs = abi.make_barriers(barriers)
        cid = C.c_int()
        _check(self.lib.mgpu_upload_chrom(self.h, C.byref(ch), bs, len(barriers), C.byref(cid)),
               "mgpu_upload_chrom")
        self.chroms[cid.value] = chrom
        return cid.value

    def upload_window(self, chrom, window_start, window_end, barriers):
        """mgpu_upload_window: a window of ``chrom`` (binding, contacts and band inside
        [window_start, window_end), moves clamped by the chromosome); returns the handle."""
        ch = chrom.as_abi()
        bs = abi.make_barriers(barriers)
        cid = C.c_int()
        _check(self.lib.mgpu_upload_window(self.h, C.byref(ch), window_start, window_end, bs, len(barriers),
                                           C.byref(cid)), "mgpu_upload_window")
        self.chroms[cid.value] = chrom
        return cid.value

    def set_chrom_config(self, chrom_id, cfg):
        """mgpu_set_chrom_config: simulate ``chrom_id`` with its own (transformed) configuration
        instead of the engine's; None restores the engine's."""
        _check(self.lib.mgpu_set_chrom_config(self.h, chrom_id, C.byref(cfg) if cfg is not None else None),
               "mgpu_set_chrom_config")

    def simulate_cells(self, chrom_id, seeds, targets, target_epochs, nlefs, band=None,
                       stats=True, ncells=None):
        """Simulate the cells given by ``seeds`` and ``targets``; contacts are added into
        ``band``.  Each of seeds, targets and band is either a host numpy array or a device
        pointer (an int, e.g. a torch tensor's data_ptr()); with device seeds and targets
        ``ncells`` is required.  Returns (missed_updates, per-cell stats array or None)."""
        def as_ptr(a, dtype, name):
            if isinstance(a, (int, np.integer)):
                if ncells is None:
                    raise ValueError(f"{name} is a device pointer: pass ncells")
                return int(a), None
            arr = np.ascontiguousarray(a, dtype=dtype)
            if arr.ndim != 1:
                raise ValueError(f"{name} must be one-dimensional")
            return arr.ctypes.data, arr

        seeds_ptr, seeds_arr = as_ptr(seeds, np.uint64, "seeds")
        targets_ptr, targets_arr = as_ptr(targets, np.uint64, "targets")
        sizes = {len(a) for a in (seeds_arr, targets_arr) if a is not None}
        if ncells is not None:
            sizes.add(int(ncells))
        if len(sizes) != 1:
            raise ValueError(f"seeds, targets and ncells disagree on the number of cells: {sizes}")
        n = sizes.pop()
        missed = C.c_uint64(0)
        st = (abi.CellStats * n)() if stats else None
        if isinstance(band, np.ndarray):
            assert band.dtype == np.uint32 and band.flags["C_CONTIGUOUS"]
            band_ptr = band.ctypes.data
        else:
            band_ptr = band
        _check(self.lib.mgpu_simulate_cells(self.h, chrom_id, seeds_ptr, targets_ptr,
                                            target_epochs, nlefs, n, band_ptr,
                                            C.addressof(missed), C.addressof(st) if st else None),
               "mgpu_simulate_cells")
        return missed.value, st

    def simulate_cells_ex(self, chrom_id, seeds, targets, target_epochs, nlefs, band, occupancy=None,
                          max_epoch_records=0):
        """mgpu_simulate_cells_ex with host arrays: ``occupancy`` (uint64, ceil(size / bin)
        counters) is added to when the config tracks the 1D LEF occupancy; with
        ``max_epoch_records`` and log_model_internal_state the per-epoch model-state records are
        returned.  Returns (missed, stats, records) where records[i] lists cell i's records."""
        seeds = np.ascontiguousarray(seeds, dtype=np.uint64)
        targets = np.ascontiguousarray(targets, dtype=np.uint64)
        n = len(seeds)
        missed = C.c_uint64(0)
        st = (abi.CellStats * n)()
        ex = abi.ExtraOutputs()
        if occupancy is not None:
            assert occupancy.dtype == np.uint64 and occupancy.flags["C_CONTIGUOUS"]
            ex.lef_1d_occupancy = occupancy.ctypes.data
        recs = written = None
        if max_epoch_records:
            recs = (abi.EpochRecord * (n * max_epoch_records))()
            written = np.zeros(n, dtype=np.uint64)
            ex.epoch_records = C.addressof(recs)
            ex.max_epoch_records = max_epoch_records
            ex.records_written = written.ctypes.data
        _check(self.lib.mgpu_simulate_cells_ex(self.h, chrom_id, seeds.ctypes.data, targets.ctypes.data,
                                               target_epochs, nlefs, n, band.ctypes.data, C.addressof(missed),
                                               C.addressof(st), C.byref(ex)), "mgpu_simulate_cells_ex")
        out = None
        if recs is not None:
            out = [[recs[i * max_epoch_records + k] for k in range(int(written[i]))] for i in range(n)]
        return missed.value, st, out

    def simulate_batch(self, tasks, bands):
        """mgpu_simulate_batch.  ``tasks`` is a sequence of (chrom_id, seed, target_contacts,
        target_epochs, num_lefs); ``bands`` maps chrom_id to a host uint32 array or a device
        pointer.  Returns (missed per chrom_id, per-task stats)."""
        n = len(tasks)
        arr = (abi.BatchTask * n)()
        for i, (cid, seed, tc, te, nl) in enumerate(tasks):
            arr[i].chrom_id = cid
            arr[i].seed = int(seed)
            arr[i].target_contacts = int(tc)
            arr[i].target_epochs = int(te)
            arr[i].num_lefs = int(nl)
        nb = max(bands) + 1 if bands else 0
        ptrs = (C.c_void_p * max(nb, 1))()
        for cid, b in bands.items():
            if isinstance(b, np.ndarray):
                assert b.dtype == np.uint32 and b.flags["C_CONTIGUOUS"]
                ptrs[cid] = b.ctypes.data
            else:
                ptrs[cid] = b
        missed = np.zeros(max(nb, 1), dtype=np.uint64)
        st = (abi.CellStats * n)()
        _check(self.lib.mgpu_simulate_batch(self.h, arr, n, ptrs, nb, missed.ctypes.data, C.addressof(st)),
               "mgpu_simulate_batch")
        return {cid: int(missed[cid]) for cid in bands}, st

    def band_to_pixels(self, band, nrows, ncols, bin_offset=0):
        """mgpu_band_to_pixels on a host uint32 band: returns (bin1_offset, bin1, bin2, count)
        numpy arrays, the pixel table in the order a cooler file stores it."""
        band = np.ascontiguousarray(band, dtype=np.uint32)
        if band.size != nrows * ncols:
            raise ValueError("band must hold nrows * ncols counts")
        offs = np.zeros(ncols + 1, dtype=np.uint64)
        nnz = C.c_uint64()
        _check(self.lib.mgpu_band_to_pixels(self.h, band.ctypes.data, nrows, ncols, bin_offset, offs.ctypes.data,
                                            None, None, None, 0, C.byref(nnz)), "mgpu_band_to_pixels")
        n = nnz.value
        b1 = np.zeros(n, dtype=np.int64)
        b2 = np.zeros(n, dtype=np.int64)
        cnt = np.zeros(n, dtype=np.uint32)
        if n:
            _check(self.lib.mgpu_band_to_pixels(self.h, band.ctypes.data, nrows, ncols, bin_offset,
                                                offs.ctypes.data, b1.ctypes.data, b2.ctypes.data,
                                                cnt.ctypes.data, n, C.byref(nnz)), "mgpu_band_to_pixels")
        return offs, b1, b2, cnt

    def simulate_cells_noalloc(self, chrom_id, seeds_ptr, targets_ptr, target_epochs, nlefs, ncells,
                               band_ptr, missed_ptr=None, stats_ptr=None):
        """mgpu_simulate_cells_noalloc: every argument buffer is a device pointer (int); the
        work is only enqueued on the context's stream (call sync() before reading results)."""
        _check(self.lib.mgpu_simulate_cells_noalloc(self.h, chrom_id, seeds_ptr, targets_ptr, target_epochs,
                                                    nlefs, ncells, band_ptr, missed_ptr, stats_ptr),
               "mgpu_simulate_cells_noalloc")

    def trace_cell(self, chrom_id, seed, target, target_epochs, nlefs, max_records=0,
                   max_epochs=0, band=None):
        """Run one cell recording per-epoch state; returns (stats, headers, arrays, all_headers)."""
        tr = abi.TraceRequest()
        tr.max_records = max_records
        arrays = {}
        headers = (abi.TraceHeader * max(1, max_records))()
        if max_records:
            tr.headers = headers
            for name in abi.TRACE_ARRAYS:
                a = np.zeros(max_records * nlefs, dtype=np.uint64)
                arrays[name] = a
                setattr(tr, name, abi.ptr64(a))
        all_headers = (abi.TraceHeader * max(1, max_epochs))()
        if max_epochs:
            tr.max_epochs = max_epochs
            tr.all_headers = all_headers
        st = abi.CellStats()
        band_ptr = band.ctypes.data if isinstance(band, np.ndarray) else band
        _check(self.lib.mgpu_trace_cell(self.h, chrom_id, seed, target, target_epochs, nlefs,
                                        band_ptr, C.byref(st), C.byref(tr)), "mgpu_trace_cell")
        return st, headers, arrays, all_headers, tr.num_epochs_recorded

    def set_stream(self, stream_handle):
        """Launch on a caller's cudaStream_t (an int handle, e.g. torch's stream.cuda_stream)."""
        _check(self.lib.mgpu_set_stream(self.h, C.c_void_p(stream_handle)), "mgpu_set_stream")

    def sync(self):
        """mgpu_sync: wait for the work issued on the context's stream."""
        _check(self.lib.mgpu_sync(self.h), "mgpu_sync")

    def last_kernel_ms(self):
        ms = C.c_double()
        _check(self.lib.mgpu_last_kernel_ms(self.h, C.byref(ms)), "mgpu_last_kernel_ms")
        return ms.value

    def set_launch_table(self, entries):
        """Tuned settings of large batched launches: entries (max_lefs, smem_budget, carveout_pct,
        max_cells_per_sm) in increasing max_lefs; an empty list clears the table."""
        arr = (abi.LaunchSetting * max(1, len(entries)))()
        for i, (ml, sb, co, mx) in enumerate(entries):
            arr[i] = abi.LaunchSetting(int(ml), int(sb), int(co), int(mx))
        _check(self.lib.mgpu_set_launch_table(self.h, arr, len(entries)), "mgpu_set_launch_table")

    def set_debug_flags(self, flags=0, smem_budget=0):
        """Force the serial restatement of some steps (bit 0 rank, 1 adjust, 2 collisions,
        3 contacts), collect the step profile (bit 4), set the carveout (bits 8-15) and the
        cells-per-SM cap (bits 16-23), and/or cap a cell's shared memory (bytes, 0 = limit)."""
        _check(self.lib.mgpu_set_debug_flags(self.h, flags, smem_budget), "mgpu_set_debug_flags")

    PROFILE_NAMES = ("burnin", "bind", "rank", "contacts", "moves", "adjust", "barriers",
                     "boundaries", "lef_bar", "primary", "correct", "secondary", "fix",
                     "extrude_release", "trace", "total", "rank_fallbacks", "adjust_fallbacks",
                     "serial_chain_walks", "serial_contact_attempts", "fix_fallbacks", "refills",
                     "stale_refills", "epochs", "rank_pdq", "rank_pass", "rank_block",
                     "rank_merge", "rank_serial")

    def last_profile(self):
        buf = (C.c_uint64 * 32)()
        _check(self.lib.mgpu_last_profile(self.h, buf), "mgpu_last_profile")
        return {name: buf[i] for i, name in enumerate(self.PROFILE_NAMES)}

    def run_phase(self, chrom_id, phase, io):
        return self.lib.mgpu_run_phase(self.h, chrom_id, phase, C.byref(io))
