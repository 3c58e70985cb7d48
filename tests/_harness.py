"""Shared helpers of the test-suite: loading the CPU oracle, building inputs, running the
reference's known-answer cases through either the oracle or the GPU library.

The oracle (oracle/modle_oracle.cpp) is test infrastructure: it is only loaded here, by
__graft_entry__.smoke() and by the CPU-baseline leg of bench.py.
"""

import ctypes as C
import json
import os
import subprocess

import numpy as np

from modlefork_gb300 import _abi as abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
U64MAX = (1 << 64) - 1

_oracle = None


def load_oracle():
    """Load (building first if needed) the CPU oracle library."""
    global _oracle
    if _oracle is not None:
        return _oracle
    if not os.path.exists(ORACLE_SO):
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    lib = C.CDLL(ORACLE_SO)
    P = C.POINTER
    lib.orc_config_defaults.argtypes = [P(abi.Config)]
    lib.orc_config_transform.argtypes = [P(abi.Config)]
    lib.orc_config_transform.restype = C.c_int
    lib.orc_num_lefs.argtypes = [P(abi.Config), C.c_uint64]
    lib.orc_num_lefs.restype = C.c_uint64
    lib.orc_contacts_per_epoch.argtypes = [P(abi.Config), C.c_uint64]
    lib.orc_contacts_per_epoch.restype = C.c_uint64
    lib.orc_task_targets.argtypes = [P(abi.Config), C.c_uint64, C.c_uint64, C.c_uint64,
                                     P(C.c_uint64), P(C.c_uint64)]
    lib.orc_task_targets.restype = C.c_int
    lib.orc_prng_seed.argtypes = [C.c_uint64, P(C.c_uint64)]
    lib.orc_prng_draws.argtypes = [C.c_uint64, C.c_uint64, P(C.c_uint64)]
    lib.orc_sample.argtypes = [C.c_uint64, C.c_int, C.c_uint64, C.c_uint64, C.c_double,
                               C.c_double, C.c_uint64, P(C.c_double)]
    lib.orc_sample.restype = C.c_uint64
    lib.orc_simulate_cell.argtypes = [P(abi.Config), P(abi.Chrom), P(abi.Barrier), C.c_uint64,
                                      C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64,
                                      P(C.c_uint32), P(abi.CellStats), P(abi.TraceRequest)]
    lib.orc_simulate_cell.restype = C.c_int
    lib.orc_simulate_cells_mt.argtypes = [P(abi.Config), P(abi.Chrom), P(abi.Barrier),
                                          C.c_uint64, P(C.c_uint64), P(C.c_uint64),
                                          C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64,
                                          P(C.c_uint32), P(C.c_uint64), P(abi.CellStats)]
    lib.orc_simulate_cells_mt.restype = C.c_int
    lib.orc_state_digest.argtypes = [C.c_uint64] + [P(C.c_uint64)] * 9
    lib.orc_state_digest.restype = C.c_uint64
    lib.orc_run_phase.argtypes = [P(abi.Config), P(abi.Chrom), P(abi.Barrier), C.c_uint64,
                                  C.c_int, P(abi.PhaseIO)]
    lib.orc_run_phase.restype = C.c_int
    lib.orc_simulate_cell_ex.argtypes = [P(abi.Config), P(abi.Chrom), P(abi.Barrier), C.c_uint64,
                                         C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64,
                                         P(C.c_uint32), P(abi.CellStats), P(abi.TraceRequest),
                                         C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64, P(C.c_uint64)]
    lib.orc_simulate_cell_ex.restype = C.c_int
    lib.orc_simulate_window_cell.argtypes = [P(abi.Config), P(abi.Chrom), C.c_uint64, C.c_uint64,
                                             P(abi.Barrier), C.c_uint64, C.c_uint64, C.c_uint64,
                                             C.c_uint64, C.c_uint64, P(C.c_uint32), P(abi.CellStats)]
    lib.orc_simulate_window_cell.restype = C.c_int
    lib.orc_band_to_pixels.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, P(C.c_uint64)]
    lib.orc_band_to_pixels.restype = C.c_int
    lib.orc_tie_counters.argtypes = [C.c_int, C.c_int, P(C.c_uint64)]
    lib.orc_tie_counters.restype = None
    lib.orc_band_shape.argtypes = [P(abi.Config), C.c_uint64, P(C.c_uint64), P(C.c_uint64)]
    lib.orc_band_shape.restype = None
    lib.orc_barrier_from_bed.argtypes = [P(abi.Chrom), C.c_uint64, C.c_uint64, C.c_char, C.c_double,
                                         C.c_double, C.c_double, P(abi.Barrier)]
    lib.orc_barrier_from_bed.restype = C.c_int
    lib.orc_xxh3_64.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, P(C.c_int)]
    lib.orc_xxh3_64.restype = C.c_uint64
    lib.orc_cell_seed.argtypes = [C.c_char_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64]
    lib.orc_cell_seed.restype = C.c_uint64
    lib.orc_libm_eval.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_uint64, C.c_double, C.c_double,
                                  C.c_double, C.c_void_p, C.c_uint64]
    lib.orc_libm_eval.restype = C.c_int
    lib.orc_sample_streams.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int, C.c_uint64, C.c_uint64,
                                       C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_uint64]
    lib.orc_sample_streams.restype = C.c_int
    _oracle = lib
    return lib


class OracleHelpers:
    """The host-side helpers of the engine's API (config defaults and transform, per-cell
    seeds, LEF counts, task targets, band shapes, BED barriers), answered by the oracle
    library alone.  ``modlefork_gb300.genome`` takes it as ``api=`` so that the CPU arm of the
    benchmark builds its workload without loading the product library."""

    def __init__(self):
        from modlefork_gb300.engine import Chromosome

        self.lib = load_oracle()
        self.Chromosome = Chromosome

    def config_defaults(self, **overrides):
        cfg = abi.Config()
        self.lib.orc_config_defaults(C.byref(cfg))
        for k, v in overrides.items():
            if not hasattr(cfg, k):
                raise KeyError(k)
            setattr(cfg, k, v)
        return cfg

    def config_transform(self, cfg):
        rc = self.lib.orc_config_transform(C.byref(cfg))
        if rc != 0:
            raise ValueError(f"orc_config_transform returned {rc}")
        return cfg

    def cell_seed(self, name, chrom_size, seed, cell_id):
        b = name.encode() if isinstance(name, str) else bytes(name)
        return self.lib.orc_cell_seed(b, len(b), chrom_size, seed, cell_id)

    def num_lefs(self, cfg, size_bp):
        return self.lib.orc_num_lefs(C.byref(cfg), size_bp)

    def band_shape(self, cfg, size_bp):
        nr, nc = C.c_uint64(), C.c_uint64()
        self.lib.orc_band_shape(C.byref(cfg), size_bp, C.byref(nr), C.byref(nc))
        return nr.value, nc.value

    def task_targets(self, cfg, size_bp, nlefs, ncells):
        t = np.zeros(ncells, dtype=np.uint64)
        e = C.c_uint64()
        rc = self.lib.orc_task_targets(C.byref(cfg), size_bp, nlefs, ncells,
                                       t.ctypes.data_as(C.POINTER(C.c_uint64)), C.byref(e))
        if rc != 0:
            raise ValueError(f"orc_task_targets returned {rc}")
        return t, e.value

    def barriers_from_bed(self, chrom, records, default_stp_active, default_stp_inactive):
        ch = chrom.as_abi()
        out = []
        b = abi.Barrier()
        for (s, e, strand, score) in records:
            rc = self.lib.orc_barrier_from_bed(C.byref(ch), s, e, strand.encode(), float(score),
                                               default_stp_active, default_stp_inactive, C.byref(b))
            if rc < 0:
                raise ValueError(f"orc_barrier_from_bed returned {rc}")
            if rc == 1:
                out.append(dict(pos=b.pos, stp_active=b.stp_active, stp_inactive=b.stp_inactive,
                                blocking_dir=b.blocking_dir))
        return out


def tie_counters(enable=False, reset=False):
    """Full-tie counters of the oracle's epoch-loop rank_lefs calls: (rank calls, calls with a
    full tie, full-tie pairs, pairs away from the chromosome ends).  Counting stays on after a
    call with ``enable`` true and is off otherwise."""
    lib = load_oracle()
    out = (C.c_uint64 * 4)()
    lib.orc_tie_counters(1 if enable else 0, 1 if reset else 0, out)
    return tuple(out)


def oracle_pixels(band, nrows, ncols, bin_offset=0):
    """The oracle's pixel table of a band: (bin1_offset, bin1, bin2, count)."""
    lib = load_oracle()
    band = np.ascontiguousarray(band, dtype=np.uint32)
    offs = np.zeros(ncols + 1, dtype=np.uint64)
    cap = int(np.count_nonzero(band))
    b1 = np.zeros(max(cap, 1), dtype=np.int64)
    b2 = np.zeros(max(cap, 1), dtype=np.int64)
    cnt = np.zeros(max(cap, 1), dtype=np.uint32)
    nnz = C.c_uint64()
    rc = lib.orc_band_to_pixels(band.ctypes.data, nrows, ncols, bin_offset, offs.ctypes.data, b1.ctypes.data,
                                b2.ctypes.data, cnt.ctypes.data, cap, C.byref(nnz))
    assert rc == 0
    n = nnz.value
    return offs, b1[:n], b2[:n], cnt[:n]


def random_band(rng, nrows, ncols, density=0.3):
    """A band with zeros outside the upper triangle's reachable rows, like a simulated one."""
    band = np.zeros((ncols, nrows), dtype=np.uint32)  # band[j, r] = column j, row r
    vals = rng.integers(1, 1000, size=band.shape, dtype=np.uint32)
    mask = rng.random(band.shape) < density
    band[mask] = vals[mask]
    band[np.arange(ncols)[:, None] < np.arange(nrows)[None, :]] = 0  # row r > column j is unused
    return band.reshape(-1)


def oracle_config(overrides=None, transform=False):
    lib = load_oracle()
    cfg = abi.Config()
    lib.orc_config_defaults(C.byref(cfg))
    for k, v in (overrides or {}).items():
        setattr(cfg, k, v)
    if transform:
        rc = lib.orc_config_transform(C.byref(cfg))
        assert rc == 0
    return cfg


def make_chrom(start, end, size=None, name=b"chr1"):
    ch = abi.Chrom()
    ch.name = name
    ch.name_len = len(name)
    ch.size = size if size is not None else end
    ch.start = start
    ch.end = end
    return ch


class PhaseState:
    """Numpy-backed state of one cell in the reference's encodings (mgpu_phase_io)."""

    def __init__(self, lefs, rev_ranks, fwd_ranks, rev_moves, fwd_moves, released=(),
                 barrier_states=None, seed=0, prng_state=None):
        n = len(lefs)
        self.n = n
        self.rev_pos = np.array([l[0] for l in lefs], dtype=np.uint64)
        self.fwd_pos = np.array([l[1] for l in lefs], dtype=np.uint64)
        self.binding_epoch = np.array([l[2] for l in lefs], dtype=np.uint64)
        for i in released:
            self.rev_pos[i] = U64MAX
            self.fwd_pos[i] = U64MAX
            self.binding_epoch[i] = U64MAX
        self.rev_rank = np.array(rev_ranks, dtype=np.uint64)
        self.fwd_rank = np.array(fwd_ranks, dtype=np.uint64)
        self.rev_move = np.array(rev_moves, dtype=np.uint64)
        self.fwd_move = np.array(fwd_moves, dtype=np.uint64)
        self.rev_collision = np.zeros(n, dtype=np.uint64)
        self.fwd_collision = np.zeros(n, dtype=np.uint64)
        self.bind_mask = None
        self.barrier_state = (np.array(barrier_states, dtype=np.uint8)
                              if barrier_states is not None else None)
        self.prng = (list(prng_state) if prng_state is not None
                     else list(prng_state_from_seed(seed)))
        self.n5 = self.n3 = self.released = 0

    def io(self, **kw):
        io = abi.PhaseIO()
        io.num_lefs = self.n
        for name in abi.TRACE_ARRAYS:
            setattr(io, name, abi.ptr64(getattr(self, name)))
        io.bind_mask = abi.ptr64(self.bind_mask)
        if self.barrier_state is not None:
            io.barrier_state = self.barrier_state.ctypes.data_as(C.POINTER(C.c_uint8))
        for k, v in kw.items():
            setattr(io, k, v)
        for k in range(4):
            io.prng_state[k] = self.prng[k]
        return io

    def absorb(self, io):
        self.prng = [io.prng_state[k] for k in range(4)]
        self.n5, self.n3, self.released = io.n5prime, io.n3prime, io.lefs_released


def prng_state_from_seed(seed):
    lib = load_oracle()
    st = (C.c_uint64 * 4)()
    lib.orc_prng_seed(C.c_uint64(seed), st)
    return [st[i] for i in range(4)]


def load_golden_cases():
    with open(os.path.join(GOLDEN, "reference_unit_tests.json")) as f:
        return json.load(f)["cases"]


def golden_inputs(case):
    """(config overrides, chromosome, barrier dicts, PhaseState) of one golden case."""
    chrom = case["chrom"] or {"start": 0, "end": (1 << 32) - 2, "size": (1 << 32) - 2}
    st = PhaseState(case["lefs"], case["rev_ranks"], case["fwd_ranks"], case["rev_moves"],
                    case["fwd_moves"], case["released"],
                    [b["state"] for b in case["barriers"]], seed=case["seed"])
    return case["config"], chrom, case["barriers"], st


def run_golden_case(case, run_phase):
    """Run the hooks of a golden case through ``run_phase(phase_id, io) -> status``."""
    _, _, _, st = golden_inputs(case)
    for step in case["steps"]:
        kw = {}
        if step["hook"] == "RANK":
            kw = dict(ranks_partially_sorted=step.get("partially_sorted", 1),
                      init_ranks=step.get("init_ranks", 0))
        io = st.io(**kw)
        rc = run_phase(abi.PHASES[step["hook"]], io)
        assert rc == 0, f"{case['name']}: {step['hook']} returned {rc}"
        st.absorb(io)
    return st


def check_golden(case, st):
    exp = case["expected"]
    out = {"rev_moves": st.rev_move, "fwd_moves": st.fwd_move,
           "rev_collisions": st.rev_collision, "fwd_collisions": st.fwd_collision,
           "rev_ranks": st.rev_rank, "fwd_ranks": st.fwd_rank}
    for key, want in exp.items():
        got = [int(x) for x in out[key]]
        assert got == [int(x) for x in want], f"{case['name']} {key}: got {got} want {want}"


def host_libm(kind, x, y=None, mu=0.0, sigma=0.0, xi=0.0, threads=None):
    """glibc's log / exp / pow / GEV noise / x < exp(y) through the oracle (the host side of
    the device's mgpu_probe_libm)."""
    lib = load_oracle()
    x = np.ascontiguousarray(x, dtype=np.float64)
    yp = None
    if y is not None:
        y = np.ascontiguousarray(y, dtype=np.float64)
        yp = y.ctypes.data
    out = np.empty_like(x)
    rc = lib.orc_libm_eval(kind, x.ctypes.data, yp, len(x), mu, sigma, xi, out.ctypes.data,
                           threads or os.cpu_count() or 1)
    assert rc == 0
    return out


# orc_sample kinds for the device probe kinds (engine.PROBE_*)
ORACLE_SAMPLE_KIND = {0: 4, 1: 8, 2: 5, 3: 6, 4: 6, 5: 7}


def host_samplers(probe_kind, seeds, per_stream, a0=0.0, a1=0.0, threads=None):
    """The oracle's samplers (glibc) on the same seeded streams as engine.probe_samplers."""
    lib = load_oracle()
    seeds = np.ascontiguousarray(seeds, dtype=np.uint64)
    out = np.empty((len(seeds), per_stream), dtype=np.float64)
    draws = np.empty(len(seeds), dtype=np.uint64)
    kind = ORACLE_SAMPLE_KIND[probe_kind]
    if kind == 6:  # binomial(t = a, p)
        a, b, p, q = int(a0), 0, a1, 0.0
    else:  # normal(p, q), poisson(p), gev(0, p, q), exponential
        a, b, p, q = 0, 0, a0, a1
    rc = lib.orc_sample_streams(seeds.ctypes.data, len(seeds), per_stream, kind, a, b, p, q, out.ctypes.data,
                                draws.ctypes.data, threads or os.cpu_count() or 1)
    assert rc == 0
    return out, draws
