"""The CPU oracle against the reference's own known-answer tests (test/units/simulation_cpu),
extracted verbatim into tests/golden/reference_unit_tests.json by tests/golden/gen_golden.py.

These pin the oracle before it is used to check the GPU kernels.
"""

import ctypes as C

import numpy as np
import pytest

from modlefork_gb300 import _abi as abi
from _harness import (check_golden, golden_inputs, load_golden_cases, load_oracle, make_chrom,
                      oracle_config, run_golden_case)

CASES = load_golden_cases()


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_reference_unit_test(case):
    lib = load_oracle()
    overrides, chrom, barriers, _ = golden_inputs(case)
    cfg = oracle_config(overrides)
    ch = make_chrom(chrom["start"], chrom["end"], chrom["size"])
    bs = abi.make_barriers(barriers)

    def run_phase(phase, io):
        return lib.orc_run_phase(C.byref(cfg), C.byref(ch), bs, len(barriers), phase, C.byref(io))

    st = run_golden_case(case, run_phase)
    check_golden(case, st)


def test_golden_fixture_is_complete():
    # 2 adjust + 4 LEF-LEF + 5 LEF-BAR + 4 ranking + 12 end-to-end process_collisions cases
    assert len(CASES) == 27
    assert sum(1 for c in CASES if c["seed"] == 752741483) == 2  # the seed-pinned cases


def _barrier_occupancy(sa, si):
    lib = load_oracle()
    # occupancy is exercised through BARRIER_INIT; here the closed form of
    # compute_occupancy_from_stp (extrusion_barriers_impl.hpp:118-128) is checked directly
    if sa + si == 0:
        return 0.0
    a, b = 1.0 - si, 1.0 - sa
    return min(max(a / (a + b), 0.0), 1.0)


def test_barrier_occupancy_known_answers():
    # "Extrusion barriers - compute_occupancy" (extrusion_barriers_test.cpp:64-94)
    assert _barrier_occupancy(1.0, 0.0) == 1.0
    assert _barrier_occupancy(0.0, 1.0) == 0.0
    assert _barrier_occupancy(0.7, 0.7) == 0.5
    assert _barrier_occupancy(0.7, 0.5) == pytest.approx(0.625)
    assert _barrier_occupancy(1.0, 0.5) == 1.0
    assert _barrier_occupancy(0.7, 1.0) == 0.0


def test_config_transform_config1():
    """Cli::transform_args on the 10 Mbp parity workload (normalisation factor 5000)."""
    cfg = oracle_config(dict(bin_size=5000, rev_extrusion_speed=2500, fwd_extrusion_speed=2500,
                             rev_speed_set=1, fwd_speed_set=1, rev_extrusion_speed_std=0.05,
                             fwd_extrusion_speed_std=0.05, avg_lef_processivity=200000,
                             barrier_occupied_stp=0.7, barrier_not_occupied_stp=0.7,
                             probability_normalization_factor=5000), transform=True)
    assert cfg.rev_extrusion_speed_std == 0.05 * 2500
    assert cfg.prob_of_lef_release == 5000 / 200000
    assert cfg.burnin_target_epochs_for_lef_activation == 200
    assert cfg.barrier_not_occupied_stp == 0.7
    assert cfg.extrusion_barrier_occupancy == 0.5
    assert cfg.probability_of_extrusion_unit_bypass == 0.1


def test_config_transform_normalisation():
    """Default normalisation factor 8000 vs speed 5000 rescales stps (cli.cpp:1138-1167)."""
    cfg = oracle_config(dict(bin_size=5000, rev_extrusion_speed=2500, fwd_extrusion_speed=2500,
                             rev_speed_set=1, fwd_speed_set=1, barrier_occupied_stp=0.7,
                             barrier_not_occupied_stp=0.7,
                             probability_normalization_factor=8000), transform=True)
    ratio = 5000 / 8000
    assert cfg.barrier_not_occupied_stp == np.exp(np.log(0.7) * ratio)
    assert cfg.probability_of_extrusion_unit_bypass == min(0.1 * ratio, 1.0)
    assert cfg.lef_bar_major_collision_pblock == 1.0
    assert cfg.lef_bar_minor_collision_pblock == 0.0


def test_prng_matches_published_xoshiro_splitmix():
    """SplitMix64 + Xoshiro256++ from their published definitions (pure-Python restatement)."""
    lib = load_oracle()
    M = (1 << 64) - 1

    def splitmix(state):
        state = (state + 0x9E3779B97F4A7C15) & M
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return state, z ^ (z >> 31)

    def rotl(x, k):
        return ((x << k) | (x >> (64 - k))) & M

    seed = 10556020843759504871
    s, st = [], seed
    for _ in range(4):
        st, z = splitmix(st)
        s.append(z)
    want = []
    for _ in range(64):
        want.append((rotl((s[0] + s[3]) & M, 23) + s[0]) & M)
        t = (s[1] << 17) & M
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = rotl(s[3], 45)
    got = (C.c_uint64 * 64)()
    lib.orc_prng_draws(C.c_uint64(seed), 64, got)
    assert list(got) == want


@pytest.mark.parametrize("kind,a,b,p,q", [
    (0, 0, 9, 0, 0), (0, 1000, 1999, 0, 0), (1, 0, 0, 0.3, 0), (2, 0, 0, 0, 0), (3, 0, 0, 0, 0),
    (4, 0, 0, 2500.0, 125.0), (5, 0, 0, 1.0, 0), (5, 0, 0, 40.0, 0), (6, 20, 0, 1 / 6, 0),
    (6, 800, 0, 1 / 6, 0), (7, 0, 0, 5000.0, 0.001), (8, 0, 0, 0, 0)])
def test_distribution_moments(kind, a, b, p, q):
    """Each restated Boost.Random distribution has the right first two moments."""
    lib = load_oracle()
    n = 200000
    out = np.zeros(n, dtype=np.float64)
    draws = lib.orc_sample(C.c_uint64(12345), kind, a, b, p, q, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    assert draws >= n or kind == 1 and p == 0
    mean, var = out.mean(), out.var()
    if kind == 0:
        assert out.min() >= a and out.max() <= b
        assert mean == pytest.approx((a + b) / 2, rel=0.01)
    elif kind == 1:
        assert mean == pytest.approx(p, abs=0.01)
    elif kind in (2, 3):
        assert 0 <= out.min() and out.max() < 1
        assert mean == pytest.approx(0.5, abs=0.01)
        assert var == pytest.approx(1 / 12, rel=0.02)
    elif kind == 4:
        assert mean == pytest.approx(p, abs=1.0)
        assert np.sqrt(var) == pytest.approx(q, rel=0.01)
        assert draws / n < 1.06  # ziggurat: one draw, plus one per wedge test (~2 %)
    elif kind == 5:
        assert mean == pytest.approx(p, rel=0.01)
        assert var == pytest.approx(p, rel=0.03)
    elif kind == 6:
        assert mean == pytest.approx(a * p, rel=0.01)
        assert var == pytest.approx(a * p * (1 - p), rel=0.03)
    elif kind == 7:
        # GEV(0, sigma, xi): mean = sigma * (Gamma(1 - xi) - 1) / xi ~ sigma * 0.5772
        assert mean == pytest.approx(p * 0.5772, rel=0.03)
    elif kind == 8:
        assert mean == pytest.approx(1.0, rel=0.01)
        assert var == pytest.approx(1.0, rel=0.03)


def test_normal_tail_and_wedge_paths_are_exercised():
    """Enough normal samples to walk through the ziggurat tail and wedges; the draw count
    exceeds the sample count by the wedge-test rate of the 128-layer ziggurat."""
    lib = load_oracle()
    n = 1_000_000
    out = np.zeros(n, dtype=np.float64)
    draws = lib.orc_sample(C.c_uint64(99), 4, 0, 0, 0.0, 1.0, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    assert np.abs(out).max() > 3.44  # beyond the tail start x_1
    assert 1.01 < draws / n < 1.06


# ---- the oracle's own host helpers (used by the CPU arm instead of the product library) ----

def test_oracle_cell_seed_matches_xxhash_vectors():
    import json
    import os

    from _harness import GOLDEN, OracleHelpers

    h = OracleHelpers()
    vecs = json.load(open(os.path.join(GOLDEN, "xxh3_vectors.json")))["vectors"]
    assert len(vecs) >= 1000
    for v in vecs:
        assert h.cell_seed(v["name"], v["size"], v["seed"], v["cell"]) == v["hash"], v


def test_oracle_xxh3_every_short_length_matches_the_engine():
    """Every input length the restatement covers (0..240 bytes) against the engine's own hash,
    itself pinned by the xxHash vectors above; longer inputs are refused."""
    from modlefork_gb300 import engine

    lib = load_oracle()
    elib = engine.load()
    rng = np.random.default_rng(5)
    ok = C.c_int()
    for n in range(0, 241):
        buf = rng.integers(0, 256, size=max(n, 1), dtype=np.uint8)
        seed = int(rng.integers(0, 2**63))
        got = lib.orc_xxh3_64(buf.ctypes.data, n, seed, C.byref(ok))
        assert ok.value == 1
        assert got == elib.mgpu_xxh3_64(buf.ctypes.data, n, seed), n
    buf = np.zeros(241, dtype=np.uint8)
    lib.orc_xxh3_64(buf.ctypes.data, 241, 0, C.byref(ok))
    assert ok.value == 0


def test_oracle_helpers_build_the_genome_workload_like_the_engine():
    from _harness import OracleHelpers
    from modlefork_gb300 import engine, genome

    h = OracleHelpers()
    cfg_o, gen_o = genome.genome_24chr(seed=11, nchroms=4, api=h)
    cfg_e, gen_e = genome.genome_24chr(seed=11, nchroms=4)
    assert bytes(cfg_o) == bytes(cfg_e)
    for (co, bo), (ce, be) in zip(gen_o, gen_e):
        assert bo == be
        size = co.simulated_size
        assert h.band_shape(cfg_o, size) == engine.band_shape(cfg_e, size)
        nl = h.num_lefs(cfg_o, size)
        assert nl == engine.num_lefs(cfg_e, size)
        to, eo = h.task_targets(cfg_o, size, nl, 7)
        te, ee = engine.task_targets(cfg_e, size, nl, 7)
        assert list(to) == list(te) and eo == ee
        for cell in (0, 1, 511):
            assert h.cell_seed(co.name, co.size, cfg_o.seed, cell) == engine.cell_seed(ce.name, ce.size,
                                                                                       cfg_e.seed, cell)
    ch = engine.Chromosome("chr1", 1000, 100, 900)
    recs = [(0, 50, "+", 0.0), (200, 201, "+", 0.0), (300, 303, "-", 0.9), (898, 900, "+", 0.0),
            (899, 900, "-", 0.0)]
    assert h.barriers_from_bed(ch, recs, 0.7, 0.7) == engine.barriers_from_bed(ch, recs, 0.7, 0.7)


def test_full_tie_counter_counts_rank_calls_and_ties():
    """Full ties (same position and binding epoch) are what the reference's tests leave unpinned
    in the ranking; the oracle counts them per epoch-loop rank call.  On the parity workload
    they appear in about 1 % of epochs, almost all of them units parked at a chromosome end."""
    from _harness import OracleHelpers, tie_counters
    from modlefork_gb300 import genome

    h = OracleHelpers()
    lib = load_oracle()
    cfg, gen = genome.parity_10mbp(seed=7, api=h)
    chrom, bars = gen[0]
    nl = h.num_lefs(cfg, chrom.simulated_size)
    targets, te = h.task_targets(cfg, chrom.simulated_size, nl, 64)
    nr, nc = h.band_shape(cfg, chrom.simulated_size)
    ch = make_chrom(chrom.start, chrom.end, chrom.size, chrom.name.encode())
    bs = abi.make_barriers(bars)

    def run(cells):
        seeds = np.array([h.cell_seed(chrom.name, chrom.size, cfg.seed, i) for i in range(cells)],
                         dtype=np.uint64)
        band = np.zeros(nr * nc, dtype=np.uint32)
        st = (abi.CellStats * cells)()
        missed = C.c_uint64()
        rc = lib.orc_simulate_cells_mt(C.byref(cfg), C.byref(ch), bs, len(bars),
                                       seeds.ctypes.data_as(C.POINTER(C.c_uint64)),
                                       targets.ctypes.data_as(C.POINTER(C.c_uint64)), te, nl, cells, 4,
                                       band.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(missed), st)
        assert rc == 0
        return sum(s.epochs for s in st)

    tie_counters(enable=False, reset=True)
    run(2)
    assert tie_counters() == (0, 0, 0, 0)  # off: nothing counted
    tie_counters(enable=True, reset=True)
    epochs = run(16)
    calls, tied, pairs, interior = tie_counters()
    assert calls >= epochs  # one rank call per epoch (plus the first binding)
    assert 0 < tied <= pairs and interior <= pairs
    assert tied < 0.05 * calls
