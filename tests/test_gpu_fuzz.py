"""Randomised parity: seeded random configurations and chromosomes, one whole cell each, GPU
against the oracle at every epoch (state digest, draws, counters, band).

The parameters cover the reference's option space around its defaults: LEF density and
lifetime, extrusion speeds and their spread, barrier stps and occupancy, bypass and block
probabilities, the contact sampling strategy and GEV noise, bin size and band width, burn-in
settings and the stopping criterion, chromosome offsets and the optional outputs.
"""

import numpy as np
import pytest

from modlefork_gb300 import _abi as abi
from modlefork_gb300 import engine

from test_gpu_parity import compare_cell, small_genome

pytestmark = pytest.mark.gpu

NCASES = 48


def random_case(k):
    rng = np.random.default_rng(1000 + k)
    speed = int(rng.integers(500, 6000))
    ov = dict(
        bin_size=int(rng.choice([1000, 2000, 5000, 10000])),
        number_of_lefs_per_mbp=float(rng.uniform(5, 60)),
        avg_lef_processivity=int(rng.integers(50_000, 500_000)),
        rev_extrusion_speed=speed, fwd_extrusion_speed=int(speed * rng.uniform(0.5, 1.5)),
        rev_speed_set=1, fwd_speed_set=1,
        rev_extrusion_speed_std=float(rng.choice([0.0, 0.05, 0.2, 30.0])),
        fwd_extrusion_speed_std=float(rng.choice([0.0, 0.05, 0.3])),
        barrier_occupied_stp=float(rng.uniform(0.3, 0.95)),
        barrier_not_occupied_stp=float(rng.uniform(0.3, 0.95)),
        probability_of_extrusion_unit_bypass=float(rng.uniform(0.0, 0.5)),
        lef_bar_major_collision_pblock=float(rng.uniform(0.5, 1.0)),
        lef_bar_minor_collision_pblock=float(rng.uniform(0.0, 0.5)),
        hard_stall_lef_stability_multiplier=float(rng.uniform(1.0, 8.0)),
        soft_stall_lef_stability_multiplier=float(rng.uniform(0.5, 2.0)),
        contact_sampling_strategy=int(rng.choice([abi.CS_LOOP | abi.CS_TAD | abi.CS_NOISIFY,
                                                  abi.CS_LOOP | abi.CS_NOISIFY, abi.CS_TAD,
                                                  abi.CS_LOOP | abi.CS_TAD])),
        tad_to_loop_contact_ratio=float(rng.choice([0.0, 1.0, 5.0, 20.0])),
        genextreme_mu=float(rng.uniform(-2000, 2000)), genextreme_sigma=float(rng.uniform(100, 10000)),
        genextreme_xi=float(rng.choice([0.0, 0.001, 0.1, -0.1])),
        probability_normalization_factor=int(rng.integers(2000, 12000)),
        # the default burn-in window; a cap keeps the burn-in finite whatever the draws
        max_burnin_epochs=int(rng.integers(500, 3000)),
        contact_sampling_interval=int(rng.integers(20_000, 100_000)),
        target_contact_density=float(rng.uniform(0.2, 2.0)),
        track_1d_lef_position=int(rng.random() < 0.3),
        seed=int(rng.integers(1, 1 << 40)),
    )
    ov["diagonal_width"] = int(ov["bin_size"] * rng.integers(20, 400))
    if rng.random() < 0.2:
        ov.update(stop_on_epochs=1, target_simulation_epochs=int(rng.integers(50, 400)), target_contact_density=-1.0)
    if rng.random() < 0.2:
        ov["skip_burnin"] = 1
    length = int(rng.integers(1_000_000, 4_000_000))
    nbar = int(rng.integers(0, max(1, length // 20_000)))
    start = int(rng.choice([0, 0, 777_777]))
    occ = "beta" if rng.random() < 0.5 else None
    return ov, length, nbar, start, occ, int(rng.integers(0, 50))


@pytest.mark.parametrize("k", range(NCASES))
def test_random_configuration(k):
    ov, length, nbar, start, occ, cell = random_case(k)
    cfg = engine.config_defaults(num_cells=32)
    for key, v in ov.items():
        setattr(cfg, key, v)
    engine.config_transform(cfg)
    chrom, bars = small_genome(cfg, length, nbar, seed=k, occupancy=occ, start=start)
    nl = engine.num_lefs(cfg, chrom.simulated_size)
    if nl == 0:
        pytest.skip("no LEFs")
    compare_cell(cfg, chrom, bars, cell_id=cell, max_epochs=60_000, mode="fast" if k % 3 else "global_scratch")
