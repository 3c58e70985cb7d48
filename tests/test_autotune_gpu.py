"""Tuned launch settings change where a batched launch keeps its per-LEF arrays and how many
cells share an SM, never what the cells compute: a large batch gives the same bands and per-cell
results with and without a launch table, and the surrogate's convolutions give the same
outputs at every pipeline depth."""

import numpy as np
import pytest
import torch

from modlefork_gb300 import _abi as abi
from modlefork_gb300 import engine, genome
from modlefork_gb300 import surrogate_ops as ops

pytestmark = pytest.mark.gpu


def _key(s):
    return (s.epochs, s.burnin_epochs, s.contacts, s.missed_updates, s.lef_epochs, s.rng_draws, s.status)


def test_launch_table_keeps_batched_results():
    cfg, gen = genome.parity_10mbp(seed=4, stop_on_epochs=1, target_simulation_epochs=30)
    chrom, bars = gen[0]
    ncells = 8 * torch.cuda.get_device_properties(0).multi_processor_count + 16  # a "large" batch
    nl = engine.num_lefs(cfg, chrom.simulated_size)
    targets, te = engine.task_targets(cfg, chrom.simulated_size, nl, ncells)
    nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
    outs = []
    for table in (None, [(100, 8192, 80, 0), (1 << 40, 12288, 100, 4)], [(1 << 40, 1 << 30, 0, 0)]):
        with engine.Engine(cfg) as eng:
            if table:
                eng.set_launch_table(table)
            cid = eng.upload_chrom(chrom, bars)
            tasks = [(cid, engine.cell_seed(chrom.name, chrom.size, cfg.seed, i), int(targets[i]), te, nl)
                     for i in range(ncells)]
            band = np.zeros(nrows * ncols, dtype=np.uint32)
            missed, st = eng.simulate_batch(tasks, {cid: band})
            outs.append((band, missed[cid], [_key(s) for s in st]))
    for band, m, st in outs[1:]:
        assert np.array_equal(band, outs[0][0]) and m == outs[0][1] and st == outs[0][2]


def test_launch_table_is_validated():
    cfg, _ = genome.parity_10mbp()
    with engine.Engine(cfg) as eng:
        for bad in ([(100, 0, 0, 0), (50, 0, 0, 0)], [(100, 0, 101, 0)], [(100, 0, 0, 300)]):
            with pytest.raises(engine.EngineError) as e:
                eng.set_launch_table(bad)
            assert e.value.code == abi.MGPU_ERR_INVALID_ARG
        eng.set_launch_table([])  # clears


def test_conv_pipeline_depths_give_the_same_outputs():
    rng = np.random.default_rng(9)
    outs = {}
    for Cout in (64, 128, 256):
        x = torch.from_numpy(rng.standard_normal((2, 300, 128)).astype(np.float32)).to("cuda", torch.bfloat16)
        w = torch.from_numpy((rng.standard_normal((Cout, 3, 128)) / 20).astype(np.float32)).to("cuda", torch.bfloat16)
        bn = Cout if Cout < 256 else 256
        saved = ops.conv_get_stages(bn)
        try:
            for stages in (2, 3, 4):
                ops.conv_set_stages(bn, stages)
                y = torch.empty(2, 300, Cout, dtype=torch.float32, device="cuda")
                ops.conv_forward(x, w, out_f32=y)
                outs[(Cout, stages)] = y.cpu().numpy()
        finally:
            ops.conv_set_stages(bn, saved)
        for stages in (3, 4):
            assert np.array_equal(outs[(Cout, stages)], outs[(Cout, 2)])  # same MMA order: bit-identical
    torch.cuda.synchronize()
    assert ops.take_error() == 0
