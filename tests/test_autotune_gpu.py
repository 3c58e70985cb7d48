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


@pytest.mark.parametrize("Cout,gated", [(64, False), (128, True), (256, False), (640, False), (384, True)])
def test_conv_kernel_forms_and_depths_give_the_same_outputs(Cout, gated):
    """The one-CTA-per-tile and the persistent kernel, with per-thread or staged (shared memory
    and TMA store) epilogues, at every pipeline depth, give bit-identical results (each tile's
    MMAs run in the same order); the default form is checked against FP64 in
    test_surrogate_kernels_gpu.py.  Shapes cover several tiles per CTA, ragged position tiles
    (rows past the sequence end, which the TMA stores drop), several sequences and the SiLU gate
    of the data gradient (which always takes the per-thread epilogue)."""
    rng = np.random.default_rng(Cout)
    B, L, Cin = 3, 1000, 128
    x = torch.from_numpy(rng.standard_normal((B, L, Cin)).astype(np.float32)).to("cuda", torch.bfloat16)
    w = torch.from_numpy((rng.standard_normal((Cout, 3, Cin)) / 20).astype(np.float32)).to("cuda", torch.bfloat16)
    bias = torch.from_numpy(rng.standard_normal(Cout).astype(np.float32)).to("cuda")
    gate = (torch.from_numpy(rng.standard_normal((B, L, Cout)).astype(np.float32)).to("cuda", torch.bfloat16)
            if gated else None)
    bn = 64 if Cout <= 64 else (256 if Cout % 256 == 0 else 128)
    saved = (ops.conv_get_stages(bn), ops.conv_get_form(bn))
    outs = {}
    try:
        for form in (0, 1, 2, 3):
            for stages in (2, 3, 4):
                ops.conv_set_form(bn, form)
                ops.conv_set_stages(bn, stages)
                y = torch.full((B, L, Cout), 7.0, dtype=torch.float32, device="cuda")
                pre = torch.full((B, L, Cout), 7.0, dtype=torch.bfloat16, device="cuda")
                post = torch.full((B, L, Cout), 7.0, dtype=torch.bfloat16, device="cuda")
                ops.conv_forward(x, w, bias=bias, act=ops.ACT_SILU, out_f32=y, out_pre=pre, out_post=post,
                                 gate=gate)
                outs[(form, stages)] = (y.cpu().numpy(), pre.float().cpu().numpy(), post.float().cpu().numpy())
    finally:
        ops.conv_set_stages(bn, saved[0])
        ops.conv_set_form(bn, saved[1])
    torch.cuda.synchronize()
    assert ops.take_error() == 0
    want = outs[(0, 2)]
    for k, got in outs.items():
        assert all(np.array_equal(g, w_) for g, w_ in zip(got, want)), k
