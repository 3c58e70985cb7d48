"""mgpu_band_to_pixels against the oracle's restatement of the cooler writer's pixel loop."""

import ctypes as C

import numpy as np
import pytest

from _harness import oracle_pixels, random_band
from modlefork_gb300 import _abi as abi
from modlefork_gb300 import engine, genome

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nrows,ncols,density", [(600, 2000, 0.3), (7, 5, 0.9), (1, 50, 0.5),
                                                 (50, 1, 1.0), (16, 16, 0.0), (3, 0, 0.5),
                                                 (600, 50000, 0.02), (33, 1000, 1.0)])
def test_pixels_match_oracle(nrows, ncols, density):
    rng = np.random.default_rng(nrows * 7 + ncols)
    band = random_band(rng, nrows, ncols, density)
    cfg = genome.parity_config()
    with engine.Engine(cfg) as eng:
        got = eng.band_to_pixels(band, nrows, ncols, bin_offset=777)
    want = oracle_pixels(band, nrows, ncols, bin_offset=777)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_pixels_of_a_simulated_band_device_buffers():
    """A simulated band through device pointers gives the oracle's table; a short capacity is
    an overflow error that still reports the size."""
    torch = pytest.importorskip("torch")
    cfg, gen = genome.parity_10mbp(seed=9)
    chrom, bars = gen[0]
    nl = engine.num_lefs(cfg, chrom.simulated_size)
    targets, te = engine.task_targets(cfg, chrom.simulated_size, nl, 8)
    seeds = np.arange(8, dtype=np.uint64) + 5
    nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
    band = np.zeros(nrows * ncols, dtype=np.uint32)
    with engine.Engine(cfg) as eng:
        cid = eng.upload_chrom(chrom, bars)
        eng.simulate_cells(cid, seeds, targets, te, nl, band)
        want = oracle_pixels(band, nrows, ncols, bin_offset=3)
        n = len(want[1])
        dev = torch.device("cuda", 0)
        d_band = torch.from_numpy(band.view(np.int32)).to(dev)
        d_off = torch.zeros(ncols + 1, dtype=torch.int64, device=dev)
        d_b1 = torch.zeros(n, dtype=torch.int64, device=dev)
        d_b2 = torch.zeros(n, dtype=torch.int64, device=dev)
        d_c = torch.zeros(n, dtype=torch.int32, device=dev)
        nnz = C.c_uint64()
        lib = eng.lib
        with pytest.raises(engine.EngineError) as e:
            engine._check(lib.mgpu_band_to_pixels(eng.h, d_band.data_ptr(), nrows, ncols, 3, d_off.data_ptr(),
                                                  d_b1.data_ptr(), d_b2.data_ptr(), d_c.data_ptr(), n - 1,
                                                  C.byref(nnz)))
        assert e.value.code == abi.MGPU_ERR_OVERFLOW and nnz.value == n
        engine._check(lib.mgpu_band_to_pixels(eng.h, d_band.data_ptr(), nrows, ncols, 3, d_off.data_ptr(),
                                              d_b1.data_ptr(), d_b2.data_ptr(), d_c.data_ptr(), n, C.byref(nnz)))
    torch.cuda.synchronize()
    assert nnz.value == n
    assert np.array_equal(d_off.cpu().numpy().view(np.uint64), want[0])
    assert np.array_equal(d_b1.cpu().numpy(), want[1])
    assert np.array_equal(d_b2.cpu().numpy(), want[2])
    assert np.array_equal(d_c.cpu().numpy().view(np.uint32), want[3])
    assert int(want[3].sum(dtype=np.uint64)) == int(band.sum(dtype=np.uint64))


def test_genome_pixel_table_offsets():
    """Bins are numbered across the genome: each chromosome's pixels carry its first bin, and the
    genome table is the chromosomes' tables in order."""
    from modlefork_gb300 import simulate

    cfg, gen = genome.genome_24chr(seed=5, nchroms=3, min_len=2_000_000, max_len=4_000_000)
    cfg.num_cells = 4
    res = simulate.simulate_genome(cfg, gen)
    b1, b2, cnt = simulate.genome_pixels(cfg, res, [c for c, _ in gen])
    first, parts = 0, []
    for r in res:
        nrows, ncols = engine.band_shape(cfg, r.chrom.simulated_size)
        parts.append(oracle_pixels(r.band, nrows, ncols, bin_offset=first))
        first += (r.chrom.size + cfg.bin_size - 1) // cfg.bin_size
    assert np.array_equal(b1, np.concatenate([p[1] for p in parts]))
    assert np.array_equal(b2, np.concatenate([p[2] for p in parts]))
    assert np.array_equal(cnt, np.concatenate([p[3] for p in parts]))
    assert np.all(np.diff(b1) >= 0) and np.all(b2 >= b1)
