"""Host-side checks that need no GPU: the C ABI library loads and exports every symbol of
include/mgpu_modle.h, and its host logic (Config derivations, task targets, per-cell seeds,
barrier import and sort, integer thresholds) matches the oracle and the golden vectors."""

import ctypes as C
import json
import os
import re

import numpy as np
import pytest

from _harness import GOLDEN, ROOT, load_oracle, oracle_config
from modlefork_gb300 import _abi as abi
from modlefork_gb300 import build as mbuild
from modlefork_gb300 import engine


@pytest.fixture(scope="module")
def lib():
    mbuild.build()
    return engine.load()


def header_functions():
    text = open(os.path.join(ROOT, "include", "mgpu_modle.h")).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)  # declarations only, not comments
    return sorted(set(re.findall(r"\b(mgpu_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_header_symbol(lib):
    names = header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layouts_match_header(lib):
    # the ctypes mirror is used across the ABI; sizes must match the C compiler's layout
    assert C.sizeof(abi.Barrier) == 32
    assert C.sizeof(abi.CellStats) == 64
    assert C.sizeof(abi.TraceHeader) == 72
    assert C.sizeof(abi.EpochRecord) == 104
    assert C.sizeof(abi.ExtraOutputs) == 32
    assert lib.mgpu_abi_version() == 2


OVERRIDES = [
    {},
    dict(rev_extrusion_speed=2500, fwd_extrusion_speed=2500, rev_speed_set=1, fwd_speed_set=1,
         avg_lef_processivity=200000, barrier_occupied_stp=0.7, barrier_not_occupied_stp=0.7,
         probability_normalization_factor=5000),
    dict(rev_extrusion_speed=2500, fwd_extrusion_speed=2500, rev_speed_set=1, fwd_speed_set=1,
         barrier_occupied_stp=0.7, probability_normalization_factor=8000),
    dict(occupancy_set=1, extrusion_barrier_occupancy=0.9, probability_of_extrusion_unit_bypass=0.3,
         lef_bar_minor_collision_pblock=0.5, probability_normalization_factor=3000),
    dict(contact_sampling_strategy=abi.CS_LOOP, stop_on_epochs=1, burnin_speed_coefficient=1.5,
         fwd_extrusion_speed_std=3.0, rev_extrusion_speed_std=0.2, bin_size=1000),
    dict(contact_sampling_strategy=abi.CS_TAD | abi.CS_NOISIFY, normalize_probabilities=0),
]


@pytest.mark.parametrize("ov", OVERRIDES)
def test_config_transform_matches_oracle(lib, ov):
    want = oracle_config(ov, transform=True).as_dict()
    cfg = engine.config_defaults(**ov)
    engine.config_transform(cfg)
    got = cfg.as_dict()
    for k in want:
        a, b = want[k], got[k]
        if isinstance(a, float) and np.isnan(a):
            assert np.isnan(b), k
        else:
            assert a == b, (k, a, b)


@pytest.mark.parametrize("size", [10_000_000, 248_956_422, 1_000_001, 3])
@pytest.mark.parametrize("ncells", [1, 64, 512])
def test_task_targets_match_oracle(lib, size, ncells):
    ol = load_oracle()
    ocfg = oracle_config({"num_cells": 512}, transform=True)
    cfg = engine.config_transform(engine.config_defaults(num_cells=512))
    nl = engine.num_lefs(cfg, size)
    assert nl == ol.orc_num_lefs(C.byref(ocfg), size)
    t, e = engine.task_targets(cfg, size, nl, ncells)
    ot = (C.c_uint64 * ncells)()
    oe = C.c_uint64()
    ol.orc_task_targets(C.byref(ocfg), size, nl, ncells, ot, C.byref(oe))
    assert list(t) == list(ot) and e == oe.value


def test_cell_seed_matches_xxhash_vectors(lib):
    vecs = json.load(open(os.path.join(GOLDEN, "xxh3_vectors.json")))["vectors"]
    assert len(vecs) >= 1000
    for v in vecs:
        got = engine.cell_seed(v["name"], v["size"], v["seed"], v["cell"])
        assert got == v["hash"], v


def test_barrier_from_bed_midpoint_and_occupancy(lib):
    ch = engine.Chromosome("chr1", 1000, 100, 900)
    bars = engine.barriers_from_bed(ch, [(0, 50, "+", 0.0), (200, 201, "+", 0.0), (300, 303, "-", 0.9),
                                         (898, 900, "+", 0.0), (899, 900, "-", 0.0)], 0.7, 0.7)
    # (s + e + 1) / 2 with integer division; barriers outside [start, end) are dropped
    assert [b["pos"] for b in bars] == [201, 302, 899]
    assert [b["blocking_dir"] for b in bars] == [abi.DIR_REV, abi.DIR_FWD, abi.DIR_REV]
    ia = 1.0 - 0.7
    want = min(max(1.0 - (ia - 0.9 * ia) / 0.9, 0.0), 1.0)
    assert bars[1]["stp_active"] == want and bars[1]["stp_inactive"] == 0.7
    assert bars[0]["stp_active"] == 0.7


def test_sort_barriers_orders_positions(lib):
    rng = np.random.default_rng(0)
    pos = rng.permutation(5000)[:3000] * 7 + 11
    arr = abi.make_barriers([dict(pos=int(p), stp_active=0.1, stp_inactive=0.2, blocking_dir=1) for p in pos])
    assert lib.mgpu_sort_barriers(arr, len(pos)) == 0
    assert [arr[i].pos for i in range(len(pos))] == sorted(int(p) for p in pos)


def test_state_digest_matches_oracle(lib):
    ol = load_oracle()
    rng = np.random.default_rng(5)
    arrs = [rng.integers(0, 1 << 63, size=37, dtype=np.uint64) for _ in range(9)]
    ptrs = [a.ctypes.data_as(C.POINTER(C.c_uint64)) for a in arrs]
    assert lib.mgpu_state_digest(37, *ptrs) == ol.orc_state_digest(37, *ptrs)


def test_prng_seed_matches_oracle(lib):
    ol = load_oracle()
    a, b = (C.c_uint64 * 4)(), (C.c_uint64 * 4)()
    lib.mgpu_prng_seed(752741483, a)
    ol.orc_prng_seed(752741483, b)
    assert list(a) == list(b)


def test_engine_fails_loudly_without_device(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(engine.EngineError) as e:
        engine.Engine(engine.config_transform(engine.config_defaults()))
    assert e.value.code in (abi.MGPU_ERR_NO_DEVICE, abi.MGPU_ERR_CUDA)


def test_batched_windows_follow_the_workload_ranges(lib):
    from modlefork_gb300 import genome

    wins = genome.batched_windows(seed=21, nwindows=400, min_len=1_000_000, max_len=250_000_000, cells=4)
    sizes = np.array([w[1].size for w in wins], dtype=np.float64)
    assert sizes.min() >= 1_000_000 and sizes.max() <= 250_000_000
    # log-uniform: about half the windows below the geometric midpoint (~15.8 Mbp)
    assert 0.4 < float(np.mean(sizes < np.sqrt(1e6 * 250e6))) < 0.6
    bins = {int(w[0].bin_size) for w in wins}
    assert bins == {1000 * k for k in range(1, 11)}
    dens = np.array([w[0].number_of_lefs_per_mbp for w in wins])
    assert dens.min() >= 5.0 and dens.max() <= 40.0
    bden = np.array([len(w[2]) / (w[1].size / 1e6) for w in wins])
    assert bden.min() > 4.0 and bden.max() < 41.0
    for cfg, chrom, bars in wins[:5]:
        assert cfg.num_cells == 4 and np.isclose(cfg.rev_extrusion_speed, 0.8 * cfg.bin_size)


def test_launch_setting_layout_and_surrogate_library_exports():
    assert C.sizeof(abi.LaunchSetting) == 24
    from modlefork_gb300 import surrogate_ops

    slib = surrogate_ops.load()
    text = open(os.path.join(ROOT, "include", "mgpu_surrogate.h")).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    names = sorted(set(re.findall(r"\b(msur_[a-z0-9_]+)\s*\(", text)))
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(slib, n)]
    assert not missing, missing
    # argument checks that run before any device work
    with pytest.raises(surrogate_ops.SurrogateKernelError):
        surrogate_ops.conv_set_stages(96, 2)
    with pytest.raises(surrogate_ops.SurrogateKernelError):
        surrogate_ops.conv_set_stages(128, 5)
    for bn, default in ((64, 4), (128, 3), (256, 4)):
        assert surrogate_ops.conv_get_stages(bn) == default
        assert surrogate_ops.conv_get_form(bn) == surrogate_ops.FORM_STAGED
        assert surrogate_ops.conv_get_persistent(bn) == 0
    with pytest.raises(surrogate_ops.SurrogateKernelError):
        surrogate_ops.conv_set_persistent(32, 1)
    for bad in ((32, 0), (128, 4), (128, -1)):
        with pytest.raises(surrogate_ops.SurrogateKernelError):
            surrogate_ops.conv_set_form(*bad)
    # the persistent bit alone, then back
    surrogate_ops.conv_set_persistent(128, 1)
    assert surrogate_ops.conv_get_form(128) == 3 and surrogate_ops.conv_get_persistent(128) == 1
    surrogate_ops.conv_set_form(128, surrogate_ops.FORM_STAGED)
    assert surrogate_ops.conv_get_persistent(128) == 0


def test_fused_convolution_arguments_are_checked_before_device_work():
    """msur_conv_forward_fused refuses odd lengths for pooling, unaligned copies and short
    strides with MSUR_ERR_INVALID_ARG before it touches a device (fake aligned addresses)."""
    from modlefork_gb300 import surrogate_ops

    lib = surrogate_ops.load()
    X, W, OUT = 1 << 20, 2 << 20, 3 << 20  # 16-byte aligned, never dereferenced

    def call(L=128, out_skip=0, skip_stride=0, out_dup=0, dup_stride=0, out_pool=0, pool_stride=0):
        return lib.msur_conv_forward_fused(X, 2, L, 64, W, 64, 3, None, 1, None, 64, out_skip or None, skip_stride,
                                           out_dup or None, dup_stride, out_pool or None, pool_stride, 64, None)

    invalid = -1  # MSUR_ERR_INVALID_ARG
    assert call(L=127, out_pool=OUT, pool_stride=64) == invalid          # pooling needs an even L
    assert call(out_skip=OUT + 8, skip_stride=64) == invalid            # unaligned copy
    assert call(out_dup=OUT, dup_stride=60) == invalid                  # stride not a multiple of 8
    assert call(out_pool=OUT, pool_stride=32) == invalid                # stride below n_valid
    assert call() == invalid                                            # no output at all
