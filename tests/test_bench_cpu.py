"""bench.py's parts that need no GPU: the reference arm (the oracle on the host cores), its
rank handling under torchrun, the algorithmic-bytes model and the committed traffic figures."""

import json
import os
import subprocess
import sys
from types import SimpleNamespace

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _run(args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, env=e,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_contract_line():
    p = _run(["--impl", "reference", "--steps", "1", "--warmup", "0", "--cpu-seconds", "1"])
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "LEF-epochs/s" and d["unit"] == "LEF-epochs/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "LEF-epochs/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["workload"] == bench.WORKLOAD


def test_reference_arm_other_ranks_exit_quietly():
    p = _run(["--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"],
             env={"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"})
    assert p.returncode == 0 and p.stdout.strip() == ""


def test_algorithmic_bytes_model():
    stats = [SimpleNamespace(lef_epochs=100, epochs=10, contacts=7), SimpleNamespace(lef_epochs=50, epochs=5, contacts=1)]
    # 24 B per LEF-epoch, 6 B per barrier-epoch, 8 B per contact
    assert bench.algorithmic_bytes(stats, 3) == 24 * 150 + 6 * 3 * 15 + 8 * 8


@pytest.mark.parametrize("kernel", ["simulate_kernel", "simulate_batch_kernel"])
def test_committed_traffic_figures(kernel):
    traffic, d = bench.dram_traffic_per_launch(1_000_000.0, kernel)
    assert d["kernel"] == kernel
    assert d["bytes_per_lef_epoch"] == pytest.approx((d["dram_bytes_read"] + d["dram_bytes_write"]) / d["lef_epochs"],
                                                     rel=1e-3)
    assert traffic == pytest.approx(d["bytes_per_lef_epoch"] * 1_000_000.0)


def test_reference_arm_loads_only_the_oracle():
    """The CPU arm derives its workload (seeds, targets, barriers) through the oracle's helpers:
    the product library stays unloaded in its process."""
    code = (
        "import sys, bench\n"
        "from types import SimpleNamespace\n"
        "bench.run_reference(SimpleNamespace(cells=4, steps=1, warmup=0, cpu_seconds=0.5, gpus=1))\n"
        "maps = open('/proc/self/maps').read()\n"
        "from modlefork_gb300 import engine\n"
        "print('PRODUCT' if ('libmgpu_modle' in maps or engine._lib is not None) else 'CLEAN')\n"
        "print('ORACLE' if 'liboracle' in maps else 'NO-ORACLE')\n")
    p = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    out = p.stdout.strip().splitlines()
    assert out[-2:] == ["CLEAN", "ORACLE"], out
