"""The device's floating-point library against the host's (glibc, which the reference links).

The epoch loop evaluates log, exp and pow on the device with CUDA's libm, while the reference
(and the oracle) use glibc's.  Two results that differ in the last bit would fork a cell's
stream only if the difference changed a decision: an accept/reject test of a sampler, the
number of draws it took, or the integer a noised contact position truncates to.  These tests
measure both on the argument streams the loop feeds the functions:

* the functions themselves, bit for bit: log of generate_canonical draws, pow(-log u, xi) at
  the configurations' xi, the GEV noise of register_contacts.cpp:48-64, exp over the
  ziggurat's wedge range;
* the integers the GEV noise reaches: truncated noised positions and their bins;
* every sampler of the loop on whole seeded streams, sample values and draw counts: the
  normal ziggurat (below_exp), the exponential ziggurat, Poisson (inversion and PTRS),
  binomial (inversion, with (1 - p)^t from the host and from the device, and BTRD) and GEV.

Raw last-bit differences are counted and reported (MGPU_LIBM_REPORT names a JSON file for the
counts); any difference in a decision, a draw count or an integer fails the test.
"""

import json
import os

import numpy as np
import pytest

from modlefork_gb300 import engine
from _harness import host_libm, host_samplers, load_oracle

pytestmark = pytest.mark.gpu

# arguments per function check and samples per sampler check
N_ARGS = int(float(os.environ.get("MGPU_LIBM_N", "1e8")))
N_SAMPLES = int(float(os.environ.get("MGPU_LIBM_SAMPLES", "3e7")))
REPORT = {}


def _report(key, value):
    REPORT[key] = value
    path = os.environ.get("MGPU_LIBM_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(REPORT, f, indent=1, sort_keys=True)


def _canonical_stream(n, seed):
    """generate_canonical<double, 53> of n raw Xoshiro256++ draws (canonical_of on the device)."""
    import ctypes as C

    lib = load_oracle()
    raw = np.empty(n, dtype=np.uint64)
    lib.orc_prng_draws(C.c_uint64(seed), C.c_uint64(n), raw.ctypes.data_as(C.POINTER(C.c_uint64)))
    u = raw.astype(np.float64) / 18446744073709551616.0
    u[u == 1.0] = 1.0 - 2.0 ** -53
    return u[u > 0.0]


def _bits_differ(a, b):
    return int(np.count_nonzero(a.view(np.uint64) != b.view(np.uint64)))


@pytest.fixture(scope="module")
def uniforms():
    return _canonical_stream(N_ARGS, 0x5EED)


def test_log_of_canonical_draws(uniforms):
    dev = engine.probe_libm(engine.PROBE_LOG, uniforms)
    host = host_libm(engine.PROBE_LOG, uniforms)
    _report("log_u", {"n": len(uniforms), "last_bit_differences": _bits_differ(dev, host)})
    np.testing.assert_allclose(dev, host, rtol=2.3e-16, atol=0)  # at most one ulp apart


@pytest.mark.parametrize("xi", [0.001, 0.01, 0.1])
def test_pow_of_neg_log_u(uniforms, xi):
    t = -host_libm(engine.PROBE_LOG, uniforms)
    xs = np.full_like(t, xi)
    dev = engine.probe_libm(engine.PROBE_POW, t, xs)
    host = host_libm(engine.PROBE_POW, t, xs)
    _report(f"pow_neglogu_xi{xi}", {"n": len(t), "last_bit_differences": _bits_differ(dev, host)})
    np.testing.assert_allclose(dev, host, rtol=4.5e-16, atol=0)


def test_gev_noise_and_the_positions_it_truncates_to(uniforms):
    """register_contacts.cpp:48-64 with the default genextreme parameters (mu 0, sigma 5000,
    xi 0.001): the noise itself, then the integer position (u64)(pos - noise) and its 5 kb bin
    for unit positions spread over a 250 Mbp chromosome."""
    mu, sigma, xi = 0.0, 5000.0, 0.001
    dev = engine.probe_libm(engine.PROBE_GEV_NOISE, uniforms, mu=mu, sigma=sigma, xi=xi)
    host = host_libm(engine.PROBE_GEV_NOISE, uniforms, mu=mu, sigma=sigma, xi=xi)
    rng = np.random.default_rng(3)
    pos = rng.integers(10_000_000, 240_000_000, size=len(uniforms)).astype(np.float64)
    ad, ah = pos - dev, pos - host
    ok = (ad >= 0) & (ah >= 0)
    flips = int(np.count_nonzero(ad[ok].astype(np.uint64) != ah[ok].astype(np.uint64)))
    bins = int(np.count_nonzero((ad[ok].astype(np.uint64) // 5000) != (ah[ok].astype(np.uint64) // 5000)))
    # the same noise added on the other side (fwd unit + noise)
    bd, bh = pos + dev, pos + host
    flips += int(np.count_nonzero(bd.astype(np.uint64) != bh.astype(np.uint64)))
    _report("gev_noise", {"n": len(uniforms), "last_bit_differences": _bits_differ(dev, host),
                          "integer_position_differences": flips, "bin_differences": bins,
                          "max_abs_difference_bp": float(np.max(np.abs(dev - host)))})
    assert flips == 0 and bins == 0


def test_exp_over_the_ziggurat_wedges():
    rng = np.random.default_rng(4)
    a = -rng.uniform(0.0, 8.0, size=N_ARGS // 4)
    dev = engine.probe_libm(engine.PROBE_EXP, a)
    host = host_libm(engine.PROBE_EXP, a)
    _report("exp_wedge", {"n": len(a), "last_bit_differences": _bits_differ(dev, host)})
    np.testing.assert_allclose(dev, host, rtol=2.3e-16, atol=0)
    # below_exp decides y < exp(a) exactly where y is next to exp(a): both sides' decisions,
    # for y one ulp either side of the host's exp(a) and at it
    decisions = 0
    for y in (np.nextafter(host, 0.0), host, np.nextafter(host, 1.0)):
        d = engine.probe_libm(engine.PROBE_BELOW_EXP, y, a)
        h = host_libm(engine.PROBE_BELOW_EXP, y, a)
        decisions += int(np.count_nonzero(d != h))
    _report("below_exp_at_the_boundary", {"n": 3 * len(a), "decision_differences": decisions})


SAMPLERS = [
    # (name, probe kind, a0, a1): the parameters the parity and genome workloads feed the loop
    ("normal_moves_2500_125", engine.PROBE_NORMAL, 2500.0, 125.0),
    ("normal_moves_4000_200", engine.PROBE_NORMAL, 4000.0, 200.0),
    ("exponential", engine.PROBE_EXPONENTIAL, 0.0, 0.0),
    ("poisson_inversion_1", engine.PROBE_POISSON, 1.0, 0.0),
    ("poisson_ptrs_24", engine.PROBE_POISSON, 24.0, 0.0),
    ("poisson_ptrs_250", engine.PROBE_POISSON, 250.0, 0.0),
    ("binomial_inversion_20", engine.PROBE_BINOMIAL, 20.0, 1.0 / 6.0),
    ("binomial_inversion_device_pow_7", engine.PROBE_BINOMIAL_DEVICE_POW, 7.0, 1.0 / 6.0),
    ("binomial_btrd_480", engine.PROBE_BINOMIAL, 480.0, 1.0 / 6.0),
    ("binomial_btrd_device_pow_4800", engine.PROBE_BINOMIAL_DEVICE_POW, 4800.0, 1.0 / 6.0),
    ("gev_5000_0.001", engine.PROBE_GEV, 5000.0, 0.001),
]


@pytest.mark.parametrize("name,kind,a0,a1", SAMPLERS, ids=[s[0] for s in SAMPLERS])
def test_sampler_streams_equal_the_host(name, kind, a0, a1):
    nstreams = 8192
    per = max(1, N_SAMPLES // nstreams)
    seeds = np.arange(1, nstreams + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
    dv, dd = engine.probe_samplers(kind, seeds, per, a0, a1)
    hv, hd = host_samplers(kind, seeds, per, a0, a1)
    value_diff = _bits_differ(dv.reshape(-1), hv.reshape(-1))
    draw_diff = int(np.count_nonzero(dd != hd))
    rec = {"samples": int(dv.size), "draws": int(hd.sum()), "value_differences": value_diff,
           "draw_count_differences": draw_diff}
    assert not np.any(dd == np.iinfo(np.uint64).max), "a device sampler hit its iteration limit"
    if kind == engine.PROBE_GEV:
        # the noise is a double the loop only adds to a unit position and truncates: its last
        # bit may differ (see test_gev_noise_...), the integers it reaches must not
        pos = np.random.default_rng(5).integers(10_000_000, 240_000_000, size=dv.size).astype(np.float64)
        d, h = dv.reshape(-1), hv.reshape(-1)
        rec["integer_position_differences"] = int(
            np.count_nonzero((pos - d).astype(np.uint64) != (pos - h).astype(np.uint64)) +
            np.count_nonzero((pos + d).astype(np.uint64) != (pos + h).astype(np.uint64)))
        _report(f"sampler_{name}", rec)
        assert draw_diff == 0 and rec["integer_position_differences"] == 0
        np.testing.assert_allclose(d, h, rtol=0, atol=2e-9)
        return
    _report(f"sampler_{name}", rec)
    assert value_diff == 0 and draw_diff == 0
