#!/usr/bin/env python3
"""Generate the ziggurat layer tables used by the normal and exponential samplers.

The epoch loop draws every LEF move from ``normal_distribution<double>`` and the normal
tail from ``exponential_distribution<double>`` (Boost.Random 1.79, selected by
``src/common/include/modle/common/random.hpp:34-53``; move generation in
``src/libmodle/cpu/simulation.cpp:264-290``).  Boost implements both with the
Marsaglia-Tsang ziggurat (2000): 128 layers plus a sign bit for the normal, 256 layers for
the exponential.  Layer ``i`` is the rectangle ``[0, x_i] x [y_i, y_{i+1}]``; ``x_1 = r`` is
the tail start, ``x_0 = v / f(r)`` is the width of the base strip of area ``v``,
``y_i = f(x_i)`` with ``y_0 = 0`` and ``x_n = 0``.

The tables are a pure function of the density, so they are recomputed here from the
mathematics at 80 significant digits (mpmath) and rounded once to the nearest double.
The output header holds exact C99 hex-float literals, so the host oracle and the device
kernels read bit-identical constants.

Usage: python gen_ziggurat_tables.py > ziggurat_tables.h
"""

import mpmath as mp

mp.mp.dps = 80


def _solve(n_layers, f, finv, tail_area, r_lo, r_hi):
    """Find the tail start r for which the layer recurrence closes exactly at x_n = 0."""

    def closure(r):
        v = r * f(r) + tail_area(r)
        x = r
        for _ in range(1, n_layers - 1):
            y = f(x) + v / x
            if y >= 1:
                return mp.mpf(1)  # recurrence overshot the mode: r is too small
            x = finv(y)
        return f(x) + v / x - 1

    lo, hi = mp.mpf(r_lo), mp.mpf(r_hi)
    assert closure(lo) > 0 > closure(hi)
    for _ in range(400):
        mid = (lo + hi) / 2
        if closure(mid) > 0:
            lo = mid
        else:
            hi = mid
    r = (lo + hi) / 2
    v = r * f(r) + tail_area(r)
    xs = [v / f(r), r]
    x = r
    for _ in range(1, n_layers - 1):
        x = finv(f(x) + v / x)
        xs.append(x)
    xs.append(mp.mpf(0))
    ys = [mp.mpf(0)] + [f(x) for x in xs[1:]]
    ys[-1] = mp.mpf(1)
    return r, v, xs, ys


def normal_tables():
    f = lambda x: mp.e ** (-(x * x) / 2)
    finv = lambda y: mp.sqrt(-2 * mp.log(y))
    tail = lambda r: mp.sqrt(mp.pi / 2) * mp.erfc(r / mp.sqrt(2))
    return _solve(128, f, finv, tail, 3.0, 4.0)


def exponential_tables():
    f = lambda x: mp.e ** (-x)
    finv = lambda y: -mp.log(y)
    tail = lambda r: mp.e ** (-r)
    return _solve(256, f, finv, tail, 7.0, 8.0)


def _hex(x):
    return float(x).hex()


def emit(name, xs, ys):
    out = [f"MGPU_ZIG_TABLE_QUAL double {name}_x[{len(xs)}] = {{"]
    out += [f"    {_hex(x)}," for x in xs]
    out.append("};")
    out.append(f"MGPU_ZIG_TABLE_QUAL double {name}_y[{len(ys)}] = {{")
    out += [f"    {_hex(y)}," for y in ys]
    out.append("};")
    return "\n".join(out)


def main():
    rn, vn, xn, yn = normal_tables()
    re_, ve, xe, ye = exponential_tables()
    print("// Generated by gen_ziggurat_tables.py - do not edit.")
    print("// Ziggurat layer tables (Marsaglia-Tsang 2000) for the unit normal (128 layers)")
    print("// and unit exponential (256 layers), rounded once to the nearest double.")
    print(f"// normal:      r = {mp.nstr(rn, 25)}, v = {mp.nstr(vn, 25)}")
    print(f"// exponential: r = {mp.nstr(re_, 25)}, v = {mp.nstr(ve, 25)}")
    print("#pragma once")
    print("#ifndef MGPU_ZIG_TABLE_QUAL")
    print("#define MGPU_ZIG_TABLE_QUAL static const")
    print("#endif")
    print(emit("mgpu_zig_normal", xn, yn))
    print(emit("mgpu_zig_exp", xe, ye))


if __name__ == "__main__":
    main()
