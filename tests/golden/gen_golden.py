#!/usr/bin/env python3
"""Extract the reference's known-answer tests for the epoch loop into JSON fixtures.

Reads (as text) the Catch2 unit tests of the reference checkout given on the command line:
  test/units/simulation_cpu/simulation_simple_unit_test.cpp
  test/units/simulation_cpu/simulation_complex_unit_test.cpp
  test/units/simulation_cpu/common.hpp (DEFAULT_PRNG seed, init_config semantics)
and writes tests/golden/reference_unit_tests.json: for every test case with exact expected
arrays, its inputs (chromosome, LEFs, barriers, ranks, moves, config overrides, PRNG seed),
the ordered list of Simulation::test_* hooks it calls, and the expected outputs.

Also writes tests/golden/xxh3_vectors.json: XXH3_64bits_withSeed values of the per-cell seed
key (name | size | cell_id, genome.cpp:317-335) computed with the xxHash 0.8.x header found
next to this checkout (pyarrow vendors one), if a C compiler and the header are available.

Usage: python gen_golden.py /path/to/reference [xxhash.h]
"""

import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))

HOOKS = {
    "test_adjust_and_clamp_moves": "ADJUST_AND_CLAMP",
    "test_detect_units_at_chrom_boundaries": "DETECT_BOUNDARIES",
    "test_detect_primary_lef_lef_collisions": "DETECT_PRIMARY",
    "test_process_lef_lef_collisions": "LEF_LEF",
    "test_detect_lef_bar_collisions": "DETECT_LEF_BAR",
    "test_correct_moves_for_lef_bar_collisions": "CORRECT_LEF_BAR",
    "test_process_collisions": "PROCESS_COLLISIONS",
    "test_fix_secondary_lef_lef_collisions": "FIX_SECONDARY",
    "test_rank_lefs": "RANK",
}

EVENT = {  # common.hpp:24-31: each named constant already includes COLLISION (0x10)
    "CHROM_BOUNDARY": 0x18,
    "LEF_BAR": 0x14,
    "LEF_LEF_PRIMARY": 0x12,
    "LEF_LEF_SECONDARY": 0x11,
}


def split_cases(text):
    starts = [m for m in re.finditer(r'TEST_CASE\("([^"]+)"', text)]
    for k, m in enumerate(starts):
        end = starts[k + 1].start() if k + 1 < len(starts) else len(text)
        line = text.count("\n", 0, m.start()) + 1
        yield m.group(1), text[m.start():end], line


def ints(s):
    return [int(x) for x in re.findall(r"-?\d+", s)]


def parse_array(block, name):
    m = re.search(r"std::array<[^>]+>\s+" + re.escape(name) + r"\s*\{([^}]*)\}", block)
    return ints(m.group(1)) if m else None


def parse_collisions(block, name):
    m = re.search(
        r"std::array<CollisionT,\s*nlefs>\s+" + re.escape(name) + r"\s*\{(.*?)\};", block, re.S)
    if not m:
        return None
    out = []
    for cm in re.finditer(r"CollisionT\{([^}]*)\}", m.group(1)):
        body = cm.group(1).strip()
        if not body:
            out.append(0)
            continue
        idx_s, ev_s = [x.strip() for x in body.split(",")]
        out.append(int(idx_s) | (EVENT[ev_s] << 56))
    return out


def parse_lefs(block, var="lefs"):
    m = re.search(r"\b" + var + r"\s*\{(.*?)\};", block, re.S)
    if not m:
        return None
    lefs = [ints(x) for x in re.findall(r"construct_lef\(([^)]*)\)", m.group(1))]
    return [[a, b, (e[0] if e else 0)] for a, b, *e in lefs]


def parse_chrom(block):
    m = re.search(r'init_chromosome\("[^"]+",\s*([^)]*)\)', block)
    if m:
        args = ints(m.group(1))
        size = args[0]
        start = args[1] if len(args) > 1 else 0
        end = min(args[2] if len(args) > 2 else size, size)
        return {"start": start, "end": end, "size": size}
    m = re.search(r'Chromosome\s+chrom\{\s*0,\s*"[^"]+",\s*(\d+),\s*(\d+),\s*(\d+)\s*\}', block)
    if m:
        s, e, z = map(int, m.groups())
        return {"start": s, "end": e, "size": z}
    return None


def parse_barriers(block):
    m = re.search(r"construct_barriers(<s>)?\((.*?)\);", block, re.S)
    if not m:
        if "ExtrusionBarriers barriers{}" in block:
            return []
        return None
    inactive = m.group(1) is not None and "State::INACTIVE" in block
    out = []
    for bm in re.finditer(r"ExtrusionBarrier\{([^}]*)\}", m.group(2)):
        parts = [x.strip() for x in bm.group(1).split(",")]
        pos, sa, si, strand = int(parts[0]), float(parts[1]), float(parts[2]), parts[3].strip("'")
        # ExtrusionBarrier(pos, stp_a, stp_i, char): '+' blocks REV (1), '-' blocks FWD (2)
        out.append({"pos": pos, "stp_active": sa, "stp_inactive": si,
                    "blocking_dir": 1 if strand == "+" else 2, "state": 0 if inactive else 1})
    return out


def parse_config(block):
    cfg = {}
    m = re.search(r"init_config\((\d+),\s*(\d+)\)", block)
    if m:  # common.hpp:135-149
        cfg.update(rev_extrusion_speed=int(m.group(1)), fwd_extrusion_speed=int(m.group(2)),
                   rev_extrusion_speed_std=0.0, fwd_extrusion_speed_std=0.0,
                   probability_of_extrusion_unit_bypass=0.0,
                   lef_bar_major_collision_pblock=1.0, lef_bar_minor_collision_pblock=0.0)
    for key in ("lef_bar_major_collision_pblock", "lef_bar_minor_collision_pblock",
                "probability_of_extrusion_unit_bypass"):
        mm = re.search(r"c\." + key + r"\s*=\s*([0-9.]+)", block)
        if mm:
            cfg[key] = float(mm.group(1))
    return cfg


def parse_seed(block, default_seed):
    m = re.search(r"random::PRNG\((\d+)ULL\)", block)
    return int(m.group(1)) if m else default_seed


def parse_steps(block):
    steps = []
    for m in re.finditer(r"\b(test_\w+)\(", block):
        if m.group(1) in HOOKS:
            steps.append((m.start(), m.group(1), block[m.end():block.find(";", m.end())]))
    return steps


def extract(path, default_seed, rel):
    text = open(path).read()
    cases = []
    for name, block, line in split_cases(text):
        steps = parse_steps(block)
        if not steps:
            continue
        if name.startswith("LEFs ranking"):
            for var, suffix in (("lefs1", "1"), ("lefs2", "2")):
                lefs = parse_lefs(block, var)
                cases.append({
                    "name": f"{name} [{var}]", "source": f"{rel}:{line}", "chrom": None,
                    "config": {}, "seed": default_seed, "lefs": lefs, "released": [],
                    "barriers": [], "rev_ranks": list(range(len(lefs))),
                    "fwd_ranks": list(range(len(lefs))), "rev_moves": [0] * len(lefs),
                    "fwd_moves": [0] * len(lefs),
                    "steps": [{"hook": "RANK", "partially_sorted": 0, "init_ranks": 1}],
                    "expected": {"rev_ranks": parse_array(block, "rev_ranks_expected" + suffix),
                                 "fwd_ranks": parse_array(block, "fwd_ranks_expected" + suffix)},
                })
            continue
        lefs = parse_lefs(block)
        exp = {}
        for key in ("rev_moves", "fwd_moves"):
            for cand in (key + "_expected", key + "_adjusted"):
                v = parse_array(block, cand)
                if v is not None:
                    exp[key] = v
        for key in ("rev_collisions", "fwd_collisions"):
            v = parse_collisions(block, key + "_expected")
            if v is not None:
                exp[key] = v
        for rk in ("rev_ranks", "fwd_ranks"):
            checks = re.findall(r"CHECK\(" + rk + r"\[(\d+)\] == (\d+)\)", block)
            if checks:
                arr = [0] * len(lefs)
                for i, v in checks:
                    arr[int(i)] = int(v)
                exp[rk] = arr
        if not exp:
            continue
        released = [int(x) for x in re.findall(r"lefs\[(\d+)\]\.release\(\)", block)]
        case = {
            "name": name, "source": f"{rel}:{line}", "chrom": parse_chrom(block),
            "config": parse_config(block), "seed": parse_seed(block, default_seed),
            "lefs": lefs, "released": released, "barriers": parse_barriers(block) or [],
            "rev_ranks": parse_array(block, "rev_ranks"), "fwd_ranks": parse_array(block, "fwd_ranks"),
            "rev_moves": parse_array(block, "rev_moves"), "fwd_moves": parse_array(block, "fwd_moves"),
            "steps": [{"hook": HOOKS[h]} for _, h, _ in steps], "expected": exp,
        }
        if case["rev_moves"] is None:
            case["rev_moves"] = [0] * len(lefs)
            case["fwd_moves"] = [0] * len(lefs)
        cases.append(case)
    return cases


XXH_PROG = r"""
#define XXH_INLINE_ALL
#include "xxhash.h"
#include <stdio.h>
#include <string.h>
#include <stdint.h>
int main(void) {
  const char* names[] = {"", "c", "chr", "chr1", "chr10", "chrX", "chr22", "chrS",
    "chromosome_with_a_longer_name_0123456789", "a_really_long_chromosome_name_that_goes_beyond_"
    "one_hundred_and_twenty_eight_bytes_of_key_material_to_reach_the_129_to_240_range_xx"};
  const uint64_t sizes[] = {0, 1, 10000000, 248956422, 4294967295ull};
  const uint64_t seeds[] = {0, 1, 10556020843759504871ull, 42};
  const uint64_t cells[] = {0, 1, 63, 511, 1000000};
  printf("[\n");
  int first = 1;
  for (unsigned a = 0; a < sizeof(names)/sizeof(*names); ++a)
   for (unsigned b = 0; b < sizeof(sizes)/sizeof(*sizes); ++b)
    for (unsigned c = 0; c < sizeof(seeds)/sizeof(*seeds); ++c)
     for (unsigned d = 0; d < sizeof(cells)/sizeof(*cells); ++d) {
      XXH3_state_t* st = XXH3_createState();
      XXH3_64bits_reset_withSeed(st, seeds[c]);
      XXH3_64bits_update(st, names[a], strlen(names[a]));
      XXH3_64bits_update(st, &sizes[b], 8);
      XXH3_64bits_update(st, &cells[d], 8);
      unsigned long long h = XXH3_64bits_digest(st);
      XXH3_freeState(st);
      printf("%s{\"name\": \"%s\", \"size\": %llu, \"seed\": %llu, \"cell\": %llu, \"hash\": %llu}",
             first ? "" : ",\n", names[a], (unsigned long long)sizes[b],
             (unsigned long long)seeds[c], (unsigned long long)cells[d], h);
      first = 0;
     }
  printf("\n]\n");
  return 0;
}
"""


def gen_xxh3(header):
    if not header or not os.path.exists(header):
        print("xxhash.h not found: xxh3_vectors.json left unchanged", file=sys.stderr)
        return
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "x.c")
        exe = os.path.join(tmp, "x")
        open(src, "w").write(XXH_PROG)
        subprocess.check_call(["gcc", "-O1", "-I", os.path.dirname(header), src, "-o", exe])
        out = subprocess.check_output([exe]).decode()
    vecs = json.loads(out)
    with open(os.path.join(HERE, "xxh3_vectors.json"), "w") as f:
        json.dump({"generator": "xxHash XXH3_64bits streaming API, header " +
                   os.path.basename(os.path.dirname(header)), "vectors": vecs}, f, indent=0)
    print(f"wrote {len(vecs)} xxh3 vectors")


def main():
    import argparse

    ap = argparse.ArgumentParser(description="Re-extract the reference's known-answer cases and the "
                                             "XXH3 vectors into tests/golden/.")
    ap.add_argument("reference", help="root of the reference source tree (MoDLE)")
    ap.add_argument("xxhash_header", help="path of an xxhash.h (xxHash 0.8.x) to build the vector generator")
    args = ap.parse_args()
    ref, header = args.reference, args.xxhash_header
    common = open(os.path.join(ref, "test/units/simulation_cpu/common.hpp")).read()
    default_seed = int(re.search(r"DEFAULT_PRNG\{random::PRNG\((\d+)ULL\)\}", common).group(1))
    cases = []
    for rel in ("test/units/simulation_cpu/simulation_simple_unit_test.cpp",
                "test/units/simulation_cpu/simulation_complex_unit_test.cpp"):
        cases += extract(os.path.join(ref, rel), default_seed, rel)
    with open(os.path.join(HERE, "reference_unit_tests.json"), "w") as f:
        json.dump({"default_seed": default_seed, "cases": cases}, f, indent=1)
    print(f"wrote {len(cases)} cases")
    gen_xxh3(header)


if __name__ == "__main__":
    main()
