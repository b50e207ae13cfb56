"""Regenerate tests/golden/reference_pins.json from the reference's own tests.

The reference is Rust and cannot be built here, so its known-answer values
are read from its test sources as text:

  crates/demosaic/tests/amaze_golden.rs   FNV-1a hashes of AMaZE output on the
                                          513x389 integer-LCG mosaic, 4 CFA
                                          layouts x {identity, (2.1, 1, 2.6)}
  crates/demosaic/src/amaze/mod.rs        bit-exact per-stage probes on the
                                          signed 53x47 fixture and its Nyquist
                                          site counts
  crates/core/src/resample.rs             exact 2x2 area-reduction values
  crates/highlight/src/regions.rs         connected-component label grids

Usage: python tests/golden/make_golden.py /path/to/reference
"""

from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def amaze_hashes(ref: str) -> dict[str, str]:
    text = open(os.path.join(ref, "crates/demosaic/tests/amaze_golden.rs")).read()
    block = text[text.index("let expected = ["):]
    block = block[: block.index("];")]
    out = {}
    for name, label, value in re.findall(r'"(\w+) (identity|balanced) ([0-9a-f]{16})"', block):
        out[f"{name.upper()} {label}"] = value
    return out


def amaze_probes(ref: str) -> dict:
    text = open(os.path.join(ref, "crates/demosaic/src/amaze/mod.rs")).read()
    block = text[text.index("const PROBES"):]
    block = block[: block.index("];")]
    probes = [
        {"plane": p, "row": int(r), "col": int(c), "value": v}
        for p, r, c, v in re.findall(r'\("(\w+)",\s*(\d+),\s*(\d+),\s*([-0-9.e]+)\)', block)
    ]
    counts = re.search(r"\(nyquist_sites, voted_sites\), \((\d+), (\d+)\)", text)
    return {"probes": probes, "nyquist_sites": int(counts.group(1)), "voted_sites": int(counts.group(2))}


def area_reduction(ref: str) -> list:
    text = open(os.path.join(ref, "crates/core/src/resample.rs")).read()
    return [
        {"x": int(x), "y": int(y), "rgb": [float(a), float(b), float(c)]}
        for x, y, a, b, c in re.findall(
            r"reduced\.pixel\((\d), (\d)\), Some\(&\[([-0-9.]+), ([-0-9.]+), ([-0-9.]+)\]", text)
    ]


def ccl_cases(ref: str) -> list:
    text = open(os.path.join(ref, "crates/highlight/src/regions.rs")).read()
    block = text[text.index("fn separate_blobs_get_compact_labels_in_raster_order"):]
    block = block[: block.index("#[test]", 10)]
    grid = re.findall(r'"([#.]+)"', block)
    match = re.search(r"assert_eq!\(\s*labels,\s*\[([^\]]*)\]", block)
    labels = [int(v) for v in re.findall(r"\d+", match.group(1))]
    count = int(re.search(r"assert_eq!\(count, (\d+)\)", block).group(1))
    return [{"grid": grid, "labels": labels, "count": count}]


def main(ref: str) -> None:
    data = {
        "source": "values read from the reference's test sources (see module docstring)",
        "amaze_hashes": amaze_hashes(ref),
        "amaze_stage": amaze_probes(ref),
        "area_2x2": area_reduction(ref),
        "ccl": ccl_cases(ref),
    }
    with open(os.path.join(HERE, "reference_pins.json"), "w") as f:
        json.dump(data, f, indent=1)
    print(f"wrote {len(data['amaze_hashes'])} hashes, {len(data['amaze_stage']['probes'])} probes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path to the reference checkout>")
    main(sys.argv[1])
