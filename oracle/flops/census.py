"""FLOP census of AMaZE on the 24 MP bench workload (measurement infrastructure).

Generates the bench mosaic with the library's seeded generator (this needs
the GPU library), runs the oracle's normalize and Opposed reconstruction on
the host, then the oracle's AMaZE compiled with counting floats
(oracle/flops/amaze_flops.cpp), which returns the bit-identical
reconstruction together with its operation counts. Prints one JSON line with
the operations per output pixel by class. AMaZE's algorithmic work is these
counts: every operation the reference performs in binary32, a division
counted as one operation.

Usage: python oracle/flops/census.py [--rows R]   (R rows from the top; default: all)
"""

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as o  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rows", type=int, default=0)
    args = ap.parse_args()
    from rohditor_gb300 import Device
    from rohditor_gb300.workloads import full_24mp

    wl = full_24mp()
    dev = Device(0)
    raw = wl.mosaic(dev)
    dev.close()
    rows = args.rows or wl.height
    raw = np.ascontiguousarray(raw[:rows])
    W = wl.width
    s = wl.sensor
    cfa = {"RGGB": 0, "BGGR": 1, "GRBG": 2, "GBRG": 3}[s.cfa]
    desc = o.sensor_desc(W, rows, W, (0, 0, W, rows), cfa, list(s.black), s.black_repeat, list(s.white))
    m, pattern = o.normalize(raw, desc)
    m, _, _, _ = o.opposed(m, pattern, s.detection_levels, s.neutral_ceiling)
    t0 = time.perf_counter()
    _, ops = o.amaze_counted(m, pattern, s.demosaic_balance)
    secs = time.perf_counter() - t0
    px = W * rows
    per_px = {k: round(v / px, 2) for k, v in ops.items()}
    per_px["fp32_ops"] = round(sum(ops.values()) / px, 2)
    print(json.dumps({"workload": f"full_24mp {W}x{rows} (bench scene), Opposed, AMaZE",
                      "output_pixels": px, "ops_per_output_pixel": per_px, "census_seconds": round(secs, 1)}))


if __name__ == "__main__":
    main()
