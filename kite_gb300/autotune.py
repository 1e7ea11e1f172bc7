"""Autotuner for the count's launch shapes.

Two knobs decide how the key-range sort is cut and launched:
  tile_fill      target tile load as a fraction of the on-chip tile capacity
                 (tile shape: more, smaller tiles vs fewer, fuller ones);
  scatter_shape  launch shape of the key-range split scatter, threads x keys
                 per thread: 0 = 256x8 up to 256 digits and 512x8 above,
                 1 = 256x16, 2 = 512x8, 3 = 512x16.
`tune` times a caller-supplied count of the real workload for every pair and
keeps the fastest; `record` writes the choice and the whole table as JSON so a
run can be reproduced with the same shapes.
"""
from __future__ import annotations

import json
import time

FILLS = (0.7, 0.85, 1.0)
SHAPES = (0, 1, 2, 3)
SHAPE_NAMES = {0: "by digits", 1: "256x16", 2: "512x8", 3: "512x16"}


def tune(run_once, fills=FILLS, shapes=SHAPES, reps: int = 2) -> tuple[dict, list]:
    """run_once(tile_fill, scatter_shape) counts the workload once and returns
    its duration in seconds.  Returns (best row, all rows)."""
    table = []
    for f in fills:
        for sh in shapes:
            run_once(f, sh)  # warm-up: buffers grow, kernels load
            best = min(run_once(f, sh) for _ in range(max(1, reps)))
            table.append({"tile_fill": f, "scatter_shape": sh, "shape": SHAPE_NAMES.get(sh, str(sh)),
                          "seconds": best})
    return min(table, key=lambda r: r["seconds"]), table


def record(path: str, best: dict, table: list, workload: str) -> None:
    with open(path, "w") as f:
        json.dump({"workload": workload, "chosen": best, "table": table, "time": time.time()}, f, indent=1)
