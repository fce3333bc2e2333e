"""Post-processing of hit-record CSV files (the reference's write_output format).

clean_receiver_direct_sun_hits mirrors scripts/post_processing/clean_direct_sun.py:6-18: it drops
every ray number whose rows include a receiver record (stage 2) but no mirror record (stage 1), i.e.
light that reaches the receiver straight from the sun, which a staged SolTrace run never records.
The kept rows are copied unchanged.  The same filter runs while writing with
`Tracer.write_output(path, staged=True)` / `native.write_hits_csv(hits, path, staged=True)`, and the
device flux maps skip those records with `staged=True`.
"""
from __future__ import annotations

import numpy as np


def direct_sun_rays(hits: np.ndarray) -> np.ndarray:
    """Boolean [N] mask of the rays of [N, 5, 4] hit records whose first interaction is the
    receiver (a stage-2 record in slot 1)."""
    return np.asarray(hits)[:, 1, 0] == 2.0


def clean_receiver_direct_sun_hits(filename: str, output_filename: str) -> None:
    """Copy the CSV `filename` to `output_filename` without the rows of the ray numbers that have
    a stage-2 row and no stage-1 row."""
    with open(filename, "r", newline="") as f:
        lines = f.read().splitlines(keepends=True)
    if not lines:
        raise ValueError(f"{filename}: empty file")
    header, rows = lines[0], lines[1:]
    numbers = np.empty(len(rows), np.int64)
    stages = np.empty(len(rows), np.float64)
    for k, line in enumerate(rows):
        a, b, _ = line.split(",", 2)
        numbers[k] = int(a)
        stages[k] = float(b)
    uniq, inv = np.unique(numbers, return_inverse=True)
    has1 = np.zeros(len(uniq), bool)
    has2 = np.zeros(len(uniq), bool)
    np.logical_or.at(has1, inv, stages == 1)
    np.logical_or.at(has2, inv, stages == 2)
    keep = (has1 | ~has2)[inv]
    with open(output_filename, "w", newline="") as f:
        f.write(header)
        f.writelines(r for r, k in zip(rows, keep) if k)
    print(f"Cleaned data saved to {output_filename}")
