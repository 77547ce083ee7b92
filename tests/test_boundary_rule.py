"""The device binning's boundary rule above 256 bins against BuildBoundaries' sequential
rule (src/core/binned_dataset.cpp:95-118), on the CPU.

The reference keeps candidate p (the sorted value at rank QuantileRank(p, m, desired),
p = 1 .. desired - 1) when it is below the maximum and above the last kept boundary. The
device keeps it when it is below the maximum and above candidate p - 1, so that every
candidate decides on its own and a prefix sum compacts the kept ones. The candidates are
non-decreasing, so the two rules agree; this checks it on seeded columns with heavy ties,
signed zeros and few distinct values, in float comparisons as both sides make them.
"""

from __future__ import annotations

import numpy as np
import pytest


def _quantile_rank(part: int, total: int, divisor: int) -> int:
    whole = part * (total // divisor)
    numerator = part * (total % divisor)
    return whole + numerator // divisor + (1 if numerator % divisor else 0) - 1


def _candidates(values: np.ndarray, max_bins: int) -> tuple[list, float]:
    v = np.sort(values[~np.isnan(values)], kind="stable")
    m = v.size
    desired = min(max_bins, m)
    return [v[_quantile_rank(p, m, desired)] for p in range(1, desired)], (v[-1] if m else 0.0)


def _sequential(values: np.ndarray, max_bins: int) -> list:
    cands, maximum = _candidates(values, max_bins)
    kept: list = []
    for c in cands:
        if c < maximum and (not kept or c > kept[-1]):
            kept.append(c)
    return kept


def _parallel(values: np.ndarray, max_bins: int) -> list:
    cands, maximum = _candidates(values, max_bins)
    return [c for p, c in enumerate(cands) if c < maximum and (p == 0 or c > cands[p - 1])]


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("max_bins", [257, 1000, 4096, 65536])
def test_parallel_boundary_rule_equals_sequential(seed, max_bins):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 20000))
    kind = seed % 4
    if kind == 0:
        x = rng.normal(size=n).astype(np.float32)
    elif kind == 1:  # heavy ties
        x = np.round(rng.normal(size=n) * 3).astype(np.float32)
    elif kind == 2:  # signed zeros among few values
        x = rng.choice(np.array([-0.0, 0.0, 1.5, -2.0], np.float32), size=n)
    else:  # lognormal with missing values
        x = np.exp(rng.normal(size=n) * 4).astype(np.float32)
        x[rng.random(n) < 0.1] = np.nan
    seq, par = _sequential(x, max_bins), _parallel(x, max_bins)
    assert len(seq) == len(par)
    assert all(a == b for a, b in zip(seq, par))  # float equality: -0 == +0
