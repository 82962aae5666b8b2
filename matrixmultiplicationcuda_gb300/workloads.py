"""Seeded synthetic workloads.

uneven_batch_specs: the batched workload of 64 independent products of uneven
size and sparsity. Per problem: M = K drawn uniformly from [512, 8192] and
rounded to a multiple of 64; block height from {16, 32, 64} (blocks bR x 16);
structure from {random, diagonal band, block-diagonal}; block density
log-uniform in [0.5 %, 25 %]; N from {128, 256, 512}; fp16 values uniform in
[-1, 1]; fp32 output.

How a density is realised per pattern:
  random     -- each block kept with probability `density`;
  band       -- half-width h = ceil(density * KB / 2) block columns around the
                diagonal, blocks in the band kept with probability
                min(1, density * KB / band length);
  blockdiag  -- dense diagonal tiles of T x T elements, T = density * K rounded
                to a multiple of 64 (at least 64), so the block density is T / K.
"""
import math

import numpy as np

from .host import (DIST_UNIFORM, PATTERN_BAND, PATTERN_BLOCKDIAG, PATTERN_RANDOM, gen_dense,
                   gen_structure, gen_values)


def uneven_batch_specs(count=64, seed=2024):
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        M = int(rng.integers(512, 8193))
        M = int(min(8192, max(512, round(M / 64) * 64)))
        bR = int(rng.choice([16, 32, 64]))
        pattern = int(rng.choice([PATTERN_RANDOM, PATTERN_BAND, PATTERN_BLOCKDIAG]))
        density = float(math.exp(rng.uniform(math.log(0.005), math.log(0.25))))
        N = int(rng.choice([128, 256, 512]))
        specs.append(dict(M=M, K=M, bR=bR, pattern=pattern, density=density, N=N,
                          seed=seed * 1000 + i))
    return specs


def _param(spec):
    KB = spec["K"] // 16
    if spec["pattern"] == PATTERN_BAND:
        return float(max(1, math.ceil(spec["density"] * KB / 2)))
    if spec["pattern"] == PATTERN_BLOCKDIAG:
        return float(max(64, int(round(spec["density"] * spec["K"] / 64)) * 64))
    return 0.0


def make_problem(spec):
    """Host arrays of one problem: (row_ptr, col_idx, fp32 block values, fp32 B)."""
    rp, ci = gen_structure(spec["M"], spec["K"], spec["bR"], spec["pattern"], spec["density"],
                           _param(spec), seed=spec["seed"])
    vals = gen_values(len(ci), spec["bR"], 16, DIST_UNIFORM, seed=spec["seed"] + 1)
    B = gen_dense(spec["K"], spec["N"], DIST_UNIFORM, seed=spec["seed"] + 2)
    return rp, ci, vals, B
