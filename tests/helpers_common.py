"""Inputs of the Standard-kernel helper tests: the reference's test
generator (a 64-bit linear congruential sequence mapped to [-1, 1),
src/solver/simd/kernels.rs:445-454, benches/rhs_swe_2d_bench.rs:19-28)."""

import numpy as np

MASK = (1 << 64) - 1


def random_vec(n: int, seed: int) -> np.ndarray:
    out = np.empty(n)
    x = seed
    for k in range(n):
        x = (x * 6364136223846793005 + 1) & MASK
        out[k] = float(x) / float(MASK) * 2.0 - 1.0
    return out
