"""The chunk-mix workload: many generation requests of uneven sizes and trees.

Sizes are drawn uniformly from {16^3, 32^3, 64^3} 3D grids and {32^2, 128^2,
512^2} 2D grids; each request uses one of eight fixed trees (the three
workload trees plus Value, CellularValue, CellularLookup(Simplex),
FractalFBm(Simplex), Add/Multiply blends); seeds are uniform int32; origins
are random integer multiples of the chunk size within [-2^20, 2^20]; step 1.
Inputs are synthetic and seeded (numpy PCG64, seed 20261203).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Tuple

import numpy as np

from tests import trees

SIZES: List[Tuple[int, ...]] = [(16, 16, 16), (32, 32, 32), (64, 64, 64), (32, 32), (128, 128), (512, 512)]


@dataclass
class Chunk:
    tree: int                    # index into trees.MIX_TREES
    count: Tuple[int, ...]
    offset: Tuple[float, ...]
    seed: int

    @property
    def points(self) -> int:
        return int(np.prod(self.count))


def make_mix(n: int = 4096, seed: int = 20261203, sizes=SIZES) -> List[Chunk]:
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        size = sizes[int(rng.integers(len(sizes)))]
        tree = int(rng.integers(len(trees.MIX_TREES)))
        s = int(rng.integers(-(2**31), 2**31 - 1))
        edge = max(size[0], 1)
        lim = (1 << 20) // edge
        offset = tuple(float(edge * int(rng.integers(-lim, lim + 1))) for _ in size)
        out.append(Chunk(tree, size, offset, s))
    return out
