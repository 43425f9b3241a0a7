"""Seeded synthetic workloads with the shapes of the benchmark
configurations (the reference ships no dump or test data)."""
from __future__ import annotations

import numpy as np

from . import engine, synth

# 64 images of uneven sizes: 32 at 128^2, 24 at 256^2, 6 at 512^2, 2 at 1024^2
BATCH_SIZES = [128] * 32 + [256] * 24 + [512] * 6 + [1024] * 2
BATCH_FREQS = (86e9, 230e9, 345e9)


def batch_dumps(n: int = 256):
    """The two dumps of the batched configuration: a = 0.5 and a = 0.9375."""
    return [synth.make_torus(n1=n, n2=n, a=0.5, seed=501), synth.make_torus(n1=n, n2=n, a=0.9375, seed=502)]


def batch_images(grid_ids, seed: int = 64, sizes=BATCH_SIZES):
    """Image descriptors: inclination uniform in [5, 175] deg, frequency from
    {86, 230, 345} GHz, M_unit log-uniform in [1e18, 1e20] g, dump chosen at
    random, all from one seed."""
    rng = np.random.default_rng(seed)
    descs = []
    for s in sizes:
        descs.append(engine.image_desc(s, s, [float(rng.choice(BATCH_FREQS))], grid=int(grid_ids[rng.integers(2)]),
                                       inclination=float(rng.uniform(5.0, 175.0)),
                                       m_unit=float(10 ** rng.uniform(18.0, 20.0))))
    return descs
