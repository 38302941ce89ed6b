"""The seeded benchmark workloads stay what the measurements quote: total
particle counts of the batched and served workloads, and digests of small
instances of each generator (positions, velocities, settings, mass, dt)."""
import hashlib

import numpy as np

from novaphy_gb300 import workloads


def _digest(ws):
    h = hashlib.sha256()
    for w in ws:
        h.update(w.x.tobytes())
        h.update(w.v.tobytes())
        h.update(repr(sorted(w.settings.items())).encode())
        h.update(np.float32(w.mass).tobytes())
        h.update(np.float32(w.dt).tobytes())
    return h.hexdigest()[:16]


def test_quoted_totals():
    assert sum(w.n for w in workloads.batched_scenes()) == 19_350_346
    served = workloads.served_scenes()
    assert len(served) == 256 and sum(w.n for w in served) == 10_102_870
    assert sum(len(w.meta["spheres"]) for w in served) == 537


def test_generators_are_deterministic():
    assert _digest(workloads.batched_scenes(nscenes=8, seed=3)) == "5c02564a4afbd39a"
    assert _digest(workloads.served_scenes(nclients=8, seed=4)) == "9e9c1de99abd9949"
    assert _digest([workloads.dam_break_8k()]) == "eeb0e91429879650"
    w = workloads.dam_break_1m()
    assert w.n == 1_000_000 and w.x.dtype == np.float32
