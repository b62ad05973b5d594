"""Host logic of the batched launch (CPU): launch-shape choice from kernel
timings, the candidate list."""
from taichi_sim_gb300 import batch


def test_pick_shapes_takes_each_kernels_fastest_per_layout():
    timings = {  # [stress_ms, velocity_ms] per CYxTXxSPT
        "4x1x1": [2.3, 1.5], "4x4x1": [2.1, 0.85], "8x4x1": [2.0, 0.9],
        "4x2x2": [1.75, 1.06], "4x4x2": [1.74, 0.71], "8x4x2": [1.77, 0.70],
    }
    best = batch.pick_shapes(timings)
    # one shot per thread: 2.0 + 0.85 = 2.85; two: 1.74 + 0.70 = 2.44
    assert best == {"block_cells": 4, "nodes_per_thread": 4, "shots_per_thread": 2,
                    "velocity_block_cells": 8, "velocity_nodes_per_thread": 4}


def test_pick_shapes_single_candidate():
    best = batch.pick_shapes({"8x2x1": [1.0, 0.5]})
    assert best == {"block_cells": 8, "nodes_per_thread": 2, "shots_per_thread": 1,
                    "velocity_block_cells": 8, "velocity_nodes_per_thread": 2}


def test_candidate_shapes():
    assert len(batch.SHAPES) == 12 and len(set(batch.SHAPES)) == 12
    assert {s[0] for s in batch.SHAPES} == {4, 8} and {s[1] for s in batch.SHAPES} == {1, 2, 4}
    assert {s[2] for s in batch.SHAPES} == {1, 2}
