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


def test_autotune_times_every_candidate_and_caches(tmp_path, monkeypatch):
    """autotune with a stand-in stepper (no GPU): every candidate is timed
    once, the choice follows pick_shapes, and a second call reads the cache."""
    import numpy as np
    from _cases import case_2d
    from taichi_sim_gb300.sim_support.simulator import Simulator

    made = []

    class FakeStepper:
        def __init__(self, sims, shots, block_cells, nodes_per_thread, shots_per_thread):
            self.shape = (block_cells, nodes_per_thread, shots_per_thread)
            made.append(self.shape)

        def profile_steps(self, n):
            cy, tx, spt = self.shape
            return [1.0 + 0.1 * cy / spt, 1.0 / tx + 0.01 * cy]   # stress, velocity

        def __enter__(self):
            return self

        def __exit__(self, *exc):
            pass

    monkeypatch.setattr(batch, "BatchStepper", FakeStepper)
    monkeypatch.setattr(batch, "_cache_path", lambda: str(tmp_path / "autotune.json"))
    sim = Simulator(case_2d(visco=1, steps=40))
    shots = [np.zeros((3,) + np.shape(sim._source_term), np.float32)]
    best, timings = batch.autotune([sim], shots, steps=2)
    assert sorted(set(made)) == sorted(batch.SHAPES) and len(made) == len(batch.SHAPES)
    assert best == batch.pick_shapes(timings)
    assert best["shots_per_thread"] == 2 and best["block_cells"] == 4 and best["velocity_nodes_per_thread"] == 4
    made.clear()
    again, _ = batch.autotune([sim], shots, steps=2)
    assert again == best and made == []
