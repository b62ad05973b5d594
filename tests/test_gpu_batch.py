"""Batched shots agree with one simulation per shot.

Every shot of a batch (phantoms of uneven sizes, shots innermost on the
device) must match the regular stepper run on that shot alone, within the
parity tolerance; and the plain stepper is itself checked against the CPU
oracle for one shot, closing the chain to the reference's kernels.
"""
import numpy as np
import pytest

from _cases import rel_l2
from oracle import oracle
from taichi_sim_gb300 import engine, workloads
from taichi_sim_gb300.batch import BatchStepper, autotune, fmc_shot_sources
from taichi_sim_gb300.sim_support.simulator import Simulator

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _phantoms(steps=160, n_elem=6):
    cfgs = workloads.fmc2d_phantoms(n_steps=steps, shapes=((72, 84), (96, 84)), n_elem=n_elem, dx=0.1, pml=8)
    for c in cfgs:  # a smaller array for the small grids
        c["probes"][0]["linear"].update(dim_a=0.3, inter_elem=0.1)
    return [Simulator(c) for c in cfgs]


def _single_shot(sim, table):
    """The regular stepper on one shot: the shot's table as the source term,
    read as source_term[k, idx] (the stride is the table's width)."""
    st = engine.Stepper.__new__(engine.Stepper)
    saved = sim._source_term, sim._n_src
    sim._source_term, sim._n_src = table, table.shape[1]
    try:
        st.__init__(sim, family=engine.WGSL2D)
    finally:
        sim._source_term, sim._n_src = saved
    return st


@pytest.mark.parametrize("shape", [(4, 1, 1), (4, 2, 1), (8, 2, 1), (8, 4, 1), (4, 1, 2), (8, 2, 2), (4, 4, 2)],
                         ids=lambda s: f"{s[0]}x{s[1]}x{s[2]}")
def test_batch_matches_single_shots(shape):
    sims = _phantoms()
    shots = [fmc_shot_sources(s) for s in sims]
    with BatchStepper(sims, shots, block_cells=shape[0], nodes_per_thread=shape[1], shots_per_thread=shape[2]) as b:
        b.run(sims[0]._n_steps)
        n, vmax, bad = b.status()
        assert n == sims[0]._n_steps and bad == -1
        for q, sim in enumerate(sims):
            tr = b.traces(q)
            syy = b.field(q, "syy")
            for s in (0, 2, shots[q].shape[0] - 1):
                with _single_shot(sim, shots[q][s]) as one:
                    one.run(sim._n_steps)
                    want_tr, want_f = one.read("traces"), one.read("syy")
                assert np.abs(want_tr).max() > 0
                assert rel_l2(tr[s], want_tr) <= TOL, (q, s, rel_l2(tr[s], want_tr))
                assert rel_l2(syy[s], want_f) <= TOL, (q, s, rel_l2(syy[s], want_f))


def test_batch_without_prefetch_is_identical(monkeypatch):
    """The batched kernels' L2 prefetch is a hint: with TS_BATCH_PREFETCH=0
    the batch gives the same bits."""
    sims = _phantoms(steps=120)
    shots = [fmc_shot_sources(s) for s in sims]
    out = {}
    for flag in ("1", "0"):
        monkeypatch.setenv("TS_BATCH_PREFETCH", flag)
        with BatchStepper(sims, shots, block_cells=4, nodes_per_thread=2, shots_per_thread=2) as b:
            b.run(120)
            assert b.status()[2] == -1
            out[flag] = [(b.traces(q), b.field(q, "syy")) for q in range(len(sims))]
    for q in range(len(sims)):
        assert np.abs(out["1"][q][0]).max() > 0
        np.testing.assert_array_equal(out["0"][q][0], out["1"][q][0])
        np.testing.assert_array_equal(out["0"][q][1], out["1"][q][1])


def test_single_shot_matches_oracle():
    sim = _phantoms(steps=120)[1]
    table = fmc_shot_sources(sim)[3]
    with _single_shot(sim, table) as one:
        one.run(sim._n_steps)
        got_tr, got_f = one.read("traces"), one.read("syy")
    saved = sim._source_term, sim._n_src
    sim._source_term, sim._n_src = table, table.shape[1]
    try:
        ref = oracle.run(sim, oracle.WGSL2D)
    finally:
        sim._source_term, sim._n_src = saved
    assert rel_l2(got_tr, ref["sens"]) <= TOL
    assert rel_l2(got_f, ref["syy"]) <= TOL


def test_autotuner_picks_and_caches(tmp_path, monkeypatch):
    from taichi_sim_gb300 import batch
    monkeypatch.setattr(batch, "_cache_path", lambda: str(tmp_path / "autotune.json"))
    sims = _phantoms(steps=40)
    shots = [fmc_shot_sources(s) for s in sims]
    best, timings = autotune(sims, shots, steps=4)
    assert set(timings) == {f"{cy}x{tx}x{spt}" for cy, tx, spt in batch.SHAPES}
    assert (best["block_cells"], best["nodes_per_thread"], best["shots_per_thread"]) in batch.SHAPES
    assert (best["velocity_block_cells"], best["velocity_nodes_per_thread"], best["shots_per_thread"]) in batch.SHAPES
    again, _ = autotune(sims, shots, steps=4)
    assert again == best and (tmp_path / "autotune.json").exists()


@pytest.mark.parametrize("shapes", [((4, 4), (8, 2), 1), ((8, 1), (4, 4), 2), ((4, 2), (8, 4), 2)],
                         ids=["4x4-8x2-s1", "8x1-4x4-s2", "4x2-8x4-s2"])
def test_split_launch_shapes_match_single_shots(shapes):
    """Stress and velocity launches with different block decompositions."""
    (cs, ts_), (cv, tv), spt = shapes
    sims = _phantoms()
    shots = [fmc_shot_sources(s) for s in sims]
    with BatchStepper(sims, shots, block_cells=cs, nodes_per_thread=ts_, shots_per_thread=spt,
                      velocity_block_cells=cv, velocity_nodes_per_thread=tv) as b:
        b.run(sims[0]._n_steps)
        assert b.status()[2] == -1
        for q, sim in enumerate(sims):
            tr = b.traces(q)
            for s in (1, shots[q].shape[0] - 1):
                with _single_shot(sim, shots[q][s]) as one:
                    one.run(sim._n_steps)
                    want = one.read("traces")
                assert rel_l2(tr[s], want) <= TOL, (q, s, rel_l2(tr[s], want))


def test_focal_law_shots_match_single_shots():
    """Plane-wave steering laws (one delay per element) batched as shots of
    one launch: each shot equals the stepper run with that law's table."""
    from taichi_sim_gb300.batch import focal_law_shot_sources
    sims = _phantoms(steps=160)
    dt = float(sims[0]._dt)
    n_el = sims[0]._probes[0].num_elem
    ramp = np.arange(n_el, dtype=np.float64)
    laws = [np.zeros(n_el), ramp * 2 * dt, ramp[::-1] * 2 * dt, np.abs(ramp - (n_el - 1) / 2) * 3 * dt]
    shots = [focal_law_shot_sources(s, laws) for s in sims]
    assert not np.array_equal(shots[0][1], shots[0][2])
    with BatchStepper(sims, shots) as b:
        b.run(sims[0]._n_steps)
        assert b.status()[2] == -1
        for q, sim in enumerate(sims):
            tr = b.traces(q)
            for s in range(len(laws)):
                with _single_shot(sim, shots[q][s]) as one:
                    one.run(sim._n_steps)
                    want = one.read("traces")
                assert rel_l2(tr[s], want) <= TOL, (q, s, rel_l2(tr[s], want))


def test_law_file_runs_as_one_batched_launch(tmp_path):
    """A ``.law`` file named in the config: every law becomes a shot of one
    launch, each equal to the stepper run with that law's delays."""
    from taichi_sim_gb300.batch import focal_law_shot_sources, run_emission_laws
    from taichi_sim_gb300.sim_support.emission_law import EmissionLaw
    cfg = workloads.fmc2d_phantoms(n_steps=150, shapes=((80, 84),), n_elem=6, dx=0.1, pml=8)[0]
    cfg["probes"][0]["linear"].update(dim_a=0.3, inter_elem=0.1)
    dt = float(Simulator(cfg)._dt)
    delays = np.stack([np.arange(6) * k * dt for k in (0.0, 1.5, -1.5)]) + 3 * dt
    EmissionLaw().write_law(str(tmp_path / "steer"), delays)
    cfg["simul_configs"]["emission_laws"] = str(tmp_path / "steer.law")
    sim = Simulator(cfg)
    assert sim._emission_laws.shape == (3, 6)
    traces, fields = run_emission_laws(sim)
    assert traces.shape == (3, sim._n_steps, sim._n_rec) and fields.shape == (3,) + tuple(sim.grid_shape())
    tables = focal_law_shot_sources(sim, list(sim._emission_laws))
    for k in range(3):
        with _single_shot(sim, tables[k]) as one:
            one.run(sim._n_steps)
            want_tr, want_f = one.read("traces"), one.read("syy")
        assert rel_l2(traces[k], want_tr) <= TOL and rel_l2(fields[k], want_f) <= TOL


def test_driver_batched_run_matches_run_emission_laws(tmp_path):
    """The reference's driver with batched=True (2D viscoelastic backend):
    the last law's traces equal the batched launch's."""
    from taichi_sim_gb300.backends import SimulatorCudaViscoelastic
    from taichi_sim_gb300.batch import run_emission_laws
    from taichi_sim_gb300.sim_support.emission_law import EmissionLaw
    cfg = workloads.fmc2d_phantoms(n_steps=120, shapes=((80, 84),), n_elem=6, dx=0.1, pml=8)[0]
    cfg["probes"][0]["linear"].update(dim_a=0.3, inter_elem=0.1)
    dt = float(Simulator(cfg)._dt)
    EmissionLaw().write_law(str(tmp_path / "steer"), np.stack([np.arange(6) * k * dt for k in (0.0, 2.0)]) + 3 * dt)
    cfg["simul_configs"]["emission_laws"] = str(tmp_path / "steer.law")
    sim = SimulatorCudaViscoelastic(cfg)
    out = sim.run(batched=True)
    traces, _ = run_emission_laws(sim)
    np.testing.assert_array_equal(out["sens_stress"], traces[-1])
    assert np.abs(out["sens_stress"]).max() > 0
