"""ExperimentDriver.run() on the CPU with stand-in implementations: the
reference's per-(iteration, law) loop, its result files
(sim_support/simulator.py:321-605) and the batched variant."""
import glob
import os

import numpy as np
import pytest

from _cases import case_2d
from taichi_sim_gb300.sim_support.emission_law import EmissionLaw
from taichi_sim_gb300.sim_support.simulator import Simulator


class FakeBackend(Simulator):
    """implementation() returns a field and traces that encode the call."""

    def __init__(self, cfg):
        super().__init__(cfg, sim_type="viscoelastic")
        self._name = "fake"
        self.calls, self.batched_calls, self.t0_seen = 0, 0, []

    def _result(self, k):
        field = np.full((self._nx, self._ny), float(k), np.float32)
        traces = np.full((self._n_steps, self._n_rec), float(k) + 0.5, np.float32)
        return {"stress": field, "sens_stress": traces, "gpu_str": "fake GPU", "sim_time": 0.01}

    def implementation(self):
        super().implementation()
        self.t0_seen.append(np.array(self._probes[0]._t0_emission, copy=True))
        self.calls += 1
        return self._result(self.calls)

    def implementation_batched(self, laws):
        self.batched_calls += 1
        return [self._result(100 + k) for k in range(len(laws))]


def _cfg(tmp_path, laws=None, n_iter=1):
    cfg = case_2d(visco=1, steps=50)
    sc = cfg["simul_configs"]
    sc.update(n_iter=n_iter, save_results=1, save_field=1, save_bscan=1, results_dir=str(tmp_path))
    if laws is not None:
        EmissionLaw().write_law(str(tmp_path / "laws"), np.asarray(laws))
        sc["emission_laws"] = str(tmp_path / "laws.law")
    return cfg


def test_run_saves_one_field_and_bscan_per_law_and_iteration(tmp_path):
    sim = FakeBackend(_cfg(tmp_path, n_iter=2))
    out = sim.run()
    assert sim.calls == 2 and out["sens_stress"][0, 0] == 2.5
    fields = sorted(glob.glob(str(tmp_path / "result_fake_*_field_stress_yy.npy")))
    bscans = sorted(glob.glob(str(tmp_path / "result_fake_*_bscan_stress.npy")))
    assert len(fields) == 2 and len(bscans) == 2
    assert [os.path.basename(f).split("_iter_")[1] for f in fields] == ["0_law_0_field_stress_yy.npy",
                                                                      "1_law_0_field_stress_yy.npy"]
    np.testing.assert_array_equal(np.load(fields[1]), np.full((sim._nx, sim._ny), 2.0, np.float32))
    desc = glob.glob(str(tmp_path / "*_desc.txt"))
    csv = glob.glob(str(tmp_path / "*GPU_.csv"))
    assert len(desc) == 1 and len(csv) == 1
    text = open(desc[0]).read()
    assert "Simulador: fake" in text and f"Tamanho da ROI: {sim._nx}x{sim._ny}" in text
    assert np.loadtxt(csv[0], delimiter=",").shape == (2,)


def test_run_sets_each_law_before_its_implementation(tmp_path):
    n_el = FakeBackend(_cfg(tmp_path))._probes[0].num_elem
    laws = [np.full(n_el, 0.3), np.linspace(0.3, 0.6, n_el)]
    sim = FakeBackend(_cfg(tmp_path, laws=laws))
    sim.run()
    assert sim.calls == 2 and sim.batched_calls == 0
    for seen, law in zip(sim.t0_seen, laws):
        np.testing.assert_allclose(seen, law, rtol=1e-6)
    assert len(glob.glob(str(tmp_path / "result_fake_*_law_1_bscan_stress.npy"))) == 1


def test_batched_run_computes_every_law_of_an_iteration_together(tmp_path):
    n_el = FakeBackend(_cfg(tmp_path))._probes[0].num_elem
    laws = [np.full(n_el, 0.3), np.linspace(0.3, 0.6, n_el), np.linspace(0.6, 0.3, n_el)]
    sim = FakeBackend(_cfg(tmp_path, laws=laws, n_iter=2))
    out = sim.run(batched=True)
    assert sim.calls == 0 and sim.batched_calls == 2
    bscans = sorted(glob.glob(str(tmp_path / "result_fake_*_bscan_stress.npy")))
    assert len(bscans) == 6
    law2 = [b for b in bscans if "_iter_1_law_2_" in b]
    np.testing.assert_array_equal(np.load(law2[0]), np.full((sim._n_steps, sim._n_rec), 102.5, np.float32))
    assert out["sens_stress"][0, 0] == 102.5


def test_models_without_a_batched_backend_refuse_batched_runs(tmp_path):
    sim = Simulator(_cfg(tmp_path), sim_type="viscoelastic")
    with pytest.raises(NotImplementedError):
        sim.run(batched=True)


def test_cuda_backend_batches_the_laws_through_the_batched_stepper(tmp_path, monkeypatch):
    """The 2D viscoelastic backend's implementation_batched, with a stand-in
    for the batched stepper (no GPU): one shot per law, its table built from
    the law's delays, results under the backend's keys."""
    from taichi_sim_gb300 import backends, batch

    seen = {}

    class FakeBatch:
        def __init__(self, sims, shots):
            seen["shots"] = shots[0]
            self.sim, self.n = sims[0], shots[0].shape[0]

        def run(self, n):
            seen["steps"] = n

        def status(self):
            return self.sim._n_steps, 0.0, -1

        def traces(self, q):
            return np.arange(self.n, dtype=np.float32)[:, None, None] * np.ones((1, self.sim._n_steps, self.sim._n_rec))

        def field(self, q, what):
            seen["field"] = what
            return np.zeros((self.n,) + tuple(self.sim.grid_shape()), np.float32)

        def __enter__(self):
            return self

        def __exit__(self, *exc):
            pass

    monkeypatch.setattr(batch, "BatchStepper", FakeBatch)
    sim = backends.SimulatorCudaViscoelastic(_cfg(tmp_path))
    n_el = sim._probes[0].num_elem
    out = sim.implementation_batched([None])
    assert len(out) == 1 and seen["steps"] == sim._n_steps and seen["field"] == "syy"
    np.testing.assert_array_equal(seen["shots"][0], np.asarray(sim._source_term, np.float32))
    laws = [np.full(n_el, 0.3, np.float32), np.linspace(0.3, 0.6, n_el).astype(np.float32)]
    out = sim.implementation_batched(laws)
    assert [set(r) for r in out] == [{"stress", "sens_stress", "gpu_str", "sim_time"}] * 2
    np.testing.assert_array_equal(seen["shots"], batch.focal_law_shot_sources(sim, laws))
    assert out[1]["sens_stress"][0, 0] == 1.0


def test_snapshot_steps_follow_the_live_view():
    from taichi_sim_gb300.sim_support.simulator import snapshot_steps
    assert snapshot_steps(240, 50) == [5, 50, 100, 150, 200]
    assert snapshot_steps(100, 5) == list(range(5, 101, 5))
    assert snapshot_steps(4, 10) == []
    assert snapshot_steps(30, 0) == list(range(1, 31))


class SnapshotBackend(FakeBackend):
    """A stand-in backend that returns the live view's frames."""

    def _result(self, k):
        from taichi_sim_gb300.sim_support.simulator import snapshot_steps
        res = super()._result(k)
        steps = snapshot_steps(self._n_steps, self._it_display)
        res["snapshots"] = np.stack([np.full((3, 4), float(s), np.float32) for s in steps])
        res["snapshot_steps"] = steps
        return res


def test_run_saves_snapshots_when_a_backend_returns_them(tmp_path):
    cfg = _cfg(tmp_path)
    cfg["simul_configs"]["save_snapshots"] = 1
    sim = SnapshotBackend(cfg)
    assert sim._save_snapshots
    sim.run()
    snaps = glob.glob(str(tmp_path / "result_fake_*_snapshots_stress.npy"))
    steps = glob.glob(str(tmp_path / "result_fake_*_snapshot_steps.npy"))
    assert len(snaps) == 1 and len(steps) == 1
    s, k = np.load(snaps[0]), np.load(steps[0])
    np.testing.assert_array_equal(k, [5, 50])   # 50 steps, it_display 50
    np.testing.assert_array_equal(s[:, 0, 0], [5.0, 50.0])
