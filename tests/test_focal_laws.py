"""Focal-law shots: per-shot source tables built from emission delays (CPU)."""
import numpy as np

from _cases import case_2d
from taichi_sim_gb300.batch import focal_law_shot_sources
from taichi_sim_gb300.sim_support.simulator import Simulator


def test_the_model_delays_give_the_model_source_term():
    sim = Simulator(case_2d(visco=1, steps=200))
    tables = focal_law_shot_sources(sim, [np.array(sim._probes[0]._t0_emission)])
    np.testing.assert_array_equal(tables[0], sim._source_term)


def test_delays_shift_each_element_and_restore_the_probe():
    sim = Simulator(case_2d(visco=1, steps=400))
    probe = sim._probes[0]
    n_el = probe.num_elem
    before = np.array(probe._t0_emission, copy=True)
    dt = float(sim._dt)
    k = np.arange(n_el) * 3                      # element e delayed by 3 e samples more
    t0 = before.astype(np.float64)
    tables = focal_law_shot_sources(sim, [t0.astype(np.float32), (t0 + k * dt).astype(np.float32)])
    base, shifted = tables[0], tables[1]
    for e in range(n_el):
        if k[e] == 0:
            np.testing.assert_array_equal(shifted[:, e], base[:, e])
        else:
            a, b = shifted[k[e]:, e].astype(np.float64), base[:-k[e], e].astype(np.float64)
            assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b)   # same wavelet, k[e] samples later
    np.testing.assert_array_equal(probe._t0_emission, before)   # restored
    np.testing.assert_array_equal(base, sim._source_term)


def test_a_model_without_laws_needs_laws():
    import pytest
    from taichi_sim_gb300.batch import run_emission_laws
    sim = Simulator(case_2d(visco=1, steps=50))
    with pytest.raises(ValueError):
        run_emission_laws(sim)


def test_plane_wave_and_focused_laws():
    from taichi_sim_gb300.batch import focused_laws, plane_wave_laws
    sim = Simulator(case_2d(visco=1, steps=200))
    probe = sim._probes[0]
    n_el = probe.num_elem
    base = float(np.min(probe._t0_emission))
    laws = plane_wave_laws(sim, [0.0, 10.0, -10.0], c=5.9)
    assert laws.shape == (3, n_el)
    np.testing.assert_allclose(laws[0], base, atol=1e-6)           # normal incidence: all together
    assert np.all(np.diff(laws[1]) > 0) and np.all(np.diff(laws[2]) < 0)
    np.testing.assert_allclose(laws[1], laws[2][::-1], atol=1e-6)  # mirror images
    pitch = float(probe.pitch)
    np.testing.assert_allclose(np.diff(laws[1]), pitch * np.sin(np.deg2rad(10.0)) / 5.9, rtol=1e-4)
    assert laws[1].min() == np.float32(base)
    cx = float(np.asarray(probe.coord_center).ravel()[0])
    foc = focused_laws(sim, [(cx, 2.0)], c=5.9)[0]
    np.testing.assert_allclose(foc, foc[::-1], atol=1e-6)           # symmetric about the centre
    assert foc[n_el // 2] > foc[0] and np.isclose(foc.min(), base)  # the centre fires last
    tables = focal_law_shot_sources(sim, laws)
    assert tables.shape[0] == 3 and not np.array_equal(tables[1], tables[2])
