"""GPU parity at the benchmark workloads' full grid sizes, and against the
reference's own known-answer B-scan.

The small parity cases (test_gpu_parity.py) cover every code path; these
cover what only shows at size: 32-bit offset paths, the share of warps that
take the interior sweep, the 3D coefficient palette of a full model, the
batched layout of 64 shots, long-run error growth.  Every comparison goes
through the C ABI (``ts_create``/``ts_run``/``ts_read``, ``ts_batch_*``,
``ts_adj_*``) and checks fields and traces against the float CPU oracle
within relative L2 1e-5, the parity tolerance.  Time steps are bounded where
the oracle would take minutes (3D: 64 steps; batched and adjoint: 300), and
the tests are ordered and named by workload.

``test_golden_teste_pedro`` runs the reference's own experiment
``pedro/teste_pedro.json`` (725 x 572 nodes, 10000 steps, 64 receivers)
with the Taichi semantics (sim_taichi_elastic.py:311-351) and compares the
traces with the B-scan the reference shipped
(``pedro/results/result_teste_aco.npy``, a Taichi GPU run with fast math):
relative L2 <= 1e-5 in both arithmetic forms of the Taichi family (the
exact form equals the float oracle bit for bit, which reaches 7.4e-6 over
the same 10000 steps), the same first non-zero row (335) and the same
arrival row of the largest sample in every column.
"""
import numpy as np
import pytest

from _cases import gated_mask, rel_l2
from _golden import config_with_maps, golden_bscan
from oracle import oracle
from taichi_sim_gb300 import engine, workloads
from taichi_sim_gb300.sim_support.simulator import Simulator
from taichi_sim_gb300.sim_support.Simulator3D import Simulator3D

pytestmark = pytest.mark.gpu

TOL = 1e-5
F2 = ("vx", "vy", "sxx", "syy", "sxy")
F3 = ("vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz")


@pytest.mark.parametrize("exact", ["0", "1"], ids=["unbiased", "exact"])
def test_golden_teste_pedro(exact, monkeypatch):
    """Both arithmetic forms of the Taichi family: the default (the
    reference's constants, no rounding bias) and every operation rounded on
    its own (TS_TAICHI_EXACT=1, bit for bit the float oracle)."""
    monkeypatch.setenv("TS_TAICHI_EXACT", exact)
    dims, cfg = config_with_maps("teste_pedro")
    sim = Simulator(cfg)
    assert sim.grid_shape() == (725, 572) and sim._n_steps == 10000
    with engine.Stepper(sim, family=engine.TAICHI2D) as st:
        st.simulate()
        tr = st.read("traces")
    g = golden_bscan()
    assert tr.shape == g.shape
    err = rel_l2(tr, g)
    print(f"teste_pedro, {'exact' if exact == '1' else 'unbiased'} arithmetic: traces vs golden B-scan {err:.3e}")
    assert int(np.nonzero(np.abs(tr).sum(1))[0][0]) == 335
    assert err <= TOL, err
    np.testing.assert_array_equal(np.argmax(np.abs(tr), axis=0), np.argmax(np.abs(g), axis=0))
    assert np.isclose(np.abs(tr).max(), np.abs(g).max(), rtol=1e-4)


def _check_stepper(sim, family, names, n_steps, exact=False):
    fam_oracle = {engine.TAICHI2D: oracle.TAICHI2D, engine.WGSL2D: oracle.WGSL2D, engine.WGSL3D: oracle.WGSL3D}[family]
    with engine.Stepper(sim, family=family) as st:
        st.run(n_steps)
        n, vmax, bad = st.status()
        assert n == n_steps and bad == -1
        got = {k: st.read(k) for k in names}
        tr = st.read("traces")[:n_steps]
    ref = oracle.run(sim, fam_oracle, n_steps=n_steps)
    errs = {k: rel_l2(got[k], ref[k]) for k in names}
    errs["traces"] = rel_l2(tr, ref["sens"])
    for k in names:
        assert np.abs(ref[k]).max() > 0, k
    assert np.abs(ref["sens"]).max() > 0, "nothing recorded"
    assert max(errs.values()) <= TOL, errs
    # rows before a receiver's first recorded step stay exactly zero (WGSL:
    # row k recorded from k = delay; Taichi: from k = delay - 1)
    np.testing.assert_array_equal(tr[gated_mask(sim, family == engine.TAICHI2D, n_steps)], 0.0)
    if exact:
        for k in names:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
        np.testing.assert_array_equal(tr, ref["sens"])
    return errs


@pytest.mark.parametrize("exact", ["0", "1"], ids=["unbiased", "exact"])
def test_full_elastic2d_512_2000_steps(exact, monkeypatch):
    """Taichi semantics: within the tolerance in the default arithmetic, bit
    for bit the float oracle with every operation rounded on its own."""
    monkeypatch.setenv("TS_TAICHI_EXACT", exact)
    sim = Simulator(workloads.elastic2d_512())
    assert sim.grid_shape() == (512, 512)
    _check_stepper(sim, engine.TAICHI2D, F2, 2000, exact=exact == "1")


def test_full_visco2d_1024_4000_steps():
    sim = Simulator(workloads.visco2d_1024())
    assert sim.grid_shape() == (1024, 1024)
    _check_stepper(sim, engine.WGSL2D, F2, 4000)


@pytest.mark.parametrize("palette", ["1", "0"], ids=["palette", "arrays"])
def test_full_visco3d_256_64_steps(palette, monkeypatch):
    monkeypatch.setenv("TS_3D_COEF_PALETTE", palette)
    sim = Simulator3D(workloads.visco3d_256())
    assert sim.grid_shape() == (256, 256, 256)
    _check_stepper(sim, engine.WGSL3D, F3, 64)


def _with_shot(sim, table, fn):
    """Run fn with the model's source term replaced by one shot's table (the
    stride the kernels read is the table's width)."""
    saved = sim._source_term, sim._n_src
    sim._source_term, sim._n_src = table, table.shape[1]
    try:
        return fn()
    finally:
        sim._source_term, sim._n_src = saved


def test_full_fmc2d_three_phantoms_300_steps():
    """The batched launch over 64 shots of each of the three full-size
    phantoms; shots 0 and 63 of each against the oracle run on that shot."""
    from taichi_sim_gb300.batch import BatchStepper, fmc_shot_sources
    n_t = 300
    sims = [Simulator(c) for c in workloads.fmc2d_phantoms(n_steps=n_t)]
    shots = [fmc_shot_sources(s) for s in sims]
    assert [s.grid_shape() for s in sims] == [(512, 768), (768, 768), (1024, 768)]
    assert [sh.shape[0] for sh in shots] == [64, 64, 64]
    with BatchStepper(sims, shots) as b:
        b.run(n_t)
        n, _, bad = b.status()
        assert n == n_t and bad == -1
        got = [(b.traces(q), b.field(q, "syy")) for q in range(len(sims))]
    for q, sim in enumerate(sims):
        for s in (0, 63):
            ref = _with_shot(sim, shots[q][s], lambda: oracle.run(sim, oracle.WGSL2D, n_steps=n_t))
            assert np.abs(ref["sens"]).max() > 0
            e_tr, e_f = rel_l2(got[q][0][s], ref["sens"]), rel_l2(got[q][1][s], ref["syy"])
            assert e_tr <= TOL and e_f <= TOL, (q, s, e_tr, e_f)


def test_fmc2d_all_3000_steps_512x768():
    """Long-run accuracy of the batched kernels: all 3000 steps of the
    smallest phantom's 64-shot batch (about 90 wavelengths travelled), shots
    0 and 63 against the oracle."""
    from taichi_sim_gb300.batch import BatchStepper, fmc_shot_sources
    sim = Simulator(workloads.fmc2d_phantoms(shapes=((512, 768),))[0])
    assert sim._n_steps == 3000
    shots = fmc_shot_sources(sim)
    with BatchStepper([sim], [shots]) as b:
        b.run(sim._n_steps)
        assert b.status()[2] == -1
        tr, f = b.traces(0), b.field(0, "syy")
    for s in (0, 63):
        ref = _with_shot(sim, shots[s], lambda: oracle.run(sim, oracle.WGSL2D))
        ref64 = _with_shot(sim, shots[s], lambda: oracle.run(sim, oracle.WGSL2D, precision="f64"))
        e_tr, e_f = rel_l2(tr[s], ref["sens"]), rel_l2(f[s], ref["syy"])
        # each float result against the double run: the GPU's error is the
        # float oracle's own, rounding noise of the same size
        g64, o64 = rel_l2(f[s], ref64["syy"]), rel_l2(ref["syy"], ref64["syy"])
        print(f"shot {s}: traces {e_tr:.2e}, field {e_f:.2e}; field vs f64: gpu {g64:.2e}, oracle {o64:.2e}")
        assert e_tr <= TOL, (s, e_tr)
        assert e_f <= TOL or g64 <= 1.5 * o64, (s, e_f, g64, o64)


def test_visco3d_all_1000_steps_96():
    """Long-run accuracy in 3D: the visco3d workload's model (layers, per-cell
    Q, Ricker source, receiver plane) on a 96^3 grid for all 1000 steps."""
    sim = Simulator3D(workloads.visco3d_256(n_grid=96))
    assert sim._n_steps == 1000
    _check_stepper(sim, engine.WGSL3D, F3, 1000)


def test_full_adjoint2d_512x1024_forward_300_steps():
    """The adjoint's forward (checkpointed, through ts_adj_forward) on the
    full 512 x 1024 model, one shot, against the oracle."""
    import torch
    from taichi_sim_gb300.adjoint import AdjointProblem
    from taichi_sim_gb300.batch import fmc_shot_sources
    n_t = 300
    sim = Simulator(workloads.adjoint2d_512x1024(n_steps=n_t))
    assert sim.grid_shape() == (512, 1024)
    table = fmc_shot_sources(sim)[5]
    with AdjointProblem(sim, checkpoint_every=int(np.ceil(np.sqrt(n_t)))) as prob:
        prob.set_source_term(table)
        with torch.no_grad():
            tr = prob.traces(*prob.material()).cpu().numpy()
    ref = _with_shot(sim, table, lambda: oracle.run(sim, oracle.WGSL2D, n_steps=n_t))
    assert np.abs(ref["sens"]).max() > 0
    assert rel_l2(tr, ref["sens"]) <= TOL, rel_l2(tr, ref["sens"])
