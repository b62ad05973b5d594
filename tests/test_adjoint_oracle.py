"""The FP64 torch transcription of the WGSL 2D step (the adjoint's autograd
oracle), pinned to the C oracle and checked for differentiability on CPU."""
import numpy as np
import pytest
import torch

from _cases import case_2d, case_adjoint, rel_l2
from oracle import oracle
from oracle.torch_wgsl2d import Wgsl2D
from taichi_sim_gb300.sim_support.simulator import Simulator


@pytest.mark.parametrize("kw", [dict(visco=1), dict(visco=0), dict(visco=1, q=(30.0, 200.0), seed=1),
                                dict(visco=1, acc=4, seed=3), dict(visco=1, t0_rx=0.2, seed=2)],
                         ids=["visco", "elastic", "visco_q", "acc4", "delayed_rx"])
def test_torch_transcription_matches_c_oracle(kw):
    """Same traces as the C oracle's double-precision run (which the golden
    B-scan pins) to rounding."""
    sim = Simulator(case_2d(steps=100, **kw))
    ref = oracle.run(sim, oracle.WGSL2D, precision="f64")
    w = Wgsl2D(sim)
    with torch.no_grad():
        tr = w.traces(*w.material(sim)).numpy()
    assert np.abs(ref["sens"]).max() > 0
    assert rel_l2(tr, ref["sens"]) < 1e-12


def test_autograd_oracle_matches_central_differences():
    """Autograd through the transcription agrees with FP64 central
    differences of the same forward (directional derivatives)."""
    true = Simulator(case_adjoint(w=36, h=36, steps=80))
    start = Simulator(case_adjoint(w=36, h=36, steps=80, true_model=False))
    w = Wgsl2D(start)
    with torch.no_grad():
        obs = w.traces(*w.material(true))
    m = [t.clone().requires_grad_(True) for t in w.material(start)]
    J = 0.5 * ((w.traces(*m) - obs) ** 2).sum()
    J.backward()
    rng = np.random.default_rng(0)
    for k in range(3):
        d = torch.as_tensor(rng.standard_normal(m[k].shape)) * m[k].detach().abs().mean() * 1e-4
        with torch.no_grad():
            mp = [x.detach().clone() for x in m]
            mm = [x.detach().clone() for x in m]
            mp[k] += d
            mm[k] -= d
            fd = (0.5 * ((w.traces(*mp) - obs) ** 2).sum() - 0.5 * ((w.traces(*mm) - obs) ** 2).sum()) / 2
        an = (m[k].grad * d).sum()
        assert abs(fd.item() - an.item()) <= 1e-5 * abs(an.item()), (k, fd.item(), an.item())
