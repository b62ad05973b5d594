"""GPU adjoint gradient (through the C ABI's ts_adj_* calls) against the FP64
autograd oracle, central finite differences and the CPU forward oracle.

Tolerances: the adjoint's forward traces within 1e-5 relative L2 of the
float oracle (the stepper's bound); gradients with respect to per-cell
lambda, mu and rho within 1e-3 relative L2 of FP64 autograd through the
torch transcription of the same discrete forward; directional derivatives
within 1e-3 of FP64 central differences of that forward.
"""
import numpy as np
import pytest
import torch

from _cases import case_2d, case_adjoint, rel_l2
from oracle import oracle
from oracle.torch_wgsl2d import Wgsl2D
from taichi_sim_gb300.adjoint import AdjointProblem, l2_misfit
from taichi_sim_gb300.batch import fmc_shot_sources
from taichi_sim_gb300.sim_support.simulator import Simulator

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-3

FWD_CASES = {
    "visco": dict(visco=1),
    "elastic": dict(visco=0),
    "visco_q": dict(visco=1, q=(30.0, 200.0), seed=1),
    "acc4": dict(visco=1, acc=4, seed=3),
    "delayed_rx": dict(visco=1, t0_rx=0.2, seed=2),
}


@pytest.mark.parametrize("ckpt", [0, 17])
@pytest.mark.parametrize("name", sorted(FWD_CASES))
def test_adjoint_forward_matches_oracle(name, ckpt):
    sim = Simulator(case_2d(steps=240, **FWD_CASES[name]))
    ref = oracle.run(sim, oracle.WGSL2D)
    with AdjointProblem(sim, checkpoint_every=ckpt) as prob:
        with torch.no_grad():
            tr = prob.traces(*prob.material()).cpu().numpy()
    assert np.abs(ref["sens"]).max() > 0
    assert rel_l2(tr, ref["sens"]) <= 1e-5


def _problem_pair(w, h, steps, **kw):
    true = Simulator(case_adjoint(w=w, h=h, steps=steps, **kw))
    start = Simulator(case_adjoint(w=w, h=h, steps=steps, true_model=False, **kw))
    return true, start


@pytest.mark.parametrize("kw", [dict(visco=1), dict(visco=0), dict(visco=1, q=(30.0, 200.0))],
                         ids=["visco", "elastic", "visco_q"])
def test_gradient_matches_fp64_autograd(kw):
    """128 x 128 nodes, 400 steps: the GPU gradient w.r.t. per-cell lambda,
    mu, rho against FP64 autograd through the torch transcription."""
    true, start = _problem_pair(128, 128, 400, **kw)
    w = Wgsl2D(start)
    with torch.no_grad():
        obs64 = w.traces(*w.material(true))
    m64 = [t.clone().requires_grad_(True) for t in w.material(start)]
    l2_misfit(w.traces(*m64), obs64).backward()
    with AdjointProblem(start) as prob:
        m = [t.clone().requires_grad_(True) for t in prob.material()]
        J = l2_misfit(prob.traces(*m), obs64.to(prob.device, torch.float32))
        J.backward()
        for name, a, b in zip(("lambda", "mu", "rho"), m, m64):
            err = rel_l2(a.grad.cpu().numpy(), b.grad.numpy())
            assert np.abs(b.grad.numpy()).max() > 0
            assert err <= GRAD_TOL, (name, err)


def test_gradient_matches_central_differences():
    """128 x 128 nodes, 400 steps: directional derivatives <grad J, d> of the
    GPU adjoint against FP64 central differences of the same discrete
    forward (the torch transcription), d a smooth bump in each parameter."""
    true, start = _problem_pair(128, 128, 400)
    w = Wgsl2D(start)
    with torch.no_grad():
        obs64 = w.traces(*w.material(true))
        m64 = w.material(start)
    with AdjointProblem(start) as prob:
        m = [t.clone().requires_grad_(True) for t in prob.material()]
        l2_misfit(prob.traces(*m), obs64.to(prob.device, torch.float32)).backward()
        grads = [t.grad.double().cpu() for t in m]
    nx, ny = start.grid_shape()
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    bump = torch.as_tensor(np.exp(-((X - 0.55 * nx) ** 2 + (Y - 0.6 * ny) ** 2) / (2 * (0.12 * nx) ** 2)))

    def J(ms):
        with torch.no_grad():
            return float(l2_misfit(w.traces(*ms), obs64))

    for k in range(3):
        d = bump * m64[k].abs().mean() * 1e-4
        mp, mm = list(m64), list(m64)
        mp[k], mm[k] = m64[k] + d, m64[k] - d
        fd = (J(mp) - J(mm)) / 2
        an = float((grads[k] * d).sum())
        assert abs(fd - an) <= GRAD_TOL * abs(an), (k, fd, an)


def test_checkpointing_matches_store_all():
    """Recomputing K-step segments from checkpoints (with 1, 3 or all
    trailing segments recorded by the forward pass) gives the gradient of
    keeping every step's features."""
    true, start = _problem_pair(64, 64, 150)
    grads = []
    with AdjointProblem(true, checkpoint_every=0) as pt, torch.no_grad():
        obs = pt.traces(*pt.material()).clone()
    # (checkpoint interval, trailing segments recorded by the forward pass)
    for ckpt, segs in ((0, 1), (7, 1), (13, 1), (None, 1), (13, 3), (7, 50)):
        with AdjointProblem(start, checkpoint_every=ckpt, record_segments=segs) as prob:
            m = [t.clone().requires_grad_(True) for t in prob.material()]
            l2_misfit(prob.traces(*m), obs).backward()
            grads.append([t.grad.cpu().numpy() for t in m])
    for g in grads[1:]:
        for a, b in zip(g, grads[0]):
            assert rel_l2(a, b) <= 1e-6


def test_repeated_backward_recomputes_the_last_segment():
    """The forward pass records the last segment for the first backward; a
    second backward of the same forward recomputes it from its checkpoint
    and gives the same coefficient gradients bit for bit."""
    true, start = _problem_pair(64, 64, 150)
    with AdjointProblem(true, checkpoint_every=0) as pt, torch.no_grad():
        obs = pt.traces(*pt.material()).clone()
    with AdjointProblem(start, checkpoint_every=13) as prob:
        coefs = prob.node_coefficients(*prob.material())
        traces, token = prob.forward_raw(*coefs)
        residual = (traces - obs.to(traces.device)).contiguous()
        first = [g.clone() for g in prob.backward_raw(residual, token)]
        second = prob.backward_raw(residual, token)
        for a, b in zip(first, second):
            assert torch.equal(a, b)
        assert max(float(a.abs().max()) for a in first) > 0


def test_shot_gradients_add_up():
    """Shots through one problem: set_source_term between shots, gradients
    accumulate in .grad; a backward after another forward is refused."""
    true, start = _problem_pair(64, 64, 150, n_elem=4)
    shots = fmc_shot_sources(start)
    with AdjointProblem(true) as pt, AdjointProblem(start) as prob:
        m = [t.clone().requires_grad_(True) for t in prob.material()]
        per_shot = []
        for s in range(2):
            pt.set_source_term(shots[s])
            prob.set_source_term(shots[s])
            with torch.no_grad():
                obs = pt.traces(*pt.material()).clone()
            mm = [t.detach().clone().requires_grad_(True) for t in m]
            l2_misfit(prob.traces(*mm), obs).backward()
            l2_misfit(prob.traces(*m), obs).backward()
            per_shot.append([t.grad.cpu().numpy() for t in mm])
        for k in range(3):
            assert rel_l2(m[k].grad.cpu().numpy(), per_shot[0][k] + per_shot[1][k]) <= 1e-6
        tr1 = prob.traces(*m)
        prob.traces(*[t.detach() for t in m])
        with pytest.raises(RuntimeError):
            l2_misfit(tr1, obs).backward()
