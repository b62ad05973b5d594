"""The parity cases exercise both sweeps of the single-shot step kernels:
warps wholly in the interior (no per-node region, strip or bounds tests) and
warps that touch a boundary strip or the grid edge (CPU-only check of the
case geometry)."""
import pytest

from _cases import interior_warps
from test_gpu_parity import CASES_2D, CASES_3D
from taichi_sim_gb300.sim_support.Simulator3D import Simulator3D
from taichi_sim_gb300.sim_support.simulator import Simulator


@pytest.mark.parametrize("name", sorted(CASES_2D))
def test_2d_cases_have_interior_warps(name):
    sim = Simulator(CASES_2D[name][0]())
    nx, ny = sim.grid_shape()
    for tx in (1, 2, 4):
        n = interior_warps(sim, tx)
        assert 0 < n < ((ny + 31) // 32) * ((nx + tx - 1) // tx)


def test_3d_cases_have_interior_warps():
    deep = [n for n in CASES_3D if interior_warps(Simulator3D(CASES_3D[n]()), 4) > 0]
    assert sorted(deep) == ["wgsl3d_acc4_deep", "wgsl3d_acc6_visco", "wgsl3d_visco_deep"]
    for n in deep:
        assert interior_warps(Simulator3D(CASES_3D[n]()), 2) > 0
