"""3D host model (``Simulator3D``).

Mirrors sim_support/Simulator3D.py of the reference: grid ``(nx, ny, nz)``
with z the ROI height, density averaged over the 8 surrounding nodes, CPML
vectors on three axes and receiver points with ``[ix, iy, iz, id]`` rows.
"""
from ._model import ModelBase
from .simulator import ExperimentDriver


class Simulator3D(ExperimentDriver, ModelBase):
    _dims = 3


__all__ = ["Simulator3D"]
