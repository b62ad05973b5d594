"""Drop-in backends: ``Simulator`` subclasses whose ``implementation()`` runs
the GB300 kernels.

They follow the reference's plugin contract (sim_support/simulator.py:608-611
and the three backends): construct with a config path, ``run()`` calls
``implementation()`` once per (iteration, emission law), and
``implementation()`` returns

* :class:`SimulatorCudaElastic` (semantics of sim_taichi_elastic.py:19-351):
  ``{"pressure": final syy, "sens_pressure": traces, "gpu_str", "sim_time"}``
* :class:`SimulatorCudaViscoelastic` (sim_webgpu_viscoelastic.py:20-555) and
  :class:`SimulatorCuda3DViscoelastic` (sim_webgpu_3D_viscoelastic.py:20-713):
  ``{"stress": final syy (2D) / szz (3D), "sens_stress": traces, "gpu_str",
  "sim_time"}``

``sim_time`` is the wall time of the step loop, as in the reference.
``StabilityError`` is raised when the velocity norm breaks the threshold.
The device state is created once and reset between shots; a new emission
law only re-uploads the source term.
"""
import time

import numpy as np

from . import engine
from .sim_support.simulator import Simulator
from .sim_support.Simulator3D import Simulator3D


def _gpu_name():
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "CUDA device"


class _CudaBackend:
    _family = engine.WGSL2D
    _field = "syy"
    _keys = ("stress", "sens_stress")

    def _stepper(self):
        st = getattr(self, "_ts_stepper", None)
        if st is None:
            st = engine.Stepper(self, family=self._family)
            self._ts_stepper = st
        else:
            # The reference builds the source term once, in the constructor,
            # so a later set_t0() does not change what is injected
            # (sim_support/simulator.py:329-337); re-sent as is.
            st.reset()
            st.set_sources(self._source_term)
        return st

    def implementation(self):
        super().implementation()
        st = self._stepper()
        t0 = time.time()
        st.simulate()
        st.status()
        sim_time = time.time() - t0
        field = st.read(self._field)
        traces = st.read("traces")
        return {self._keys[0]: field, self._keys[1]: traces, "gpu_str": _gpu_name(), "sim_time": sim_time}


class SimulatorCudaElastic(_CudaBackend, Simulator):
    """2D isotropic elastic stepper with the Taichi backend's semantics."""

    _family = engine.TAICHI2D
    _keys = ("pressure", "sens_pressure")

    def __init__(self, file_config):
        super().__init__(file_config)
        self._name = "CUDA-split-elastic"


class SimulatorCudaViscoelastic(_CudaBackend, Simulator):
    """2D (visco)elastic stepper with the WebGPU backend's semantics."""

    _family = engine.WGSL2D

    def __init__(self, file_config):
        super().__init__(file_config, sim_type="viscoelastic")
        self._name = "CUDA-viscoelastic"

    def implementation_batched(self, laws):
        """Every emission law as a shot of one batched launch
        (:class:`~taichi_sim_gb300.batch.BatchStepper`); ``None`` runs the
        source term as built.  One result dict per law, with the keys of
        :meth:`implementation` and ``sim_time`` the launch's share per law."""
        from .batch import BatchStepper, focal_law_shot_sources
        laws = list(laws)
        if len(laws) == 1 and laws[0] is None:
            st = np.asarray(self._source_term, np.float32)
            shots = (st[:, None] if st.ndim == 1 else st)[None]
        else:
            shots = focal_law_shot_sources(self, laws)
        t0 = time.time()
        with BatchStepper([self], [shots]) as b:
            b.run(self._n_steps)
            _, vmax, bad = b.status()
            if bad >= 0:
                raise engine.StabilityError("Simulacao tornando-se instavel", float(np.sqrt(np.float32(vmax))))
            traces, fields = b.traces(0), b.field(0, self._field)
        sim_time = (time.time() - t0) / len(shots)
        return [{self._keys[0]: fields[k], self._keys[1]: traces[k], "gpu_str": _gpu_name(), "sim_time": sim_time}
                for k in range(len(shots))]


class SimulatorCuda3DViscoelastic(_CudaBackend, Simulator3D):
    """3D (visco)elastic stepper with the WebGPU 3D backend's semantics."""

    _family = engine.WGSL3D
    _field = "szz"

    def __init__(self, file_config):
        super().__init__(file_config, sim_type="viscoelastic")
        self._name = "CUDA-3D-viscoelastic"


__all__ = ["SimulatorCudaElastic", "SimulatorCudaViscoelastic", "SimulatorCuda3DViscoelastic"]
