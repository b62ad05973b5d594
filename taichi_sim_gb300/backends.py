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
With ``show_anim`` or ``save_snapshots`` set, ``implementation()`` also
returns ``"snapshots"``: the ROI of the field (3D: its middle y plane) after
every step the reference's live view shows, copied on the device as the run
goes (``ts_copy_field``, no synchronisation per frame), and
``"snapshot_steps"``.
The device state is created once and reset between shots; a new emission
law only re-uploads the source term.
"""
import time

import numpy as np

from . import engine
from .sim_support import StabilityError
from .sim_support.simulator import Simulator, snapshot_steps
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
        snaps = None
        if getattr(self, "_show_anim", False) or getattr(self, "_save_snapshots", False):
            snaps, steps = self._simulate_with_snapshots(st)
        else:
            st.simulate()
        st.status()
        sim_time = time.time() - t0
        field = st.read(self._field)
        traces = st.read("traces")
        res = {self._keys[0]: field, self._keys[1]: traces, "gpu_str": _gpu_name(), "sim_time": sim_time}
        if snaps is not None:
            res["snapshots"], res["snapshot_steps"] = snaps, steps
        return res

    def _snapshot_view(self, t):
        """The part of a field the live view shows: the ROI (3D: its middle y plane)."""
        roi = self._roi
        if self._dims == 2:
            return t[roi.get_ix_min():roi.get_ix_max(), roi.get_iz_min():roi.get_iz_max()]
        return t[roi.get_ix_min():roi.get_ix_max(), t.shape[1] // 2, roi.get_iz_min():roi.get_iz_max()]

    def _simulate_with_snapshots(self, st, check_every=256):
        """Run every step, copying the field on the device after each step
        the live view would show; stability is checked every
        ``check_every`` steps as in :meth:`engine.Stepper.simulate`."""
        import torch
        steps = snapshot_steps(self._n_steps, self._it_display)
        stream = torch.cuda.Stream()
        h = stream.cuda_stream
        stage = torch.empty(tuple(st.shape), dtype=torch.float32, device="cuda")
        stack = torch.empty((len(steps),) + tuple(self._snapshot_view(stage).shape), dtype=torch.float32,
                            device="cuda")
        done = checked = 0

        def check():
            _, vmax, bad = st.status()
            if bad >= 0:
                value = vmax if st.family == engine.TAICHI2D else float(np.sqrt(np.float32(vmax)))
                raise StabilityError("Simulacao tornando-se instavel", value)

        for i, s in enumerate(steps):
            st.run(s - done, stream=h)
            done = s
            st.copy_field(self._field, stage.data_ptr(), stream=h)
            with torch.cuda.stream(stream):
                stack[i].copy_(self._snapshot_view(stage))
            if done - checked >= check_every:
                check()
                checked = done
        if done < self._n_steps:
            st.run(self._n_steps - done, stream=h)
        check()
        stream.synchronize()
        return stack.cpu().numpy(), steps


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
