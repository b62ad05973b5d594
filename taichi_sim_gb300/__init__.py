"""taichi_sim_gb300: GB300-native staggered-grid (visco)elastic time stepper.

* :mod:`taichi_sim_gb300.sim_support` - host model with the reference
  project's ``sim_support`` API (tables bit-identical to the reference's).
* :mod:`taichi_sim_gb300.engine` - ctypes binding of the C ABI
  (``include/taichi_sim_gb300.h``) and :class:`~taichi_sim_gb300.engine.Stepper`.
* :mod:`taichi_sim_gb300.backends` - drop-in ``Simulator`` subclasses whose
  ``implementation()`` runs the sm_103a kernels.
"""
__version__ = "0.1.0"
