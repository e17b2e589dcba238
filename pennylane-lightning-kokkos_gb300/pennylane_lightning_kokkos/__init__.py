"""GB300-native state-vector core behind the LightningKokkos interface.

``lightning_kokkos_qubit_ops`` (pybind11) keeps the reference module's class
surface (``LightningKokkos_C64/C128``, the observable classes,
``AdjointJacobianKokkos_*``); ``_native`` is the ctypes view of the C ABI in
``include/plk_gb300.h``.  Both run hand-written sm_103a kernels from
``libplk_gb300.so``; there is no CPU fallback.
"""
__version__ = "0.33.0-gb300"
