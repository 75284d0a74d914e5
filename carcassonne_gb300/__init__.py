"""carcassonne_gb300: the center-site optimisation path of gcross/Carcassonne on
one NVIDIA GB300 (sm_103a).

Python host code over torch CUDA tensors calls libcarcgb300.so (hand-written
CUDA kernels behind a C ABI, include/carcassonne_gb300.h).  The submodules
keep the reference's layout and names: ``data``, ``sparse``,
``tensors._2d.dense``, ``tensors._2d.sparse``, ``compression``, ``system``
and ``utils``.
"""
__version__ = "0.1.0"
