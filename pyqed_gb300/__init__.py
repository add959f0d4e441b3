"""GB300-native Lindblad master-equation propagator.

Drop-in for ``pyqed.oqs.LindbladSolver`` (binggu56/pyqed, ``pyqed/oqs.py``):
the Python surface mirrors the reference; the RK4 propagation runs in
hand-written sm_103a CUDA kernels behind the C ABI of
``include/lindblad_gb300.h``.
"""
from .mol import Result, load_result
from .oqs import LindbladSolver, liouvillian
from .batch import propagate_batch, correlation_batch
from .redfield import RedfieldSolver, redfield_batch
from .heom import HEOMSolver, heom_batch
from .spectral import Lindblad_solver
from . import workloads

__all__ = ["LindbladSolver", "Result", "load_result", "liouvillian", "propagate_batch",
           "correlation_batch", "RedfieldSolver", "redfield_batch", "HEOMSolver", "heom_batch", "Lindblad_solver", "workloads"]
__version__ = "0.1.0"
