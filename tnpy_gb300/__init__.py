"""tnpy_gb300 -- GB300 (sm_103a) drop-in for tnpy's FiniteDMRG / TSDRG / linalg path.

Importing the package loads libtnx.so (the hand-written CUDA kernels behind a
C ABI, include/tnx.h); it raises ImportError when the library has not been
built. There is no CPU fallback.
"""
import logging

logger = logging.getLogger("tnpy")
if not logger.handlers:
    _h = logging.StreamHandler()
    _h.setFormatter(logging.Formatter("%(asctime)s [%(filename)s] %(levelname)s: %(message)s"))
    logger.addHandler(_h)
logger.setLevel(logging.WARNING)

from . import _lib  # noqa: E402  (fails loudly when libtnx.so is missing)
from . import autotune, linalg, model  # noqa: E402
from .finite_dmrg import BatchedFiniteDMRG, FiniteDMRG, Metric, ShiftInvertDMRG, StreamedFiniteDMRG  # noqa: E402
from .matrix_product_state import (  # noqa: E402
    Direction,
    Environment,
    MatrixProductState,
    MatrixProductStateMeasurements,
)
from .exact_diagonalization import ExactDiagonalization  # noqa: E402
from .operators import FullHamiltonian, MatrixProductOperator, SpinOperators  # noqa: E402
from .tsdrg import (  # noqa: E402
    TSDRG,
    BatchedTSDRG,
    HighEnergyTreeTensorNetworkSDRG,
    ShiftInvertTreeTensorNetworkSDRG,
    TensorTree,
    TreeTensorNetworkSDRG,
)

__all__ = [
    "FiniteDMRG", "ShiftInvertDMRG", "BatchedFiniteDMRG", "StreamedFiniteDMRG", "Metric", "Direction", "Environment", "MatrixProductState",
    "MatrixProductStateMeasurements", "FullHamiltonian", "MatrixProductOperator", "SpinOperators",
    "linalg", "model", "logger", "ExactDiagonalization", "TSDRG", "TreeTensorNetworkSDRG", "BatchedTSDRG", "TensorTree",
    "HighEnergyTreeTensorNetworkSDRG", "ShiftInvertTreeTensorNetworkSDRG",
]
