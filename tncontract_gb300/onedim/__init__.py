"""1-D tensor networks (MPS / MPO) on the GPU."""
from .onedim_core import *  # noqa: F401,F403
from .onedim_core import MatrixProductState, MatrixProductOperator  # noqa: F401
from .onedim_utils import *  # noqa: F401,F403
