"""tncontract_gb300: a GB300 (sm_103a) engine for tncontract's tensor-network
hot path -- labelled contraction, SVD truncation and the MPS/MPO sweeps built
on them -- behind tncontract's own Python API.

    import tncontract_gb300 as tn
    A = tn.Tensor(np.random.rand(2, 3), labels=["a", "b"])

Tensor data lives on the current CUDA device; every data operation runs in
the package's native library (``_lib/libtncontract_gb300.so``, built by
``tncontract_gb300._build``).  There is no CPU fallback.
"""
from .tensor import *  # noqa: F401,F403
from .tensor import tensor_qr, tensor_lq, conjugate  # noqa: F401
from .label import *  # noqa: F401,F403
from .tncon import con  # noqa: F401
from . import tensor  # noqa: F401
from . import onedim  # noqa: F401
from . import matrices  # noqa: F401
from . import twodim  # noqa: F401

__version__ = "0.1.0"
