"""Host side of the GB300 Shan-Chen step: deck parsing, plugins, C-ABI binding.

The compute path is libtaxila_gb300.so (CUDA, sm_103a); this package mirrors
the reference's driver API around it (see ``taxila.lbm``).
"""
from . import params  # noqa: F401
from .params import TxParams, default_params  # noqa: F401
