"""mbem_gb300: the dense mollified-BEM hot path of brendanjmeade/mbem on one GB300.

Kernel drivers (``kernels``), the region-model API (``model``), the
calibrated dense backend (``backends.dense``), deflated FGMRES (``la``) and
the stress readout (``evaluate``) run hand-written sm_103a CUDA through the
C ABI declared in ``include/mbem_gb300.h``.
"""

from . import defaults  # noqa: F401

__version__ = "0.1.0"
