"""kymatio_gb300 -- the kymatio scattering hot path, rebuilt for one NVIDIA GB300.

``Scattering2D`` and ``Scattering1D`` are drop-ins for ``kymatio.torch``'s
frontends (same constructor arguments, buffers, errors and output layout);
the transforms run as hand-written sm_103a CUDA kernels behind the C ABI of
``include/kymatio_gb300.h``.
"""
from .scattering2d import Scattering2D

__all__ = ['Scattering2D']
__version__ = '0.1.0'
