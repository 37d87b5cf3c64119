"""kymatio_gb300 -- the kymatio scattering hot path, rebuilt for one NVIDIA GB300.

``Scattering2D``, ``Scattering1D`` and ``TimeFrequencyScattering`` are
drop-ins for ``kymatio.torch``'s frontends (same constructor arguments,
buffers, errors and output layout); the transforms run as hand-written
sm_103a CUDA kernels behind the C ABI of ``include/kymatio_gb300.h``.
"""
from .jtfs import TimeFrequencyScattering
from .scattering1d import Scattering1D
from .scattering2d import Scattering2D

__all__ = ['Scattering2D', 'Scattering1D', 'TimeFrequencyScattering']
__version__ = '0.1.0'
