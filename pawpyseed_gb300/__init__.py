"""GB300-native band-projection path of pawpyseed.

``Wavefunction`` and ``Projector`` keep the reference's Python API for the
``aug_real`` (default) and ``pseudo`` methods; the numerical work runs in
``lib/libpawpy_gpu.so`` (hand-written CUDA for sm_103a) behind the reference's
C entry points (``include/pawpy_gpu.h``).
"""

from .vaspio import CoreRegion, PAWpyError, Pseudopotential, Structure, Vasprun  # noqa: F401


def __getattr__(name):
    # Wavefunction/Projector load the CUDA library on first use only.
    if name in ("Wavefunction", "Timer"):
        from . import wavefunction

        return getattr(wavefunction, name)
    if name == "Projector":
        from .projector import Projector

        return Projector
    raise AttributeError(name)
