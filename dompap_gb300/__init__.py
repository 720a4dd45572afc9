"""dompap_gb300 — GB300-native (sm_103a) molecular-dynamics hot path of dompap.

``Simulation`` is a drop-in for ``dompap.Simulation``: the same setters,
observables and method strings, with the neighbour list, pair forces, energy,
virial and the Langevin / NVE integrators running as hand-written CUDA kernels
behind the C ABI of ``include/dompap_gpu.h`` (``libdompap_gpu.so``). Pair
potentials given as SymPy strings are compiled to device code with NVRTC.
"""

__version__ = "0.1.0"

from .simulation import Simulation  # noqa: E402
from . import tools  # noqa: E402

__all__ = ["Simulation", "tools"]
