"""GB300 (sm_103a) coherent facet kernels for soundersim.

Drop-in replacements for ``soundersim.kernels.coherent.coherent_cluttergram``,
``soundersim.kernels.multilayer.refracted_cluttergram`` and
``soundersim.kernels.incoherent.incoherent_cluttergram`` backed by the CUDA
library ``libsoundercuda.so`` (built in-tree by ``build.py``).
"""

from .coherent import coherent_cluttergram, prepare_coherent  # noqa: F401
from .multilayer import prepare_refracted, refracted_cluttergram  # noqa: F401
from .incoherent import incoherent_cluttergram, prepare_incoherent  # noqa: F401,E501
