"""spectrum_gb300: the test-particle SDE stepping path of SPECTRUM, written for one GB300.

The compute path is hand-written CUDA for sm_103a in ``csrc/`` behind the C ABI declared in
``include/spx.h``; this package holds the host-side mirror of the reference's plugin interface
(``DataContainer`` blobs, plugin prototypes with the reference class names, a ``SimulationGPU``
driver with the reference's public method names) and the ctypes binding to the library.
"""
from .datacontainer import DataContainer  # noqa: F401
from . import plugins, units, problem, workloads  # noqa: F401
