"""kwant_gb300: the kernel polynomial method of Kwant on one GB300 (sm_103a).

A drop-in for the KPM path of Kwant: ``kwant_gb300.kpm`` mirrors
``kwant.kpm`` (SpectralDensity, Correlator, conductivity, ...) and
``kwant_gb300.operator`` mirrors ``kwant.operator`` Density / Current, with
the Chebyshev recursion, operator moments, kernel damping, DCT
reconstruction, spectral bounds and the Kubo-Bastin contraction running as
hand-written CUDA kernels behind a C ABI (include/kwant_gb300.h).

``kwant_gb300.lattices`` assembles the Hamiltonians of the benchmark models
directly from arrays; ``kwant_gb300.system.LatticeSystem`` is the finite
system type they produce.
"""

__version__ = '0.1.0'

from . import system, lattices, replicas  # noqa: F401  (host-only)


def __getattr__(name):
    # Modules that need the CUDA library load lazily, so that the host-only
    # parts import without it.
    if name in ('kpm', 'operator', '_lib', 'batch', 'surrogate'):
        import importlib
        return importlib.import_module('.' + name, __name__)
    raise AttributeError(name)
