"""lair's LU hot path (getrf / getrs) on one GB300, behind lair's interface.

Modules mirror lair's public surface:

- ``lair_gb300.lapack``   -- ``getrf`` / ``getrs`` (src/lapack/getrf.rs, getrs.rs)
- ``lair_gb300.lu``       -- ``Factorized`` with p/l/u/is_singular/solve/into_pl
                             (src/decomposition/lu.rs)
- ``lair_gb300.equation`` -- ``solve`` (src/equation.rs)
- ``lair_gb300.errors``   -- ``InvalidInput`` (src/lib.rs)

All numerical work runs in liblair_gb300.so (CUDA, sm_103a) through the C ABI
in include/luhot.h; there is no CPU fallback.
"""
from . import equation, lapack, lu  # noqa: F401
from .errors import InvalidInput  # noqa: F401

__version__ = "0.1.0"
