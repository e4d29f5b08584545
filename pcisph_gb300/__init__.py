"""GB300 (sm_103a) PCISPH time step: hand-written CUDA behind a C ABI.

The compute path is ``libpcisph_gb300.so`` (``pcisph_gb300/csrc``, ABI in
``include/pcisph_gpu.h``). ``Fluid`` mirrors the reference's sim::Fluid;
``RadixSort`` replaces clogs::Radixsort; ``scenes`` builds the analytic
workloads. There is no CPU fallback: without the built library, using the
step raises.
"""
from . import scenes  # noqa: F401
from .batch import Batch  # noqa: F401
from .fluid import Fluid, RadixSort, default_options, derive_params, hash_keys, setup_scene  # noqa: F401
