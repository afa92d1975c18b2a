"""superintervals_gb300 -- GB300-native batch overlap queries with the
SuperIntervals semantics (kcleal/superintervals), behind a C-ABI.

The compute runs in hand-written sm_103a kernels in libsi_gpu.so; this package
is the Python host side.  Importing the query classes needs the built library
(see build_ext.py); there is no CPU fallback.
"""
from . import workloads  # noqa: F401  (pure numpy, importable without the library)

__all__ = ["GpuIndex", "IntervalMap", "SIError", "workloads"]


def __getattr__(name):
    if name in ("GpuIndex", "IntervalMap", "SIError"):
        from . import interval_map
        return getattr(interval_map, name)
    raise AttributeError(name)
