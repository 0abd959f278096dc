"""gppsigma -- GB300-native GPP sigma reduction (BerkeleyGW General Plasmon Pole).

The compute path is libgpp_gb300.so (hand-written sm_103a CUDA kernels behind
the C ABI of include/gpp_gb300.h); this package holds its ctypes binding, the
host-side mirror of the reference's operator interface and the seeded
synthetic workloads.
"""
from . import build, capi, workload  # noqa: F401

__all__ = ["build", "capi", "workload", "ops"]


def __getattr__(name):
    if name == "ops":
        import importlib
        return importlib.import_module(__name__ + ".ops")
    raise AttributeError(name)
