"""ubootgl_gb300: the ubootgl fluid time step on GB300 (sm_103a).

The compute path is the in-tree CUDA library built by ubootgl_gb300/build.py
(C ABI: include/ubootgl_gb300.h).  This package is a thin host-side mirror of
the reference's Simulation / MG interfaces plus seeded synthetic workloads.
"""
from . import workload  # noqa: F401


def __getattr__(name):
    # Lazy: importing the package must not require the CUDA library, but
    # touching the compute API does (no CPU fallback).
    if name in ("Simulation", "MG", "rbgs", "calculateResidualField"):
        from . import simulation
        return getattr(simulation, name)
    raise AttributeError(name)
