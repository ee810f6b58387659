"""mantiis_gb300: GB300-native (sm_103a) D2Q9 multi-block lattice Boltzmann time
step of MANTIIS, behind the C ABI of include/mantiis_gpu.h.

    from mantiis_gb300 import Solver, HostGrid, default_params
"""
from .native import (  # noqa: F401
    SIM_ADSORPTION,
    SIM_COUPLED,
    SIM_TRANSPORT,
    Batch,
    HostGrid,
    MantiisError,
    Solver,
    default_params,
    generate_disks,
    lib,
    pore_properties,
    pore_properties_gpu,
    units,
)

__all__ = [
    "Solver",
    "Batch",
    "HostGrid",
    "MantiisError",
    "default_params",
    "generate_disks",
    "pore_properties",
    "pore_properties_gpu",
    "units",
    "lib",
    "SIM_TRANSPORT",
    "SIM_ADSORPTION",
    "SIM_COUPLED",
]
