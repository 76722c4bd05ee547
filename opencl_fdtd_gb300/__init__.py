"""
GB300-native FDTD time stepping with the API of opencl_fdtd (opencl_fdtd/__init__.py:1-5).
"""
from .simulation import Simulation, type_to_C, Event

__author__ = "opencl_fdtd_gb300 authors"

version = "0.4"
__version__ = "0.4+gb300.1"
