"""speo_gb300 -- GB300 (sm_103a) island-model differential evolution.

Python side of the library: the ctypes binding of the C ABI (include/speo_gb300.h), the
seeded instance generator, and device tables for the extended entry points. The compute
path is libspeo_gb300.so; nothing here computes on the CPU.
"""
from . import _lib
from ._lib import SpeoError, check, load
from .instances import make_instance, run_seed

__all__ = ["_lib", "SpeoError", "check", "load", "make_instance", "run_seed"]
