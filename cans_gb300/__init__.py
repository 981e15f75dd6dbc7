"""cans_gb300: the CaNS pressure-correction path on one GB300 (sm_103a).

The product is libcans_gb300.so (C ABI in include/cans_gb300.h, CUDA sources in
cans_gb300/csrc/).  `cans` binds it with ctypes; `driver` orders the calls of one
time step as the reference's src/main.f90 does.
"""
from . import build  # noqa: F401
