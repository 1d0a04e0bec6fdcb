"""instaheat_gb300 -- GB300-native (sm_103a) implementation of InstaHeat's
right-hand side and DOPRI853/RK4 time stepping behind a C ABI.

``instaheat_gb300.gpu`` binds libinstaheat_gpu.so (include/instaheat_gpu.h);
``instaheat_gb300.build`` compiles it in tree.
"""
from . import build  # noqa: F401

__all__ = ["build", "gpu"]
