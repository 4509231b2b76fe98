"""GB300-native CNS_NoSpec RK3 advance.

The product is libcns_gb300.so (hand-written sm_103a kernels behind the C ABI in
include/cns_gb300.h); this package builds it, binds it with ctypes and mirrors the
reference's call surface (cpu/header.h:98-156) on numpy arrays.
"""
from .initdata import ALAM, CFL, ETA, NC, NG, box_dx, fill_periodic, initial_state, normwise_error  # noqa: F401
from ._lib import CNS_ASSEMBLE_DIRECT, CNS_ASSEMBLE_FX, CNS_ASSEMBLE_TMA, CNS_ASSEMBLE_TMA_FX, CNS_ASSEMBLE_TMA_WS, CNS_FP64, CNS_MIXED, CnsError, load  # noqa: F401
from .solver import (Batch, Box, advance_host, ctoprim, diffterm, fill_boundary, hypterm, new_advance,  # noqa: F401
                     read_configurations)

__all__ = ["Box", "Batch", "ctoprim", "hypterm", "diffterm", "fill_boundary", "new_advance", "advance_host",
           "read_configurations", "initial_state", "box_dx", "CNS_FP64", "CNS_MIXED", "CnsError", "load"]
