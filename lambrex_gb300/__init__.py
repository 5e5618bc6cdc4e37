"""lambrex_gb300 -- GB300 (sm_103a) implementation of LAMBReX's D3Q15 lattice
Boltzmann time step behind the reference's ``AmrSim`` / ``lambrex.h`` API.

The compute path is the CUDA library ``liblbx_cuda.so`` (built in-tree by
``lambrex_gb300.build.build()``); ``lambrex_gb300.lbx`` binds it.
"""
from .lbx import (AmrSim, LbxError, lambrexFinalise, lambrexInit, lib,  # noqa: F401
                  F64, F32_SHIFTED, AMR_FAITHFUL, AMR_CONSERVATIVE, NV)
