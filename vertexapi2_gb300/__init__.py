"""GB300 Gather-Apply-Scatter engine (drop-in for vertexAPI2's GPU engine).

The product is libgas_gb300.so (hand-written sm_103a CUDA behind the C ABI in
include/gas_gb300.h) plus the C++ header include/gas_gb300/gpugas.cuh.  This
package is the Python host mirror of that ABI used by the tests and the
benchmark.
"""
from ._lib import (GasError, PROGRAM_BFS, PROGRAM_CC, PROGRAM_PAGERANK, PROGRAM_PPR,
                   PROGRAM_SSSP, load)
from .engine import GASBatch, GASEngine, GASServer, device_supported

__all__ = ["GASEngine", "GASBatch", "GASServer", "GasError", "load", "device_supported", "PROGRAM_BFS", "PROGRAM_SSSP",
           "PROGRAM_CC", "PROGRAM_PAGERANK", "PROGRAM_PPR"]
