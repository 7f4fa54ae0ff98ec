"""gpu4gst_code_gb300 — exact group Steiner trees (DPBF) on GB300.

The solver is libgst.so (CUDA kernels for sm_103a behind the C ABI of
include/gst.h). This package holds the in-tree build, the ctypes binding
(native) and the host-side mirror of the reference's DPBF call surface
(dpbf).
"""
from . import native
from .native import CSR, Graph, GSTError, Result, Status

__all__ = ["native", "Graph", "Result", "Status", "GSTError", "CSR"]
