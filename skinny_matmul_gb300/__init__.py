"""skinny_matmul_gb300 -- GB300 (sm_103a) tall-skinny products behind a C ABI.

TSMTTSM  C = alpha * A^T B + beta * C   and   TSMM  C = alpha * A B + beta * C  (in place when
A is C), in float / double / complex float / complex double, with double-double accumulation and
an FP64 split-precision tensor-core path; SVQB orthogonalisation on top.  The compute runs in
libskinny.so (include/skinny.h); this package binds it and mirrors the reference's launcher API.
"""
from .api import Handle, Server, default_handle, launchers, svqb, svqb_host_dd, tsmm, tsmttsm  # noqa: F401
from .lib import SkinnyError  # noqa: F401

__all__ = ["Handle", "Server", "default_handle", "launchers", "svqb", "svqb_host_dd", "tsmm", "tsmttsm", "SkinnyError"]
