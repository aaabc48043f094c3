"""ctypes front end of oracle/ref_runner.cpp: the REFERENCE's own kernels, run on the GPU.

TEST INFRASTRUCTURE ONLY: imported by tests/ (parity against the reference's kernels on the same
seeded inputs) and by bench.py (the reference kernels' GB/s on the same box, beside the CPU
reference arm), never by the product package.

The kernels are the reference's headers compiled for sm_103a into oracle/_ref/*.cubin by
`make -C oracle ref` (only where the reference tree exists; the cubins then travel with the
repository copy).  ref_runner.cpp restates each launcher's launch configuration.

Buffers are torch CUDA tensors (flat storage in the reference's layout) or raw device addresses.
Several reference kernels read a few elements past the operand they are given (GENV5 reads
column M of a row when M is not a multiple of 32, genv5.cuh:44-46; SPECSMALL reads the wider
operand's width from the narrower one, specsmall.cuh:56-61), so callers allocate every operand
with `padded()`.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(_HERE, "_ref")
RUNNER = os.path.join(_HERE, "_build", "libref_runner.so")
PAD_ELEMS = 4096  # > the largest over-read of any instantiated kernel (31 elements)

DT = {"float32": 0, "float64": 1, "complex128": 3}
_lib = None
_init_msg = None


def built() -> bool:
    return os.path.isdir(REF_DIR) and any(f.endswith(".cubin") for f in os.listdir(REF_DIR))


def runner():
    global _lib
    if _lib is None:
        if not os.path.exists(RUNNER):
            from . import oracle as O
            O.build()
        lib = ctypes.CDLL(RUNNER)
        u, i, d, sz = ctypes.c_size_t, ctypes.c_int, ctypes.c_double, ctypes.c_size_t
        up = ctypes.c_uint64
        lib.ref_last_error.restype = ctypes.c_char_p
        lib.ref_init.argtypes = [ctypes.c_char_p]
        lib.ref_init.restype = i
        lib.ref_kernel_count.restype = i
        lib.ref_kernel_name.argtypes = [i]
        lib.ref_kernel_name.restype = ctypes.c_char_p
        lib.ref_tsmttsm_temp_bytes.argtypes = [ctypes.c_char_p, i, i, i, i, i]
        lib.ref_tsmttsm_temp_bytes.restype = sz
        lib.ref_tsmttsm.argtypes = [ctypes.c_char_p, i, i, i, i, up, i, d, up, i, d, up, i, i, up, u, up]
        lib.ref_tsmttsm.restype = i
        lib.ref_tsmm.argtypes = [ctypes.c_char_p, i, i, i, i, up, i, d, d, up, i, d, d, up, i, i, up]
        lib.ref_tsmm.restype = i
        _lib = lib
    return _lib


def init() -> str | None:
    """Loads the cubins on the current GPU; returns None when ready, else the reason."""
    global _init_msg
    if _init_msg is not None:
        return _init_msg or None
    if not built():
        _init_msg = "reference kernels not built (oracle/_ref has no cubin: `make -C oracle ref`)"
        return _init_msg
    import torch
    torch.cuda.init()
    torch.zeros(1, device="cuda")  # primary context current on this thread
    lib = runner()
    n = lib.ref_init(REF_DIR.encode())
    _init_msg = "" if n > 0 else f"ref_init failed: {lib.ref_last_error().decode()}"
    return _init_msg or None


def kernel_names() -> list[str]:
    lib = runner()
    return [lib.ref_kernel_name(i).decode() for i in range(lib.ref_kernel_count())]


def padded(n_elems: int, dtype, device="cuda"):
    """A flat tensor of n_elems followed by PAD_ELEMS zeros (returns the n_elems view; the
    padding keeps the reference kernels' over-reads inside the allocation)."""
    import torch
    base = torch.zeros(n_elems + PAD_ELEMS, dtype=dtype, device=device)
    return base[:n_elems]


def _ptr(x) -> int:
    return x if isinstance(x, int) else x.data_ptr()


def _stream(stream) -> int:
    import torch
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    return stream if isinstance(stream, int) else stream.cuda_stream


def _check(rc: int, what: str) -> bool:
    if rc < 0:
        raise RuntimeError(f"{what}: {runner().ref_last_error().decode()}")
    return rc == 1


def tsmttsm(variant: str, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, block_count, dtype="float64",
            stream=None, temp=None) -> bool:
    """C = alpha A^T B + beta C with the reference kernel `variant` ("GENV5", "GENV3X",
    "SPECSMALL", "SPECSMALL_PQ").  Returns False where the reference's launcher returns false."""
    import torch
    lib = runner()
    dt = DT[dtype]
    need = lib.ref_tsmttsm_temp_bytes(variant.encode(), dt, M, N, ldc, block_count)
    if temp is None or temp.numel() < need:
        temp = torch.empty(max(need, 16), dtype=torch.uint8, device="cuda")
    rc = lib.ref_tsmttsm(variant.encode(), dt, M, N, K, _ptr(A), lda, float(alpha), _ptr(B), ldb,
                         float(beta), _ptr(C), ldc, block_count, temp.data_ptr(), temp.numel(),
                         _stream(stream))
    return _check(rc, f"ref_tsmttsm {variant} {M}x{N}")


def tsmm(variant: str, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, block_count, dtype="float64",
         stream=None) -> bool:
    """C = alpha A B + beta C with the reference kernel `variant` ("FIX3", "FIX_FB",
    "FIX_IP_GHOST").  Returns False where the reference's launcher returns false."""
    lib = runner()
    al, be = complex(alpha), complex(beta)
    rc = lib.ref_tsmm(variant.encode(), DT[dtype], M, N, K, _ptr(A), lda, al.real, al.imag, _ptr(B), ldb,
                      be.real, be.imag, _ptr(C), ldc, block_count, _stream(stream))
    return _check(rc, f"ref_tsmm {variant} {M}x{N}")
