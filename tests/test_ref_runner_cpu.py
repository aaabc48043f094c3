"""CPU checks of the runner of the reference's own kernels (oracle/ref_runner.cpp): it builds,
loads without a GPU, exports its entry points, and fails cleanly where it cannot run."""
import os

import pytest


def test_runner_builds_and_exports():
    from oracle import oracle as O
    from oracle import ref_gpu
    O.build()
    lib = ref_gpu.runner()
    for name in ("ref_init", "ref_kernel_count", "ref_kernel_name", "ref_last_error", "ref_tsmttsm_temp_bytes",
                 "ref_tsmttsm", "ref_tsmm"):
        assert hasattr(lib, name), name


def test_runner_temp_bytes_follow_reference_layouts():
    from oracle import ref_gpu
    lib = ref_gpu.runner()
    # blockCount * N * ldc accumulators (genv5.cuh:20)
    assert lib.ref_tsmttsm_temp_bytes(b"GENV5", 1, 8, 8, 9, 100) == 100 * 8 * 9 * 8
    assert lib.ref_tsmttsm_temp_bytes(b"SPECSMALL_PQ", 1, 4, 4, 4, 10) == 10 * 4 * 4 * 16
    assert lib.ref_tsmttsm_temp_bytes(b"SPECSMALL", 0, 4, 4, 4, 10) == 10 * 4 * 4 * 4


def test_launch_before_init_is_an_error_not_a_crash():
    from oracle import ref_gpu
    lib = ref_gpu.runner()
    rc = lib.ref_tsmttsm(b"GENV5", 1, 8, 8, 16, 0, 8, 1.0, 0, 8, 0.0, 0, 8, 1, 0, 0, 0)
    assert rc == -1
    assert b"ref_init" in lib.ref_last_error()


def test_reference_cubins_built_where_reference_tree_exists():
    from oracle import oracle as O
    from oracle import ref_gpu
    if not os.path.isdir(os.path.join(O.REFERENCE_TREE, "tsmttsm")):
        pytest.skip("no reference tree on this machine; the cubins come prebuilt")
    O.build()
    assert ref_gpu.built()
    parts = sorted(f for f in os.listdir(ref_gpu.REF_DIR) if f.endswith(".cubin"))
    assert len(parts) == 5, parts
