"""GPU tests of the autotuner: tuning records an entry, the table round-trips through JSON into a
new handle, and products run with the tuned launch shapes still meet their accuracy bounds."""
import json

import numpy as np
import pytest

import common

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_autotune_roundtrip_and_accuracy(handle):
    from skinny_matmul_gb300 import Handle
    handle.autotune("tsmttsm", "float64", 8, 8, 1 << 18, acc="auto")
    handle.autotune("tsmm", "float64", 8, 8, 1 << 18, acc="native")
    handle.autotune("tsmttsm", "float32", 16, 16, 1 << 18, acc="native")
    table = json.loads(handle.tune_export())
    keys = {(e["op"], e["dtype"], e["acc"], e["M"], e["N"]) for e in table["entries"]}
    assert (0, 1, 3, 8, 8) in keys and (1, 1, 0, 8, 8) in keys and (0, 0, 0, 16, 16) in keys
    for e in table["entries"]:
        assert e["us"] > 0 and e["method"] >= 0
    h2 = Handle(0)
    h2.tune_import(handle.tune_export())
    assert json.loads(h2.tune_export())["entries"] == table["entries"]
    rng = np.random.default_rng(1)
    M = N = 8
    K = 300001
    A, B = rng.uniform(-1, 1, K * M), rng.uniform(-1, 1, K * N)
    Cd = dev(np.zeros(M * N))
    h2.tsmttsm(M, N, K, dev(A), M, 1.0, dev(B), N, 0.0, Cd, M, acc="auto")
    torch.cuda.synchronize()
    exp, den = common.tsmttsm_expected(M, N, K, A, M, B, N, np.zeros(M * N), M, 1.0, 0.0)
    assert common.normwise(Cd.cpu().numpy(), exp, den) <= common.tol(np.float64, K)
    h2.close()


def test_tune_import_rejects_malformed(handle):
    from skinny_matmul_gb300 import SkinnyError
    with pytest.raises(SkinnyError, match="BAD_ARG"):
        handle.tune_import('{"entries": [{"op": 0, "dtype": 1}]}')
