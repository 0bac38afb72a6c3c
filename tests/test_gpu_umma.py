"""The 5th-generation tensor-core path of the learned correction (tcgen05.mma
with the FP32 accumulator in tensor memory, BF16 operands in the canonical
K-major shared-memory layout): one 128-row tile through the C ABI against a
float64 product of the same BF16-rounded operands.  Tolerance: FP32
accumulation, |D - ref| <= 2e-6 * sum_k |a_k b_k| (K <= 256 terms)."""
import ctypes

import numpy as np
import pytest

import idefix_gb300 as ig

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from idefix_gb300 import build

    build.build_library()
    return ig.load_library()


def _bf16(x):
    torch = pytest.importorskip("torch")
    return torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()


@pytest.mark.parametrize("n,k", [(16, 16), (128, 64), (128, 224), (16, 128), (64, 224), (256, 32)])
def test_umma_tile_matches_bf16_product(lib, n, k):
    rng = np.random.default_rng(n * 1000 + k)
    A = rng.standard_normal((128, k)).astype(np.float32)
    B = rng.standard_normal((n, k)).astype(np.float32)
    D = np.zeros((128, n), dtype=np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    rc = lib.idfx_check_umma(n, k, A.ctypes.data_as(fp), B.ctypes.data_as(fp), D.ctypes.data_as(fp))
    assert rc == ig.OK
    a, b = _bf16(A).astype(np.float64), _bf16(B).astype(np.float64)
    ref = a @ b.T
    bound = 2e-6 * (np.abs(a) @ np.abs(b).T) + 1e-30
    err = np.abs(D.astype(np.float64) - ref)
    assert np.all(err <= bound), float((err / bound).max())
