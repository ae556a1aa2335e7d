"""The tensor-core tile routine of the multifrontal solver's FP32 trailing
update (GPU): C −= A·B with tcgen05 kind::tf32 MMAs on split operands
(x = TF32 part + FP32 remainder, three products), FP32 accumulators in tensor
memory, K in chunks of 16 through two shared-memory stages.  Against the FP64
product on the host: error within 2e-6 of max(|A|·|B|) (FP32-level accuracy; a
single TF32 product would be near 1e-3).
"""
import ctypes

import numpy as np
import pytest

from muscade_gpu import _lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    _lib.build()
    return _lib.load()


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (128, 128, 8), (200, 300, 37), (1, 1, 1), (130, 129, 64),
                                   (256, 128, 32), (100, 260, 33), (256, 256, 256), (128, 128, 100),
                                   (300, 200, 17), (129, 127, 255), (4096, 4096, 256)])
def test_tf32x3_tile_update_matches_fp64_product(lib, M, N, K):
    rng = np.random.default_rng(M * 1000 + N * 10 + K)
    A = np.asfortranarray(rng.normal(size=(M, K)).astype(np.float32))
    B = np.asfortranarray(rng.normal(size=(K, N)).astype(np.float32))
    C0 = np.asfortranarray(rng.normal(size=(M, N)).astype(np.float32))
    C = C0.copy(order="F")
    pf = ctypes.POINTER(ctypes.c_float)
    rc = lib.mgpu_tc_gemm_check(0, M, N, K, A.ctypes.data_as(pf), B.ctypes.data_as(pf), C.ctypes.data_as(pf))
    assert rc == 0
    ref = C0.astype(np.float64) - A.astype(np.float64) @ B.astype(np.float64)
    scale = np.max(np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64))
    err = np.max(np.abs(C - ref)) / scale
    print(f"M={M} N={N} K={K}: max error {err:.2e} of max(|A||B|)")
    assert err <= 2e-6, err
