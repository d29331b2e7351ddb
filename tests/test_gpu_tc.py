"""tcgen05 building blocks (kind::tf32 MMA, smem descriptors, TMEM layout)
against numpy, through the C ABI: single TF32 to ~1e-3 relative, 3xTF32 to
~1e-6 relative (the split-precision scheme of the fast Legendre path)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,K", [(32, 64), (16, 8), (64, 64), (48, 32), (64, 24)])
def test_tc_gemm_selftest(cuda, N, K):
    import torch
    from my_swampe_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(N * 1000 + K)
    A = rng.standard_normal((128, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    dA = torch.tensor(A, device=cuda)
    dB = torch.tensor(B, device=cuda)
    for split3, tol in ((0, 2e-3), (1, 2e-6)):
        dD = torch.full((128, N), float("nan"), device=cuda)
        rc = lib.swp_tc_selftest(dA.data_ptr(), dB.data_ptr(), dD.data_ptr(), N, K, split3,
                                 torch.cuda.current_stream().cuda_stream)
        assert rc == 0
        D = dD.cpu().numpy().astype(np.float64)
        err = np.max(np.abs(D - ref)) / np.max(np.abs(ref))
        assert err < tol, (split3, err)
