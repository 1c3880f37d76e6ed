"""tcgen05 path: one bf16 tile through shared-memory descriptors and TMEM,
against an fp32 product of the same bf16 values."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,K", [(16, 16), (144, 64), (256, 256), (48, 128)])
def test_tc_probe_tile(N, K):
    import torch

    from pyturb_gb300 import _lib

    g = torch.Generator().manual_seed(N * 1000 + K)
    A = torch.randn((128, K), generator=g).to(torch.bfloat16)
    B = torch.randn((N, K), generator=g).to(torch.bfloat16)
    dA, dB = A.cuda().contiguous(), B.cuda().contiguous()
    D = torch.full((128, N), float("nan"), device="cuda")
    _lib.call("pt_tc_probe", N, K, dA.data_ptr(), dB.data_ptr(), D.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    want = A.double() @ B.double().T
    got = D.cpu().double()
    err = (got - want).abs().max().item() / want.abs().max().item()
    assert err < 1e-5, err
