"""tcgen05 descriptor encodings, pinned by exact small-integer GEMMs, and the
tensor-core forms of the mixture density against the FP64 oracle."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["bf16", "tf32"])
@pytest.mark.parametrize("n,k", [(16, 16), (64, 32), (80, 64), (128, 48), (256, 64)])
def test_tc_gemm_selftest_exact(issm, cuda, kind, n, k):
    prec = issm.native.PREC_BF16 if kind == "bf16" else issm.native.PREC_TF32
    g = torch.Generator(device=cuda).manual_seed(n * 131 + k)
    a = torch.randint(-4, 5, (128, k), generator=g, device=cuda).float()
    b = torch.randint(-4, 5, (n, k), generator=g, device=cuda).float()
    c = torch.full((128, n), float("nan"), device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    issm.native.call("issm_tc_selftest", issm.native.ptr(a), issm.native.ptr(b), issm.native.ptr(c), n, k, prec,
                     issm.native.ptr(status), issm.native.stream_ptr())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert torch.equal(c, a @ b.T)
