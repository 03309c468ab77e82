"""issm_resampling_cdf_static (fixed device scratch, no allocation) against
issm_resampling_cdf (caller workspace) through the C ABI. Collected last so it
also runs after every other GPU test has used the library."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _workspace_cdf(native, lw, dtype_code):
    n = lw.numel()
    lib = native.lib()
    nb = int(lib.issm_reduce_workspace_bytes(n))
    ws = torch.empty(nb, dtype=torch.uint8, device=lw.device)
    out = torch.empty_like(lw)
    native.call("issm_resampling_cdf", native.ptr(lw), n, dtype_code, native.ptr(out), native.ptr(ws), nb,
                native.stream_ptr())
    return out


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("n", [1, 4097, 1 << 20])
def test_static_cdf_matches_workspace_cdf(issm, cuda, dtype, n):
    native = issm.native
    g = torch.Generator(device=cuda).manual_seed(n)
    lw = (torch.randn(n, generator=g, device=cuda, dtype=torch.float64) * 3.0).to(dtype)
    if n > 10:
        lw[::7] = -float("inf")
    code = native.dtype_code(dtype)
    expected = _workspace_cdf(native, lw, code)
    # two calls in a row on the same scratch
    for _ in range(2):
        out = torch.full_like(lw, float("nan"))
        native.call("issm_resampling_cdf_static", native.ptr(lw), n, code, native.ptr(out), native.stream_ptr())
        torch.cuda.synchronize()
        assert torch.allclose(out, expected, rtol=1e-6, atol=1e-7, equal_nan=False)
        assert float(out[-1]) == pytest.approx(1.0, rel=1e-6)


def test_static_cdf_rejects_sizes_beyond_its_scratch(issm, cuda):
    lib = issm.native.lib()
    limit = int(lib.issm_resampling_cdf_static_max())
    assert limit == 1 << 27
    # the size check comes before any pointer is touched
    assert lib.issm_resampling_cdf_static(1, limit + 1, 0, 1, None) == -9
    assert "scratch" in lib.issm_status_string(-9).decode()
    assert lib.issm_resampling_cdf_static(None, 16, 0, None, None) == -1
