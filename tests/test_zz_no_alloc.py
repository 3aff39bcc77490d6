"""The allocation-free text entry point, hd_lower_triangular_text_noalloc.

It is for callers that cannot allocate device memory: applications whose
device memory belongs to their own allocator or sits under a fixed budget, and
loops that cannot pay for cudaMalloc/cudaFree. Its scratch is a fixed array
inside the library.

Through the C ABI, its text must equal what the existing file writer
(hd_write_lower_triangular) produces for the same lower triangle. The check
runs on two calls in a row: the second is smaller, so stale scratch from the
first call would show. This file is named to be collected last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_text_matches_file_writer(tmp_path):
    torch = pytest.importorskip("torch")
    from hammingdist_gb300 import abi

    ctx = abi.Context(0)
    try:
        rng = np.random.default_rng(2024)
        for n, dtype, high in ((3001, np.uint16, 65536), (700, np.uint8, 256)):
            lt = rng.integers(0, high, size=n * (n - 1) // 2).astype(dtype)
            path = str(tmp_path / f"lt_{n}.txt")
            ctx.write_lower_triangular(lt, n, path)  # the existing entry point
            with open(path, "rb") as f:
                want = f.read()
            d_lt = torch.from_numpy(lt.view(np.uint8).copy()).to("cuda:0")
            d_text = torch.zeros(len(want) + 4096, dtype=torch.uint8, device="cuda:0")
            torch.cuda.synchronize()
            nb = ctx.lower_triangular_text_noalloc(d_lt.data_ptr(), n, dtype, d_text.data_ptr(),
                                                   d_text.numel())
            assert nb == len(want)
            assert d_text[:nb].cpu().numpy().tobytes() == want
    finally:
        ctx.close()


def test_noalloc_limits_are_reported():
    torch = pytest.importorskip("torch")
    from hammingdist_gb300 import abi

    ctx = abi.Context(0)
    try:
        # beyond the fixed scratch: rejected before any work
        with pytest.raises(abi.HDError) as e:
            ctx.lower_triangular_text_noalloc(0, 262145, np.uint8, 0, 0)
        assert e.value.code == -4 and "limit" in str(e.value)
        # text that does not fit: reported, not written
        lt = np.arange(10, dtype=np.uint8)  # n = 5
        d_lt = torch.from_numpy(lt).to("cuda:0")
        d_text = torch.zeros(4, dtype=torch.uint8, device="cuda:0")
        torch.cuda.synchronize()
        with pytest.raises(abi.HDError) as e:
            ctx.lower_triangular_text_noalloc(d_lt.data_ptr(), 5, np.uint8, d_text.data_ptr(), 4)
        assert "too small" in str(e.value)
        assert int(d_text.sum().item()) == 0
    finally:
        ctx.close()


def test_noalloc_limit_is_checked_first():
    # nsamples above the fixed scratch's 262,144 fails before any device
    # memory is touched (the buffers here are null); fewer than 2 samples
    # give no text
    from hammingdist_gb300 import abi

    ctx = abi.Context(0)
    try:
        with pytest.raises(abi.HDError, match="fixed scratch limit of 262144"):
            ctx.lower_triangular_text_noalloc(0, 262_145, np.uint8, 0, 0)
        assert ctx.lower_triangular_text_noalloc(0, 1, np.uint8, 0, 0) == 0
    finally:
        ctx.close()
