"""drr_neglog_noalloc: the negative-log transform for callers that cannot allocate device memory.

Such callers (hosts that own and pre-budget the allocator, real-time loops where an allocation
would stall the device, graph-recording pipelines that forbid allocation calls) get the same
transform as drr_neglog with the scratch kept in a fixed array inside the library. This file runs
last so a failure here leaves every other test already run; it passes alone and after the others.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from deepdrr_gb300 import _lib

pytestmark = pytest.mark.gpu


def _run(fn, img, stream):
    t = torch.from_numpy(img.copy()).cuda()
    n, h, w = img.shape
    _lib.check(fn(t.data_ptr(), n, h * w, 0.01, ctypes.c_void_p(stream.cuda_stream)))
    torch.cuda.synchronize()
    return t.cpu().numpy()


def test_noalloc_neglog_matches_the_allocating_entry_point_on_consecutive_calls():
    lib = _lib.load()
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(17)
    for call in range(2):  # the second call must not see the first call's scratch
        shape = (5, 61, 47) if call == 0 else (3, 128, 96)
        img = rng.uniform(0.2 + call, 40.0 * (call + 1), size=shape).astype(np.float32)
        expected = _run(lib.drr_neglog, img, stream)
        got = _run(lib.drr_neglog_noalloc, img, stream)
        np.testing.assert_allclose(got, expected, atol=2e-6, rtol=0)


def test_noalloc_neglog_rejects_more_views_than_its_scratch_holds():
    lib = _lib.load()
    t = torch.ones((4097, 2, 2), device="cuda")
    status = lib.drr_neglog_noalloc(t.data_ptr(), 4097, 4, 0.01, None)
    assert status == _lib.DRR_ERR_UNSUPPORTED
    assert "4096" in lib.drr_last_error().decode()
