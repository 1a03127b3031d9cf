"""The split base case that allocates nothing, through the C ABI.

Its scratch is a static device array shared by every call, so the test runs
it twice in a row (and at two sizes) and checks each result against the
allocating split entry point, bit for bit (the split arithmetic is exact
integer work, so both must agree exactly).  Collected last on purpose: if it
fails, a run that stops at the first failure has run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(m, seed, cuda):
    import torch
    rng = np.random.default_rng(seed)
    A = torch.from_numpy(rng.uniform(-1, 1, m * m)).to(cuda)
    B = torch.from_numpy(rng.uniform(-1, 1, m * m) * 2.0 ** rng.integers(-20, 21, m * m)).to(cuda)
    return A, B


def test_noalloc_matches_allocating_entry_point_twice(caps, cuda):
    import torch
    L = caps.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        for m in (512, 200):
            A, B = _inputs(m, 100 * call + m, cuda)
            ref = torch.full_like(A, float("nan"))
            caps.leaf_gemm(A, B, ref, m, form="split", scheme="digits")  # the scheme the no-allocation path runs
            got = torch.full_like(A, float("nan"))
            st = L.caps_leaf_gemm_split_noalloc_dev(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
                                                    ctypes.c_void_p(got.data_ptr()), m, 0, 0, stream)
            assert st == 0, L.caps_last_cuda_error()
            torch.cuda.synchronize()
            assert torch.equal(got, ref), (call, m)


def test_noalloc_rejects_sizes_beyond_its_scratch(caps, cuda):
    import torch
    t = torch.zeros(600 * 600, dtype=torch.float64, device=cuda)
    with pytest.raises(caps.CapsError) as e:
        caps.leaf_gemm_split_noalloc(t, t, t.clone(), 600)
    assert e.value.status == 2
    assert "512" in caps.lib().caps_last_cuda_error().decode()
