"""The split base case that allocates nothing, through the C ABI.

Some callers cannot let a library allocate device memory: their memory is all
handed to their own pool allocator, or they call from code that cannot take
the device-wide synchronisation of cudaMalloc / cudaFree.  The no-allocation
entry point keeps its scratch in a static device array shared by every call.
So the test runs it twice in a row, at two sizes, and checks each result
bit for bit against the oracle's exact CPU model of the digit arithmetic and
against the allocating split entry point (the split arithmetic is exact
integer work, so all three must agree exactly).  It also checks that a second
call leaves the device's free memory unchanged.  Collected last on purpose: if
it fails, a run that stops at the first failure has run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(m, seed):
    rng = np.random.default_rng(seed)
    A = rng.uniform(-1, 1, m * m)
    B = rng.uniform(-1, 1, m * m) * 2.0 ** rng.integers(-20, 21, m * m)
    return A, B


def _call(L, A, B, C, m, s, nd, stream):
    return L.caps_leaf_gemm_split_noalloc_dev(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
                                              ctypes.c_void_p(C.data_ptr()), m, s, nd, stream)


@pytest.mark.parametrize("s,nd", [(8, 8), (0, 0)])
def test_noalloc_matches_model_and_allocating_entry_point_twice(caps, oracle_mod, cuda, s, nd):
    import torch
    L = caps.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        for m in (512, 200):
            hA, hB = _inputs(m, 100 * call + m + s)
            A, B = torch.from_numpy(hA).to(cuda), torch.from_numpy(hB).to(cuda)
            got = torch.full_like(A, float("nan"))
            st = _call(L, A, B, got, m, s, nd, stream)
            assert st == 0, L.caps_last_cuda_error()
            torch.cuda.synchronize()
            # float data need all 8 digits and 8 diagonals when the count is automatic
            model = oracle_mod.split_gemm(hA, hB, m, s or 8, nd or 8)
            assert np.array_equal(got.cpu().numpy(), model), (call, m)
            ref = torch.full_like(A, float("nan"))
            caps.leaf_gemm(A, B, ref, m, form="split", scheme="digits", slices=s, diagonals=nd)
            torch.cuda.synchronize()
            assert torch.equal(got, ref), (call, m)


def test_noalloc_second_call_leaves_free_memory_unchanged(caps, cuda):
    import torch
    L = caps.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    m = 384
    hA, hB = _inputs(m, 5)
    A, B = torch.from_numpy(hA).to(cuda), torch.from_numpy(hB).to(cuda)
    C = torch.empty_like(A)
    assert _call(L, A, B, C, m, 0, 0, stream) == 0  # first call: address look-up, lazy module loads
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert _call(L, A, B, C, m, 0, 0, stream) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_sizes_beyond_its_scratch(caps, cuda):
    import torch
    t = torch.zeros(600 * 600, dtype=torch.float64, device=cuda)
    with pytest.raises(caps.CapsError) as e:
        caps.leaf_gemm_split_noalloc(t, t, t.clone(), 600)
    assert e.value.status == 2
    assert "512" in caps.lib().caps_last_cuda_error().decode()
