"""GPU parity of the Cholesky subproject's multiply, C = alpha C - A B^T
(cholesky/mult.h:6, mult.cpp:11-137 on one rank), through the C ABI and the
reference-named C++ `mult`, against the oracle restatement and the
subproject's own mult() outputs (tests/golden/ref_chol.npz)."""
import ctypes
import hashlib
import importlib.util
import os

import numpy as np
import pytest

from helpers import caps_of, mat_of, dd_of

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def golden_module():
    spec = importlib.util.spec_from_file_location("mg", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def gpu_chol(caps, A, B, C, n, r, alpha, form="plain", pattern=None, scheme="auto", device="cuda:0"):
    import torch
    dA = torch.from_numpy(A).to(device)
    dB = torch.from_numpy(B).to(device)
    dC = torch.from_numpy(np.array(C)).to(device)
    caps.chol_mult(dC, dA, dB, n, r, alpha, pattern=pattern, form=form, scheme=scheme)
    torch.cuda.synchronize()
    return dC.cpu().numpy()


def scaled_error(oracle_mod, out, A, B, C, n, r, alpha):
    """max |out - (alpha C - A B^T)| / (|alpha C| + |A| |B|^T), the product
    taken in double-double."""
    Am, Bm, Cm = (mat_of(oracle_mod, x, n, r, 1) for x in (A, B, C))
    hi, lo = dd_of(oracle_mod, Am, np.ascontiguousarray(Bm.T))
    ac = alpha * Cm if alpha != 0 else np.zeros_like(Cm)
    d = ((mat_of(oracle_mod, out, n, r, 1) - ac) + hi) + lo
    scale = np.abs(ac) + np.abs(Am) @ np.abs(Bm).T
    return float(np.max(np.abs(d) / np.where(scale > 0, scale, 1)))


@pytest.mark.parametrize("form", ["plain", "split"])
@pytest.mark.parametrize("n,r,alpha,pattern", [(56, 2, 1.0, None), (64, 0, 1.0, ""), (128, 3, 0.0, "bdb"),
                                               (96, 1, 2.5, "b"), (2048, 2, -1.0, "dd"), (512, 3, 1.0, "hhd")])
def test_chol_mult_integers_bitexact(caps, oracle_mod, cuda, form, n, r, alpha, pattern):
    """Integer data: the same bits as the oracle (and so as the reference's
    classical update); alpha = 0 runs with C full of NaN, which must stay unread."""
    rng = np.random.default_rng(n * 7 + r)
    A, B, C = (rng.integers(-64, 65, n * n).astype(np.float64) for _ in range(3))
    if alpha == 0:
        C[:] = np.nan
    want = oracle_mod.chol_mult(C, A, B, n, r, alpha)
    got = gpu_chol(caps, A, B, C, n, r, alpha, form=form, pattern=pattern)
    assert np.array_equal(got, want), (form, n, r, alpha)


def test_chol_mult_reference_integer_goldens(caps, oracle_mod, cuda):
    """The subproject's own mult() outputs on integer data (its DFS branch at
    n = 2048 included), bit for bit, both forms."""
    mg = golden_module()
    g = np.load(os.path.join(ROOT, "tests", "golden", "ref_chol.npz"))
    for n, r, alpha, kind, seed in mg.CHOL_CASES:
        if kind != "int":
            continue
        A, B, C = mg.chol_inputs(n, kind, seed)
        key = "chol_%d_%d_%s" % (n, r, kind)
        for form in ("plain", "split"):
            out = gpu_chol(caps, A, B, C, n, r, alpha, form=form)
            if key in g.files:
                assert np.array_equal(out, g[key]), (key, form)
            else:
                assert hashlib.sha256(out.tobytes()).digest() == bytes(g[key + "_sha256"]), (key, form)


@pytest.mark.parametrize("form", ["plain", "split"])
def test_chol_mult_float_error_vs_reference(caps, oracle_mod, cuda, form):
    """Float data.  The reference's classical update is pinned only by its own
    outputs (ref_chol.npz); this library's product is Strassen-Winograd with r
    levels, whose error grows with r (9x the classical error at n = 128, r = 3
    for FP64 leaves).  So the GPU result is held to the oracle's restatement
    of the same Strassen update -- alpha C + A (-B^T) with r 'd' steps and
    classical leaves, then one scale-add -- at most 2x its scaled error plus
    2^-52, and to 2^-40 outright; both errors against a double-double
    product, scaled by |alpha C| + |A| |B|^T."""
    mg = golden_module()
    g = np.load(os.path.join(ROOT, "tests", "golden", "ref_chol.npz"))
    oracle_mod.use_blas(False)
    for n, r, alpha, kind, seed in mg.CHOL_CASES:
        key = "chol_%d_%d_%s" % (n, r, kind)
        if kind != "float" or key not in g.files:
            continue
        A, B, C = mg.chol_inputs(n, kind, seed)
        out = gpu_chol(caps, A, B, C, n, r, alpha, form=form)
        nbt = caps_of(oracle_mod, -np.ascontiguousarray(mat_of(oracle_mod, B, n, r, 1).T), r)
        prod = oracle_mod.multiply(A, nbt, n, r, 1, "d" * r)
        strassen = prod if alpha == 0 else alpha * C + prod
        e_str = scaled_error(oracle_mod, strassen, A, B, C, n, r, alpha)
        e_gpu = scaled_error(oracle_mod, out, A, B, C, n, r, alpha)
        e_ref = scaled_error(oracle_mod, g[key], A, B, C, n, r, alpha)
        assert e_gpu <= 2 * e_str + 2.0 ** -52 and e_gpu <= 2.0 ** -40, (key, form, e_gpu, e_str, e_ref)


def test_chol_mult_host_entry_and_cxx_mult(caps, oracle_mod, cuda):
    """Host arrays through caps_chol_mult_host and through the reference-named
    C++ mult(double*, double*, double*, int, int, int, double)."""
    n, r = 256, 2
    rng = np.random.default_rng(5)
    A, B, C = (rng.integers(-9, 10, n * n).astype(np.float64) for _ in range(3))
    want = oracle_mod.chol_mult(C, A, B, n, r, 1.0)
    C1 = C.copy()
    caps.chol_mult(C1, A, B, n, r, 1.0, form="split")
    assert np.array_equal(C1, want)
    L = caps.lib()
    mult = getattr(L, "_Z4multPdS_S_iiid")
    dp = ctypes.POINTER(ctypes.c_double)
    mult.argtypes = [dp, dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
    mult.restype = None
    C2 = C.copy()
    mult(C2.ctypes.data_as(dp), A.ctypes.data_as(dp), B.ctypes.data_as(dp), n, 1, r, 1.0)
    assert np.array_equal(C2, want)


def test_chol_mult_rejects_multi_rank(caps, cuda):
    import torch
    x = torch.zeros(64 * 64, dtype=torch.float64, device=cuda)
    with pytest.raises(caps.CapsError) as e:
        caps.chol_mult(x, x.clone(), x.clone(), 64, 2, x=8)
    assert e.value.status == 7
