"""GPU parity of the rectangular subproject's rectMM on one rank
(rect-class/rectmm.cpp), through the C ABI, against the subproject's own
outputs (tests/golden/ref_rect.npz, made by its rectMM built from its sources)
and the oracle's restatement.  Integer data: bit-exact.  Float data: the
reference's leaves are OpenBLAS dgemm, these are FP64 DMMA, so each written
entry is within the classical bound k u sum|a||b| of the reference's, and
every entry the one-rank walk never writes keeps C's starting value."""
import importlib.util
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _golden_module():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(ROOT, "tests", "golden",
                                                                              "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def _key(m, n, k, r, patt, div, kind):
    return "rect_%d_%d_%d_%d_%s_%s_%s" % (m, n, k, r, patt or "-", "".join(map(str, div)) or "-", kind)


def _leaf(m, n, k, r, div):
    for l in range(r):
        m, n, k = m // div[3 * l], n // div[3 * l + 1], k // div[3 * l + 2]
    return m, n, k


def _gpu(caps, cuda, A, B, C, m, n, k, r, patt, div):
    import torch
    dA, dB = torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda)
    dC = torch.from_numpy(C.copy()).to(cuda)
    caps.rect_mm(dA, dB, dC, m, n, k, r, patt, div)
    torch.cuda.synchronize()
    return dC.cpu().numpy()


def test_rect_mm_matches_reference_rectmm(caps, cuda):
    mg = _golden_module()
    g = np.load(os.path.join(ROOT, "tests", "golden", "ref_rect.npz"))
    for m, n, k, r, patt, div, kind, seed in mg.RECT_CASES:
        A, B, C0 = mg.rect_inputs(m, n, k, kind, seed)
        ref = g[_key(m, n, k, r, patt, div, kind)]
        got = _gpu(caps, cuda, A, B, C0, m, n, k, r, patt, div)
        case = (m, n, k, r, patt, div, kind)
        if kind == "int":
            assert np.array_equal(got, ref), case
            continue
        untouched = ref == C0  # float data: a written entry equals its start value only by chance
        assert np.array_equal(got[untouched], C0[untouched]), case
        assert np.array_equal(got == C0, untouched), case
        k0 = _leaf(m, n, k, r, div)[2]
        assert np.max(np.abs(got - ref)) <= 2 * k0 * k0 * 2.0 ** -53, case  # |a|, |b| <= 1


@pytest.mark.parametrize("m,n,k,r,patt,div", [
    (1024, 768, 512, 2, "dd", [2, 1, 1, 1, 2, 1]),      # every divk = 1, divm or divn = 1: the exact product
    (512, 384, 768, 2, "DD", [2, 2, 2, 2, 3, 2]),       # overwrites and overlapping blocks at both levels
    (200, 100, 50, 1, "d", [5, 4, 2]),                  # leaves of 40 x 25 x 25 (partial tiles)
    (96, 96, 96, 0, "", []),
])
def test_rect_mm_integers_exact_vs_oracle(caps, oracle_mod, cuda, m, n, k, r, patt, div):
    rng = np.random.default_rng(m + n + k + r)
    A = rng.integers(-64, 65, m * k).astype(np.float64)
    B = rng.integers(-64, 65, k * n).astype(np.float64)
    C0 = rng.integers(-64, 65, m * n).astype(np.float64)
    ref = oracle_mod.rect_mm(A, B, C0, m, n, k, r, patt, div)
    assert np.array_equal(_gpu(caps, cuda, A, B, C0, m, n, k, r, patt, div), ref)
    # the host entry point: the same, C copied in and back
    C = C0.copy()
    caps.rect_mm(A, B, C, m, n, k, r, patt, div)
    assert np.array_equal(C, ref)


def test_rect_mm_errors_leave_c_alone(caps, cuda):
    import torch
    t = torch.zeros(64 * 48, dtype=torch.float64, device=cuda)
    for patt, div, status in (("b", [2, 2, 1], 7), ("x", [2, 2, 1], 1), ("d", [3, 1, 1], 2)):
        C = torch.full((64 * 48,), 5.0, dtype=torch.float64, device=cuda)
        with pytest.raises(caps.CapsError) as e:
            caps.rect_mm(t, t, C, 64, 48, 32, 1, patt, div)
        assert e.value.status == status
        torch.cuda.synchronize()
        assert bool((C == 5.0).all())
