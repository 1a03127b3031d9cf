"""CPU tests: the oracle against the reference's own fixtures and outputs."""
import ctypes
import hashlib
import os

import numpy as np
import pytest

from helpers import caps_of, mat_of, dd_of

from oracle.oracle import reference_dir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = reference_dir() or ""
REFLIB = os.path.join(ROOT, "oracle", "_ref", "libcapsref.so")


def test_fixture_conversion_matches_reference_files(ref_tests):
    """The committed npz fixtures equal the reference's text files (when present)."""
    if not os.path.isdir(os.path.join(REF, "tests")):
        pytest.skip("reference sources not present")
    for n in (28, 56):
        toks = open(os.path.join(REF, "tests", "test%d.in" % n)).read().split()
        vals = np.array([int(float(t)) for t in toks[1:]], dtype=np.int64)
        assert np.array_equal(vals[: n * n].reshape(n, n), ref_tests["A%d" % n])
        assert np.array_equal(vals[n * n:].reshape(n, n), ref_tests["B%d" % n])


@pytest.mark.parametrize("n", [28, 42, 56, 196, 294, 392])
def test_oracle_reference_known_answers(oracle_mod, ref_tests, n):
    """Every one-rank (-b, -r) line of the reference's .params passes with deviation 0."""
    A = ref_tests["A%d" % n].astype(np.float64)
    B = ref_tests["B%d" % n].astype(np.float64)
    exact = A.astype(np.int64) @ B.astype(np.int64)
    assert hashlib.sha256(exact.tobytes()).digest() == bytes(ref_tests["C%d_sha256" % n])
    oracle_mod.use_blas(False)
    params = ref_tests["params%d" % n]
    assert len(params) > 0
    for bs, r in params:
        if n >= 294 and r < 2:
            continue  # classical leaf of 294^3..392^3 is slow on CPU and covered at r >= 2
        C = mat_of(oracle_mod, oracle_mod.multiply(caps_of(oracle_mod, A, r, bs), caps_of(oracle_mod, B, r, bs), n, r, bs,
                                                   "d" * r), n, r, bs)
        assert np.array_equal(C, exact.astype(np.float64)), (n, bs, r)


def test_oracle_matches_reference_float_goldens(oracle_mod):
    """Oracle + numpy's OpenBLAS reproduces the reference's own multiply() bit for bit."""
    if not oracle_mod.use_blas(True):
        pytest.skip("numpy OpenBLAS not found")
    try:
        g = np.load(os.path.join(ROOT, "tests", "golden", "ref_float.npz"))
        from make_golden_cases import FLOAT_CASES
    except ImportError:
        import importlib.util
        spec = importlib.util.spec_from_file_location("mg", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
        mg = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mg)
        FLOAT_CASES = mg.FLOAT_CASES
        g = np.load(os.path.join(ROOT, "tests", "golden", "ref_float.npz"))
    for n, r, bs, pat, seed in FLOAT_CASES:
        rng = np.random.default_rng(seed)
        A = rng.uniform(-1, 1, n * n)
        B = rng.uniform(-1, 1, n * n)
        C = oracle_mod.multiply(A, B, n, r, bs, pat)
        assert np.array_equal(C, g["C_%d_%d_%d" % (n, r, bs)]), (n, r, bs)
    oracle_mod.use_blas(False)


def test_oracle_layout_matches_reference(oracle_mod):
    g = np.load(os.path.join(ROOT, "tests", "golden", "ref_layout.npz"))
    for key in g.files:
        _, n, r, bs = key.split("_")
        n, r, bs = int(n), int(r), int(bs)
        perm = oracle_mod.to_caps(np.arange(n * n, dtype=np.float64), n, r, bs)
        assert np.array_equal(perm.astype(np.int32), g[key]), key
        back = oracle_mod.from_caps(perm, n, r, bs)
        assert np.array_equal(back, np.arange(n * n, dtype=np.float64))


@pytest.mark.skipif(not os.path.exists(REFLIB), reason="reference build not present")
def test_oracle_bitexact_vs_live_reference(oracle_mod):
    class Desc(ctypes.Structure):
        _fields_ = [(f, ctypes.c_int) for f in ("lda", "nrec", "nproc", "nprocr", "nprocc", "nproc_summa", "bs")]
    L = ctypes.CDLL(REFLIB)
    mul = getattr(L, "_Z8multiplyPdS_S_13MatDescriptorPc")
    dp = ctypes.POINTER(ctypes.c_double)
    mul.argtypes = [dp, dp, dp, Desc, ctypes.c_char_p]
    mul.restype = None
    assert oracle_mod.use_blas(True)
    for n, r, bs, pat in [(112, 3, 1, b"ddd"), (80, 2, 5, b"dd"), (256, 2, 1, b"dd")]:
        rng = np.random.default_rng(n)
        A = rng.uniform(-1, 1, n * n) * 2.0 ** rng.integers(-20, 21, n * n)
        B = rng.uniform(-1, 1, n * n)
        C = np.zeros(n * n)
        mul(A.ctypes.data_as(dp), B.ctypes.data_as(dp), C.ctypes.data_as(dp), Desc(n, r, 1, 1, 1, 1, bs), pat)
        assert np.array_equal(C, oracle_mod.multiply(A, B, n, r, bs, pat.decode()))
    oracle_mod.use_blas(False)


def test_counters_match_reference_counts(oracle_mod):
    """additions/multiplications as counters.cpp counts them (1.463e9 additions at n=8192, r=3)."""
    import caps_gb300
    f = caps_gb300.flop_counts(8192, 3)
    m = 1024
    adds = 15 * sum(7 ** l * (8192 >> (l + 1)) ** 2 for l in range(3))
    assert adds == 1463812096 or abs(adds - 1.463e9) < 1e7
    assert f.actual == adds + 2 * 343 * m ** 3
    oracle_mod.use_blas(False)
    oracle_mod.reset_counters()
    n, r = 56, 2
    A = np.ones(n * n)
    oracle_mod.multiply(A, A, n, r, 1, "dd")
    a, mu = oracle_mod.counters()
    fl = caps_gb300.flop_counts(n, r)
    assert a + mu == fl.actual


def test_drand48_stream_matches_libc(oracle_mod):
    libc = ctypes.CDLL(None)
    libc.drand48.restype = ctypes.c_double
    libc.srand48.argtypes = [ctypes.c_long]
    libc.srand48(3)
    want = np.array([2 * libc.drand48() - 1 for _ in range(5000)])
    assert np.array_equal(oracle_mod.drand48_stream(5000, seed=3), want)


def test_dd_gemm_exact_on_small_rationals(oracle_mod):
    from fractions import Fraction
    rng = np.random.default_rng(0)
    n = 6
    A = rng.uniform(-1, 1, (n, n)) * 2.0 ** rng.integers(-30, 30, (n, n))
    B = rng.uniform(-1, 1, (n, n))
    hi, lo = dd_of(oracle_mod, A, B)
    for i in range(n):
        for j in range(n):
            ex = sum(Fraction(A[i, k]) * Fraction(B[k, j]) for k in range(n))
            got = Fraction(hi[i, j]) + Fraction(lo[i, j])
            assert abs(float(got - ex)) <= 2.0 ** -100 * max(1.0, abs(float(ex))) * 64


def test_split_model_integer_exact(oracle_mod):
    rng = np.random.default_rng(5)
    m = 40
    A = rng.integers(-1024, 1025, (m, m)).astype(np.float64)
    B = rng.integers(-1024, 1025, (m, m)).astype(np.float64)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    C = oracle_mod.split_gemm(np.ascontiguousarray(A.T).reshape(-1), np.ascontiguousarray(B.T).reshape(-1), m, 2, 3)
    assert np.array_equal(C.reshape(m, m).T, exact)


def test_split_model_float_error(oracle_mod):
    rng = np.random.default_rng(6)
    m = 64
    A = rng.uniform(-1, 1, (m, m))
    B = rng.uniform(-1, 1, (m, m))
    hi, lo = dd_of(oracle_mod, A, B)
    C = oracle_mod.split_gemm(np.ascontiguousarray(A.T).reshape(-1), np.ascontiguousarray(B.T).reshape(-1), m, 8, 8)
    C = C.reshape(m, m).T
    ab = np.abs(A) @ np.abs(B)
    assert np.max(np.abs((C - hi) - lo) / ab) < 2.0 ** -48


def _residue_model_py(A, B):
    """Independent statement of the residue scheme's leaf value: scaled
    integers from exact rational arithmetic, product in Python integers,
    one correctly rounded division by a power of two."""
    import math
    from fractions import Fraction
    m = A.shape[0]

    def low_bit(v):  # exponent of the lowest set bit of v != 0
        fr = Fraction(abs(v))
        if fr.denominator > 1:
            return -(fr.denominator.bit_length() - 1)  # odd numerator over 2^k
        n = fr.numerator
        return (n & -n).bit_length() - 1

    def line_scales(lines):
        E, bits = [], 0
        for line in lines:
            nz = [v for v in line if v != 0.0]
            if not nz:
                E.append(None)
                continue
            e = max(math.frexp(v)[1] for v in nz)  # |v| < 2^e
            lsb = min(low_bit(v) for v in nz)
            E.append(e)
            bits = max(bits, e - lsb + 1)
        return E, min(bits, 55)

    def rnd(x):  # round half to even of a Fraction
        f = math.floor(x)
        d = x - f
        return f + (1 if d > Fraction(1, 2) or (d == Fraction(1, 2) and f % 2) else 0)

    Ea, ta = line_scales([A[i, :] for i in range(m)])
    Eb, tb = line_scales([B[:, j] for j in range(m)])
    X = [[0 if Ea[i] is None else rnd(Fraction(A[i, k]) * Fraction(2) ** (ta - Ea[i])) for k in range(m)]
         for i in range(m)]
    Y = [[0 if Eb[j] is None else rnd(Fraction(B[k, j]) * Fraction(2) ** (tb - Eb[j])) for k in range(m)]
         for j in range(m)]
    C = np.zeros((m, m))
    for i in range(m):
        for j in range(m):
            if Ea[i] is None or Eb[j] is None:
                continue
            s = sum(X[i][k] * Y[j][k] for k in range(m))
            sh = (ta - Ea[i]) + (tb - Eb[j])
            C[i, j] = s / 2 ** sh if sh >= 0 else float(s * 2 ** -sh)  # int / int: correctly rounded
    return C, (ta, tb)


@pytest.mark.parametrize("kind", ["uniform", "wide", "ints", "tiny"])
def test_residue_model_matches_exact_rounding(oracle_mod, kind):
    m = 12
    rng = np.random.default_rng(len(kind))
    if kind == "uniform":
        A, B = rng.uniform(-1, 1, (m, m)), rng.uniform(-1, 1, (m, m))
    elif kind == "wide":
        A = rng.uniform(-1, 1, (m, m)) * 2.0 ** rng.integers(-20, 21, (m, m))
        B = rng.uniform(-1, 1, (m, m)) * 2.0 ** rng.integers(-20, 21, (m, m))
    elif kind == "ints":
        A = rng.integers(-2 ** 30, 2 ** 30, (m, m)).astype(np.float64)
        B = rng.integers(-2 ** 30, 2 ** 30, (m, m)).astype(np.float64)
    else:
        A = rng.uniform(-1, 1, (m, m)) * 1e-160
        B = rng.uniform(-1, 1, (m, m)) * 1e-160
        A[2, :] = 0.0
        B[5, 7] = 5e-324
    C, t = oracle_mod.split_gemm_residues(A.T.copy().reshape(-1), B.T.copy().reshape(-1), m)
    Cp, tp = _residue_model_py(A, B)
    assert t == tp
    assert np.array_equal(C.reshape(m, m).T, Cp)


def _golden_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("mg", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def test_chol_mult_oracle_matches_reference_mult(oracle_mod):
    """The restated Cholesky mult() (C = alpha C - A B^T, one rank) with numpy's
    OpenBLAS reproduces the subproject's own mult() bit for bit, its DFS branch
    (n = 2048 > 1024) included."""
    if not oracle_mod.use_blas(True):
        pytest.skip("numpy OpenBLAS not found")
    mg = _golden_module()
    g = np.load(os.path.join(ROOT, "tests", "golden", "ref_chol.npz"))
    try:
        for n, r, alpha, kind, seed in mg.CHOL_CASES:
            A, B, C = mg.chol_inputs(n, kind, seed)
            out = oracle_mod.chol_mult(C, A, B, n, r, alpha)
            key = "chol_%d_%d_%s" % (n, r, kind)
            if key in g.files:
                assert np.array_equal(out, g[key]), key
            else:
                assert hashlib.sha256(out.tobytes()).digest() == bytes(g[key + "_sha256"]), key
    finally:
        oracle_mod.use_blas(False)


@pytest.mark.parametrize("n,r,alpha", [(56, 2, 1.0), (64, 3, 0.0), (2048, 1, -3.0)])
def test_chol_mult_oracle_integers_exact(oracle_mod, n, r, alpha):
    """Integer data: the oracle equals the exact alpha C - A B^T, with or
    without a BLAS; alpha = 0 leaves C unread (C holds NaN here)."""
    rng = np.random.default_rng(n + r)
    A, B, C = (rng.integers(-9, 10, n * n).astype(np.float64) for _ in range(3))
    if alpha == 0:
        C[:] = np.nan
    # |entries| <= 9: every partial sum of the float64 product is an integer
    # below 2^53, so numpy's float product is exact
    Af, Bf = mat_of(oracle_mod, A, n, r, 1), mat_of(oracle_mod, B, n, r, 1)
    Cf = np.zeros((n, n)) if alpha == 0 else mat_of(oracle_mod, C, n, r, 1)
    exact = alpha * Cf - Af @ Bf.T
    for blas in (False, True):
        if blas and not oracle_mod.use_blas(True):
            continue
        try:
            out = oracle_mod.chol_mult(C, A, B, n, r, alpha)
        finally:
            oracle_mod.use_blas(False)
        assert np.array_equal(mat_of(oracle_mod, out, n, r, 1), exact), (n, r, alpha, blas)


def _rect_key(m, n, k, r, patt, div, kind):
    return "rect_%d_%d_%d_%d_%s_%s_%s" % (m, n, k, r, patt or "-", "".join(map(str, div)) or "-", kind)


def test_rect_mm_oracle_matches_reference_rectmm(oracle_mod):
    """The restated one-rank rectMM (rect-class/rectmm.cpp) with numpy's
    OpenBLAS reproduces the subproject's own rectMM bit for bit, including
    its one-rank DFS walk: each k block overwriting C, and with divm, divn > 1
    C blocks of neighbouring columns overlapping (blocks never written keep
    C's starting values)."""
    if not oracle_mod.use_blas(True):
        pytest.skip("numpy OpenBLAS not found")
    mg = _golden_module()
    g = np.load(os.path.join(ROOT, "tests", "golden", "ref_rect.npz"))
    try:
        for m, n, k, r, patt, div, kind, seed in mg.RECT_CASES:
            A, B, C = mg.rect_inputs(m, n, k, kind, seed)
            out = oracle_mod.rect_mm(A, B, C, m, n, k, r, patt, div)
            assert np.array_equal(out, g[_rect_key(m, n, k, r, patt, div, kind)]), (m, n, k, r, patt, div)
    finally:
        oracle_mod.use_blas(False)


def test_rect_mm_oracle_quirks_and_exact_cases(oracle_mod):
    """Integer data, classical leaves: with every divk = 1 and divm or divn
    = 1 at every level the one-rank rectMM is the exact product in the block
    layout; with divk = 2 only the last k block's product survives; a 'b'
    step is rejected (one rank cannot take it)."""
    rng = np.random.default_rng(3)
    m, n, k = 64, 32, 48
    A = rng.integers(-9, 10, m * k).astype(np.float64)
    B = rng.integers(-9, 10, k * n).astype(np.float64)
    C = np.full(m * n, np.nan)
    # r = 1, divisions (2, 1, 1): A blocks of 32 x 48 rows stacked, B whole, C two blocks
    out = oracle_mod.rect_mm(A, B, C, m, n, k, 1, "d", [2, 1, 1])
    Ab = [A[i * 32 * k:(i + 1) * 32 * k].reshape(k, 32).T for i in range(2)]  # column-major blocks
    Bm = B.reshape(n, k).T
    for i in range(2):
        got = out[i * 32 * n:(i + 1) * 32 * n].reshape(n, 32).T
        assert np.array_equal(got, (Ab[i].astype(np.int64) @ Bm.astype(np.int64)).astype(np.float64))
    # divk = 2: C = A(:, last k block) B(last k block, :), each block
    # column-major in its own range
    out = oracle_mod.rect_mm(A, B, C, m, n, k, 1, "d", [1, 1, 2])
    Ak = A[m * 24:].reshape(24, m).T
    Bk = B[24 * n:].reshape(n, 24).T
    assert np.array_equal(out.reshape(n, m).T, (Ak.astype(np.int64) @ Bk.astype(np.int64)).astype(np.float64))
    with pytest.raises(ValueError):
        oracle_mod.rect_mm(A, B, C, m, n, k, 1, "b", [2, 1, 1])
