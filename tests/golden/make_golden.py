"""Generates the committed golden fixtures under tests/golden/.

Run in the build container, where the reference sources and its unmodified
one-rank build (oracle/build_ref.sh -> oracle/_ref/libcapsref.so) exist:

    python tests/golden/make_golden.py [REFERENCE_DIR]

1. ref_tests.npz -- the reference's own integer known-answer tests
   (tests/test{28,42,56,196,294,392}.{in,correct,params}): A and B as uint8,
   the SHA-256 of the exact int64 product (checked equal to .correct here),
   and every valid one-rank (-b, -r) parameter pair from the .params files.
2. ref_float.npz -- outputs of the reference's own multiply() (numpy's
   OpenBLAS dgemm at the leaves) on seeded uniform[-1,1) inputs in CAPS
   layout; the oracle with the same BLAS must reproduce them bit for bit.
3. ref_layout.npz -- the reference's distributeFrom1Proc applied to the ramp
   0..n^2-1 (column-major), i.e. the CAPS layout permutation.
4. ref_chol.npz -- outputs of the Cholesky subproject's own mult()
   (cholesky/mult.cpp, one rank; oracle/_ref/libcholref.so) on seeded
   inputs in its recursive layout: C = alpha C - A B^T.
5. ref_rect.npz -- outputs of the rectangular subproject's own rectMM()
   (rect-class/rectmm.cpp, one rank, DFS steps; oracle/_ref/librectref.so)
   on seeded inputs in its block layout, C starting from seeded values.

`python tests/golden/make_golden.py [REFERENCE_DIR] [NAME ...]` regenerates
only the named fixtures (tests, float, layout, chol, rect) when names are
given.
"""
import ctypes
import hashlib
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def read_matrix_file(path):
    with open(path) as f:
        toks = f.read().split()
    return toks


def ref_tests(refdir):
    out = {}
    sizes = [28, 42, 56, 196, 294, 392]
    for n in sizes:
        toks = read_matrix_file(os.path.join(refdir, "tests", "test%d.in" % n))
        assert int(toks[0]) == n
        vals = np.array([int(float(t)) for t in toks[1:]], dtype=np.int64)
        A = vals[: n * n].reshape(n, n)
        B = vals[n * n: 2 * n * n].reshape(n, n)
        C = np.array([int(float(t)) for t in read_matrix_file(os.path.join(refdir, "tests", "test%d.correct" % n))],
                     dtype=np.int64).reshape(n, n)
        assert np.array_equal(A @ B, C), "numpy product differs from test%d.correct" % n
        params = []
        with open(os.path.join(refdir, "tests", "test%d.params" % n)) as f:
            for line in f:
                m = re.search(r"-n (\d+) .* -b (\d+) -r (\d+)", line)
                if m and m.group(1) == "1":
                    params.append((int(m.group(2)), int(m.group(3))))
        out["A%d" % n] = A.astype(np.uint8)
        out["B%d" % n] = B.astype(np.uint8)
        out["C%d_sha256" % n] = np.frombuffer(hashlib.sha256(C.tobytes()).digest(), dtype=np.uint8)
        out["params%d" % n] = np.array(params, dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "ref_tests.npz"), **out)
    print("ref_tests.npz:", sum(len(out["params%d" % n]) for n in sizes), "one-rank parameter lines")


class Desc(ctypes.Structure):
    _fields_ = [(f, ctypes.c_int) for f in ("lda", "nrec", "nproc", "nprocr", "nprocc", "nproc_summa", "bs")]


FLOAT_CASES = [(56, 2, 1, "dd", 11), (64, 3, 2, "ddd", 12), (96, 1, 4, None, 13), (128, 2, 1, "dd", 14)]


def ref_float(reflib):
    L = ctypes.CDLL(reflib)
    mul = getattr(L, "_Z8multiplyPdS_S_13MatDescriptorPc")
    dp = ctypes.POINTER(ctypes.c_double)
    mul.argtypes = [dp, dp, dp, Desc, ctypes.c_char_p]
    mul.restype = None
    out = {}
    for n, r, bs, pat, seed in FLOAT_CASES:
        rng = np.random.default_rng(seed)
        A = rng.uniform(-1, 1, n * n)
        B = rng.uniform(-1, 1, n * n)
        C = np.zeros(n * n)
        mul(A.ctypes.data_as(dp), B.ctypes.data_as(dp), C.ctypes.data_as(dp), Desc(n, r, 1, 1, 1, 1, bs),
            pat.encode() if pat else None)
        out["C_%d_%d_%d" % (n, r, bs)] = C
    np.savez_compressed(os.path.join(HERE, "ref_float.npz"), **out)
    print("ref_float.npz:", list(out))


def ref_layout(reflib):
    L = ctypes.CDLL(reflib)
    dist = getattr(L, "_Z19distributeFrom1Proc13MatDescriptorPdS0_")
    dp = ctypes.POINTER(ctypes.c_double)
    dist.argtypes = [Desc, dp, dp]
    dist.restype = None
    out = {}
    for n, r, bs in [(56, 2, 7), (56, 3, 1), (48, 2, 4), (28, 0, 4), (64, 3, 2)]:
        I = np.arange(n * n, dtype=np.float64)
        O = np.zeros(n * n)
        dist(Desc(n, r, 1, 1, 1, 1, bs), O.ctypes.data_as(dp), I.ctypes.data_as(dp))
        out["perm_%d_%d_%d" % (n, r, bs)] = O.astype(np.int32)
    np.savez_compressed(os.path.join(HERE, "ref_layout.npz"), **out)
    print("ref_layout.npz:", list(out))


# The Cholesky subproject's mult() (C = alpha C - A B^T, cholesky/mult.cpp),
# one rank: (n, r, alpha, kind, seed).  n = 2048 > 1024 runs its DFS branch;
# that output is stored as a SHA-256 (the test regenerates the inputs).
CHOL_CASES = [(32, 0, 1.0, "float", 21), (64, 2, 1.0, "float", 22), (96, 1, 0.0, "float", 23),
              (128, 3, 2.5, "float", 24), (56, 2, 1.0, "int", 25), (2048, 2, 1.0, "float", 26),
              (2048, 1, 0.5, "int", 27)]


def chol_inputs(n, kind, seed):
    rng = np.random.default_rng(seed)
    if kind == "int":
        return [rng.integers(-9, 10, n * n).astype(np.float64) for _ in range(3)]
    return [rng.uniform(-1, 1, n * n) for _ in range(3)]


def ref_chol(chollib):
    L = ctypes.CDLL(chollib)
    argc = ctypes.c_int(0)
    argv = ctypes.POINTER(ctypes.c_char_p)()
    getattr(L, "_Z17initCommunicationPiPPPc")(ctypes.byref(argc), ctypes.byref(argv))
    getattr(L, "_Z10initTimersv")()
    init_sizes = getattr(L, "_Z9initSizesiii")
    init_sizes.argtypes = [ctypes.c_int] * 3
    mult = getattr(L, "_Z4multPdS_S_iiid")
    dp = ctypes.POINTER(ctypes.c_double)
    mult.argtypes = [dp, dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
    mult.restype = None
    out = {}
    for n, r, alpha, kind, seed in CHOL_CASES:
        A, B, C = chol_inputs(n, kind, seed)
        init_sizes(1, r, n)
        mult(C.ctypes.data_as(dp), A.ctypes.data_as(dp), B.ctypes.data_as(dp), n, 1, r, alpha)
        key = "chol_%d_%d_%s" % (n, r, kind)
        if n > 256:
            out[key + "_sha256"] = np.frombuffer(hashlib.sha256(C.tobytes()).digest(), dtype=np.uint8)
        else:
            out[key] = C
    np.savez_compressed(os.path.join(HERE, "ref_chol.npz"), **out)
    print("ref_chol.npz:", list(out))


# The rectangular subproject's rectMM (rect-class/rectmm.cpp), one rank, DFS
# steps: (m, n, k, r, pattern, divisions, kind, seed).  C starts from seeded
# values: the blocks the reference's one-rank walk never writes keep them.
RECT_CASES = [(64, 48, 32, 0, "", [], "float", 31), (64, 48, 32, 1, "d", [2, 2, 1], "float", 32),
              (64, 48, 32, 1, "d", [1, 1, 2], "int", 33), (96, 64, 48, 2, "dd", [2, 2, 2, 3, 2, 2], "int", 34),
              (60, 40, 24, 2, "dD", [3, 2, 1, 2, 2, 3], "float", 35),
              (128, 128, 128, 2, "dd", [1, 2, 1, 2, 1, 1], "int", 36),
              (256, 96, 512, 1, "d", [2, 3, 4], "float", 37)]


def rect_inputs(m, n, k, kind, seed):
    rng = np.random.default_rng(seed)
    if kind == "int":
        return [rng.integers(-9, 10, size).astype(np.float64) for size in (m * k, k * n, m * n)]
    return [rng.uniform(-1, 1, size) for size in (m * k, k * n, m * n)]


def ref_rect(rectlib):
    L = ctypes.CDLL(rectlib)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    init = getattr(L, "_Z13initSizesRectiiiiiPi")
    init.argtypes = [ctypes.c_int] * 5 + [ip]
    rect = getattr(L, "_Z6rectMMPdS_S_iiiiiPcPi")
    rect.argtypes = [dp, dp, dp] + [ctypes.c_int] * 5 + [ctypes.c_char_p, ip]
    rect.restype = None
    out = {}
    for m, n, k, r, patt, div, kind, seed in RECT_CASES:
        A, B, C = rect_inputs(m, n, k, kind, seed)
        d = (ctypes.c_int * max(1, 3 * r))(*div)
        init(m, n, k, 1, r, d)
        rect(A.ctypes.data_as(dp), B.ctypes.data_as(dp), C.ctypes.data_as(dp), m, n, k, 1, r, patt.encode(), d)
        out["rect_%d_%d_%d_%d_%s_%s_%s" % (m, n, k, r, patt or "-", "".join(map(str, div)) or "-", kind)] = C
    np.savez_compressed(os.path.join(HERE, "ref_rect.npz"), **out)
    print("ref_rect.npz:", list(out))


if __name__ == "__main__":
    refdir = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    names = set(sys.argv[2:]) or {"tests", "float", "layout", "chol", "rect"}
    reflib = os.path.join(ROOT, "oracle", "_ref", "libcapsref.so")
    if "tests" in names:
        ref_tests(refdir)
    if "float" in names:
        ref_float(reflib)
    if "layout" in names:
        ref_layout(reflib)
    if "chol" in names:
        ref_chol(os.path.join(ROOT, "oracle", "_ref", "libcholref.so"))
    if "rect" in names:
        ref_rect(os.path.join(ROOT, "oracle", "_ref", "librectref.so"))
