"""CPU oracle for the CAPS Strassen multiply path -- TEST INFRASTRUCTURE.

Only the tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
use this module, and only as the checker (or as the timed CPU restatement of
the reference's own CPU path).  The product library never imports it.

The C restatement lives in ``caps_oracle.c`` (each function cites the CAPS
source lines it follows).  ``build()`` compiles it with gcc/OpenMP; when
numpy's bundled OpenBLAS is present its ILP64 ``dgemm`` is installed as the
base-case multiply, which is what the reference links (``dgemm-blas.cpp:4-13``).
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "caps_oracle.c")
LIB = os.path.join(HERE, "libcaps_oracle.so")

_lib = None
_blas = None

_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)


def build(force: bool = False) -> str:
    """Compile the oracle shared library (gcc, OpenMP).  Returns its path."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", tmp, SRC, "-lm"])
        os.replace(tmp, LIB)
    return LIB


def reference_dir():
    """Directory of the reference sources, or None where they are absent: the
    CAPS_REFERENCE_DIR environment variable, else the directory
    build_ref.sh built oracle/_ref from (it records it there)."""
    cands = [os.environ.get("CAPS_REFERENCE_DIR")]
    try:
        with open(os.path.join(HERE, "_ref", "REFERENCE_DIR")) as f:
            cands.append(f.read().strip())
    except OSError:
        pass
    for c in cands:
        if c and os.path.isfile(os.path.join(c, "multiply.cpp")):
            return c
    return None


def openblas_path():
    """Path of numpy's bundled ILP64 OpenBLAS, or None."""
    try:
        d = os.path.join(os.path.dirname(np.__file__), os.pardir, "numpy.libs")
        cands = sorted(glob.glob(os.path.join(d, "libscipy_openblas64_*.so")))
        return os.path.realpath(cands[0]) if cands else None
    except Exception:
        return None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.caps_oracle_layout_index.restype = ctypes.c_int64
        L.caps_oracle_layout_index.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int64,
                                               ctypes.c_int64, ctypes.c_int64]
        for f in (L.caps_oracle_to_caps, L.caps_oracle_from_caps):
            f.restype = None
            f.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int64, _dp, _dp]
        L.caps_oracle_multiply.restype = ctypes.c_int
        L.caps_oracle_multiply.argtypes = [_dp, _dp, _dp, ctypes.c_int64, ctypes.c_int,
                                           ctypes.c_int64, ctypes.c_char_p]
        L.caps_oracle_dd_gemm.restype = None
        L.caps_oracle_dd_gemm.argtypes = [ctypes.c_int64, _dp, _dp, _dp, _dp]
        L.caps_oracle_dd_entries.restype = None
        L.caps_oracle_dd_entries.argtypes = [ctypes.c_int64, _dp, _dp, _i64p, _i64p,
                                             ctypes.c_int64, _dp, _dp]
        L.caps_oracle_absprod_entries.restype = None
        L.caps_oracle_absprod_entries.argtypes = [ctypes.c_int64, _dp, _dp, _i64p, _i64p,
                                                  ctypes.c_int64, _dp]
        L.caps_oracle_split_gemm.restype = None
        L.caps_oracle_split_gemm.argtypes = [ctypes.c_int64, _dp, _dp, ctypes.c_int,
                                             ctypes.c_int, _dp]
        L.caps_oracle_set_dgemm.restype = None
        L.caps_oracle_split_gemm_residues.restype = None
        L.caps_oracle_split_gemm_residues.argtypes = [ctypes.c_int64, _dp, _dp, _dp, ctypes.POINTER(ctypes.c_int)]
        L.caps_oracle_rect_mm.restype = ctypes.c_int
        L.caps_oracle_rect_mm.argtypes = [_dp, _dp, _dp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                          ctypes.c_int, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
        L.caps_oracle_split_gemm_residues_bits.restype = None
        L.caps_oracle_split_gemm_residues_bits.argtypes = [ctypes.c_int64, _dp, _dp, _dp, ctypes.POINTER(ctypes.c_int),
                                                           ctypes.c_int]
        L.caps_oracle_set_dgemm.argtypes = [ctypes.c_void_p]
        L.caps_oracle_set_threads.restype = None
        L.caps_oracle_set_threads.argtypes = [ctypes.c_int]
        L.caps_oracle_counters.restype = None
        L.caps_oracle_counters.argtypes = [_i64p, _i64p]
        L.caps_oracle_reset_counters.restype = None
        L.caps_oracle_multiply_sample.restype = ctypes.c_int
        L.caps_oracle_multiply_sample.argtypes = [_dp, _dp, _dp, ctypes.c_int64, ctypes.c_int, ctypes.c_int64,
                                                  ctypes.c_char_p, ctypes.c_int, _dp, _dp]
        L.caps_oracle_chol_mult.restype = None
        L.caps_oracle_chol_mult.argtypes = [_dp, _dp, _dp, ctypes.c_int64, ctypes.c_int, ctypes.c_double]
        L.caps_oracle_set_threads(os.cpu_count() or 1)
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().caps_oracle_set_threads(int(n))
    if _blas is not None:
        _blas.scipy_openblas_set_num_threads64_(ctypes.c_int(int(n)))


def use_blas(enable: bool = True, threads: int | None = None) -> bool:
    """Install numpy's OpenBLAS dgemm as the base case (True if available)."""
    global _blas
    L = lib()
    if not enable:
        L.caps_oracle_set_dgemm(None)
        return False
    path = openblas_path()
    if path is None:
        L.caps_oracle_set_dgemm(None)
        return False
    if _blas is None:
        _blas = ctypes.CDLL(path)
        _blas.scipy_openblas_set_num_threads64_.argtypes = [ctypes.c_int]
        _blas.scipy_openblas_set_num_threads64_.restype = None
    fn = ctypes.cast(_blas.scipy_dgemm_64_, ctypes.c_void_p).value
    L.caps_oracle_set_dgemm(ctypes.c_void_p(fn))
    if threads:
        _blas.scipy_openblas_set_num_threads64_(int(threads))
    return True


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def layout_index(n, nrec, bs, r, c) -> int:
    return int(lib().caps_oracle_layout_index(n, nrec, bs, r, c))


def to_caps(colmajor_flat: np.ndarray, n: int, nrec: int, bs: int = 1) -> np.ndarray:
    out = np.empty(n * n, dtype=np.float64)
    lib().caps_oracle_to_caps(n, nrec, bs, _p(np.ascontiguousarray(colmajor_flat, dtype=np.float64)), _p(out))
    return out


def from_caps(caps_flat: np.ndarray, n: int, nrec: int, bs: int = 1) -> np.ndarray:
    out = np.empty(n * n, dtype=np.float64)
    lib().caps_oracle_from_caps(n, nrec, bs, _p(np.ascontiguousarray(caps_flat, dtype=np.float64)), _p(out))
    return out


def multiply(A: np.ndarray, B: np.ndarray, n: int, nrec: int, bs: int = 1,
             pattern: str | None = None) -> np.ndarray:
    """Strassen-Winograd multiply of CAPS-layout A, B (flat float64)."""
    C = np.empty(n * n, dtype=np.float64)
    pat = pattern.encode() if pattern is not None else None
    rc = lib().caps_oracle_multiply(_p(np.ascontiguousarray(A)), _p(np.ascontiguousarray(B)),
                                    _p(C), n, nrec, bs, pat)
    if rc == -1:
        raise ValueError("Invalid pattern")
    if rc == -2:
        raise ValueError("matrix size not divisible by 2^nrec*bs")
    return C


def chol_mult(C: np.ndarray, A: np.ndarray, B: np.ndarray, n: int, r: int, alpha: float = 1.0) -> np.ndarray:
    """The Cholesky subproject's multiply on one rank (cholesky/mult.cpp:11-137):
    alpha C - A B^T for flat float64 matrices in its recursive layout (the CAPS
    layout with nrec = r, bs = 1).  Returns a new array; C is unread when
    alpha = 0."""
    out = np.array(C, dtype=np.float64, copy=True) if alpha != 0 else np.empty(n * n, dtype=np.float64)
    lib().caps_oracle_chol_mult(_p(out), _p(np.ascontiguousarray(A, dtype=np.float64)),
                                _p(np.ascontiguousarray(B, dtype=np.float64)), n, r, float(alpha))
    return out


def multiply_sample(A: np.ndarray, B: np.ndarray, C: np.ndarray, n: int, nrec: int, bs: int = 1,
                    pattern: str | None = None, child: int = 1):
    """Bounded sample of multiply(): (t_top_sums, t_one_subproduct) in seconds."""
    t_top, t_sub = ctypes.c_double(), ctypes.c_double()
    pat = pattern.encode() if pattern is not None else None
    rc = lib().caps_oracle_multiply_sample(_p(A), _p(B), _p(C), n, nrec, bs, pat, child,
                                           ctypes.byref(t_top), ctypes.byref(t_sub))
    if rc != 0:
        raise ValueError("bad sample arguments")
    return t_top.value, t_sub.value


def counters():
    a, m = ctypes.c_int64(), ctypes.c_int64()
    lib().caps_oracle_counters(ctypes.byref(a), ctypes.byref(m))
    return a.value, m.value


def reset_counters():
    lib().caps_oracle_reset_counters()


def dd_gemm(A_cm: np.ndarray, B_cm: np.ndarray, n: int):
    """Classical product in double-double of column-major n x n A, B: (hi, lo)."""
    hi = np.empty(n * n, dtype=np.float64)
    lo = np.empty(n * n, dtype=np.float64)
    lib().caps_oracle_dd_gemm(n, _p(np.ascontiguousarray(A_cm)), _p(np.ascontiguousarray(B_cm)), _p(hi), _p(lo))
    return hi, lo


def dd_entries(A_cm: np.ndarray, B_cm: np.ndarray, n: int, rows, cols):
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    hi = np.empty(len(rows), dtype=np.float64)
    lo = np.empty(len(rows), dtype=np.float64)
    lib().caps_oracle_dd_entries(n, _p(np.ascontiguousarray(A_cm)), _p(np.ascontiguousarray(B_cm)),
                                 rows.ctypes.data_as(_i64p), cols.ctypes.data_as(_i64p), len(rows),
                                 _p(hi), _p(lo))
    return hi, lo


def absprod_entries(A_cm, B_cm, n, rows, cols):
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    out = np.empty(len(rows), dtype=np.float64)
    lib().caps_oracle_absprod_entries(n, _p(np.ascontiguousarray(A_cm)), _p(np.ascontiguousarray(B_cm)),
                                      rows.ctypes.data_as(_i64p), cols.ctypes.data_as(_i64p), len(rows),
                                      _p(out))
    return out


def split_gemm(A_cm: np.ndarray, B_cm: np.ndarray, m: int, s: int, nd: int) -> np.ndarray:
    """Exact CPU model of the split-integer leaf product (column-major)."""
    C = np.empty(m * m, dtype=np.float64)
    lib().caps_oracle_split_gemm(m, _p(np.ascontiguousarray(A_cm)), _p(np.ascontiguousarray(B_cm)),
                                 int(s), int(nd), _p(C))
    return C


def split_gemm_residues(A_cm: np.ndarray, B_cm: np.ndarray, m: int, bits: int = 55):
    """Exact CPU model of the residue scheme's leaf product (column-major):
    the 128-bit integer product of the scaled operands, rounded once.
    bits: cap on the operand bits (55 unless the tuner or caller asks fewer).
    Returns (C, (t_a, t_b))."""
    C = np.empty(m * m, dtype=np.float64)
    t = (ctypes.c_int * 2)()
    lib().caps_oracle_split_gemm_residues_bits(m, _p(np.ascontiguousarray(A_cm)), _p(np.ascontiguousarray(B_cm)),
                                               _p(C), t, int(bits))
    return C, (t[0], t[1])


def rect_mm(A: np.ndarray, B: np.ndarray, C: np.ndarray, m: int, n: int, k: int, r: int, patt: str,
            div) -> np.ndarray:
    """One-rank rectMM (rect-class/rectmm.cpp) of A (m x k) and B (k x n) in
    the subproject's block layout, onto a copy of C (blocks the reference
    never writes keep C's entries).  div: 3 r division factors (m, n, k per
    level).  Raises ValueError for a step one rank cannot take."""
    out = np.array(C, dtype=np.float64, copy=True)
    d = (ctypes.c_int * max(1, 3 * r))(*[int(x) for x in div])
    st = lib().caps_oracle_rect_mm(_p(np.ascontiguousarray(A)), _p(np.ascontiguousarray(B)), _p(out), m, n, k,
                                   int(r), patt.encode() if patt else b"", d)
    if st:
        raise ValueError("rectMM on one rank takes 'd' steps only")
    return out


# ---------------------------------------------------------------------------
# input streams and error metrics shared by tests and bench
# ---------------------------------------------------------------------------

def drand48_stream(count: int, seed: int | None = None) -> np.ndarray:
    """2*drand48()-1 values as randombenchmark.cpp:19-22 draws them.

    drand48 is the 48-bit LCG x <- (0x5DEECE66D x + 0xB) mod 2^48 with
    x0 = 0 (glibc's state before any seeding) or (seed << 16) | 0x330E after
    srand48(seed); the double is x / 2^48.
    """
    a, c, mask = 0x5DEECE66D, 0xB, (1 << 48) - 1
    x0 = 0 if seed is None else (((seed & 0xFFFFFFFF) << 16) | 0x330E)
    # jump-ahead by blocks: x_{i+1} = a x_i + c; vectorise with powers of a
    out = np.empty(count, dtype=np.float64)
    blk = 1 << 16
    # coefficients for x_{k} = A_k x_0 + C_k (mod 2^48), k = 1..blk
    Ak = np.empty(blk, dtype=object)
    Ck = np.empty(blk, dtype=object)
    A_, C_ = 1, 0
    for k in range(blk):
        A_ = (A_ * a) & mask
        C_ = (C_ * a + c) & mask
        Ak[k] = A_
        Ck[k] = C_
    Ak_u = np.array([int(v) for v in Ak], dtype=np.uint64)
    Ck_u = np.array([int(v) for v in Ck], dtype=np.uint64)
    x = x0
    pos = 0
    while pos < count:
        n = min(blk, count - pos)
        # 48-bit products without overflow: split x into 24-bit halves
        xl, xh = np.uint64(x & 0xFFFFFF), np.uint64(x >> 24)
        A = Ak_u[:n]
        al, ah = A & np.uint64(0xFFFFFF), A >> np.uint64(24)
        m48 = np.uint64(mask)
        v = (al * xl + ((al * xh + ah * xl) << np.uint64(24)) + Ck_u[:n]) & m48
        out[pos:pos + n] = 2.0 * (v.astype(np.float64) / float(1 << 48)) - 1.0
        x = int(v[-1])
        pos += n
    return out


def error_metrics(C: np.ndarray, hi: np.ndarray, lo: np.ndarray, absprod: np.ndarray) -> dict:
    """Error of C against the double-double classical product.

    elementwise = max_ij |C - C_dd|_ij / (|A||B|)_ij
    normwise    = ||C - C_dd||_F / ||C_dd||_F   (over the same entries)
    """
    d = (C - hi) - lo
    ew = np.max(np.abs(d) / np.where(absprod > 0, absprod, 1.0)) if d.size else 0.0
    ref = hi + lo
    nw = float(np.linalg.norm(d) / max(np.linalg.norm(ref), 1e-300))
    return {"max_elementwise_rel": float(ew), "normwise_rel": nw}
