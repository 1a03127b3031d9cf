"""caps_gb300 -- CAPS Strassen multiply on one GB300 GPU.

Python mirror of the reference's multiply interface (multiply.h:13,
matrix.h:8-16, communication.h:34-35) over the C ABI of libcaps_gb300.so
(include/caps_gb300.h).  Device arrays are torch CUDA tensors (float64,
contiguous); host arrays are numpy float64 arrays.  Errors raise CapsError
carrying the library status; an invalid pattern raises with the reference's
message "Invalid pattern" (multiply.cpp:100-104).

There is no CPU fallback: if the CUDA library is missing, importing a
function that needs it raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libcaps_gb300.so")

CAPS_FORM_PLAIN = 0
CAPS_FORM_SPLIT = 1

STATUS = {
    0: "CAPS_OK",
    1: "CAPS_ERR_INVALID_PATTERN",
    2: "CAPS_ERR_SIZE",
    3: "CAPS_ERR_BUDGET",
    4: "CAPS_ERR_CUDA",
    5: "CAPS_ERR_ALLOC",
    6: "CAPS_ERR_TIMEOUT",
    7: "CAPS_ERR_UNSUPPORTED",
    8: "CAPS_ERR_ARG",
}

# every extern "C" function of include/caps_gb300.h
C_ABI_SYMBOLS = [
    "caps_options_init", "caps_multiply_dev", "caps_multiply_host", "caps_to_caps_layout_dev",
    "caps_from_caps_layout_dev", "caps_leaf_gemm_dev", "caps_workspace_size", "caps_resolve_pattern",
    "caps_get_counters", "caps_reset_counters", "caps_set_phase_timing", "caps_multiply_batched_dev",
    "caps_status_string", "caps_last_cuda_error", "caps_debug_fail_allocations", "caps_release_cache",
    "caps_leaf_gemm_split_noalloc_dev", "caps_autotune_entry", "caps_chol_mult_dev", "caps_chol_mult_host",
    "caps_debug_starve_split_gemm", "caps_autotune_entry_ex", "caps_autotune_info",
    "caps_rect_mm_dev", "caps_rect_mm_host", "caps_debug_tune_cache_line",
]


class CapsError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status
        self.name = STATUS.get(status, str(status))


class MatDescriptor(ctypes.Structure):
    """struct MatDescriptor (matrix.h:8-16); one rank: nproc = nprocr = nprocc = nproc_summa = 1."""
    _fields_ = [("lda", ctypes.c_int), ("nrec", ctypes.c_int), ("nproc", ctypes.c_int),
                ("nprocr", ctypes.c_int), ("nprocc", ctypes.c_int), ("nproc_summa", ctypes.c_int),
                ("bs", ctypes.c_int)]

    @classmethod
    def make(cls, lda: int, nrec: int, bs: int = 1, hybrid: int = 1) -> "MatDescriptor":
        """hybrid: subproducts an 'h' step runs at once (the nproc_summa field)."""
        return cls(lda, nrec, 1, 1, 1, int(hybrid), bs)


class TuneInfo(ctypes.Structure):
    """caps_tune_info: one autotuner choice with all its axes."""
    _fields_ = [("n", ctypes.c_int), ("form", ctypes.c_int), ("nrec", ctypes.c_int), ("pattern", ctypes.c_char * 8),
                ("scheme", ctypes.c_int), ("tile_rows", ctypes.c_int), ("tile_cols", ctypes.c_int),
                ("operand_bits", ctypes.c_int), ("moduli", ctypes.c_int), ("gate_rejected", ctypes.c_int),
                ("leaf_gate", ctypes.c_int), ("from_cache", ctypes.c_int), ("seconds", ctypes.c_double)]


class Options(ctypes.Structure):
    _fields_ = [("form", ctypes.c_int), ("slices", ctypes.c_int), ("diagonals", ctypes.c_int),
                ("split_scheme", ctypes.c_int), ("workspace_limit", ctypes.c_longlong),
                ("plain_tile", ctypes.c_int), ("operand_bits", ctypes.c_int),
                ("reserved", ctypes.c_longlong * 3)]


class Counters(ctypes.Structure):
    _fields_ = [("additions", ctypes.c_longlong), ("multiplications", ctypes.c_longlong),
                ("time_add", ctypes.c_double), ("time_mul", ctypes.c_double),
                ("time_rearrange", ctypes.c_double), ("workspace_peak_bytes", ctypes.c_longlong),
                ("split_slices", ctypes.c_int), ("split_diagonals", ctypes.c_int),
                ("kernel_launches", ctypes.c_longlong), ("time_leaf_gemm", ctypes.c_double),
                ("leaf_gemm_launches", ctypes.c_longlong), ("leaf_gemm_m3", ctypes.c_double),
                ("add_bytes", ctypes.c_longlong), ("split_moduli", ctypes.c_int), ("split_pad", ctypes.c_int),
                ("host_first_inputs", ctypes.c_double), ("host_all_inputs", ctypes.c_double),
                ("host_compute_end", ctypes.c_double), ("host_copy_back_end", ctypes.c_double)]


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded libcaps_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libcaps_gb300.so is not built (run caps_gb300/build.py); "
                              "there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        vp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
        D = MatDescriptor
        OP = ctypes.POINTER(Options)
        L.caps_options_init.argtypes = [OP]
        L.caps_options_init.restype = None
        L.caps_multiply_dev.argtypes = [vp, vp, vp, D, ctypes.c_char_p, OP, vp]
        L.caps_multiply_dev.restype = ctypes.c_int
        L.caps_multiply_host.argtypes = [dp, dp, dp, D, ctypes.c_char_p, OP]
        L.caps_multiply_host.restype = ctypes.c_int
        L.caps_to_caps_layout_dev.argtypes = [vp, vp, D, vp]
        L.caps_to_caps_layout_dev.restype = ctypes.c_int
        L.caps_from_caps_layout_dev.argtypes = [vp, vp, D, vp]
        L.caps_from_caps_layout_dev.restype = ctypes.c_int
        L.caps_leaf_gemm_dev.argtypes = [vp, vp, vp, ctypes.c_int, OP, vp]
        L.caps_leaf_gemm_dev.restype = ctypes.c_int
        L.caps_workspace_size.argtypes = [D, ctypes.c_char_p, OP, ctypes.POINTER(ctypes.c_longlong)]
        L.caps_workspace_size.restype = ctypes.c_int
        L.caps_resolve_pattern.argtypes = [D, ctypes.c_char_p, OP, ctypes.c_char_p, ctypes.c_int]
        L.caps_resolve_pattern.restype = ctypes.c_int
        L.caps_get_counters.argtypes = [ctypes.POINTER(Counters)]
        L.caps_get_counters.restype = None
        L.caps_reset_counters.argtypes = []
        L.caps_reset_counters.restype = None
        L.caps_set_phase_timing.argtypes = [ctypes.c_int]
        L.caps_set_phase_timing.restype = None
        L.caps_multiply_batched_dev.argtypes = [ctypes.c_int, vp, vp, vp, ctypes.POINTER(ctypes.c_int), OP, vp]
        L.caps_multiply_batched_dev.restype = ctypes.c_int
        L.caps_status_string.argtypes = [ctypes.c_int]
        L.caps_status_string.restype = ctypes.c_char_p
        L.caps_last_cuda_error.argtypes = []
        L.caps_last_cuda_error.restype = ctypes.c_char_p
        L.caps_debug_fail_allocations.argtypes = [ctypes.c_int]
        L.caps_debug_fail_allocations.restype = None
        L.caps_debug_starve_split_gemm.argtypes = [ctypes.c_int]
        L.caps_debug_starve_split_gemm.restype = None
        L.caps_release_cache.argtypes = []
        L.caps_release_cache.restype = None
        L.caps_leaf_gemm_split_noalloc_dev.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]
        L.caps_leaf_gemm_split_noalloc_dev.restype = ctypes.c_int
        i_, d_ = ctypes.c_int, ctypes.c_double
        L.caps_chol_mult_dev.argtypes = [vp, vp, vp, i_, i_, i_, d_, ctypes.c_char_p, OP, vp]
        L.caps_chol_mult_dev.restype = ctypes.c_int
        L.caps_chol_mult_host.argtypes = [dp, dp, dp, i_, i_, i_, d_, ctypes.c_char_p, OP]
        L.caps_chol_mult_host.restype = ctypes.c_int
        ip = ctypes.POINTER(ctypes.c_int)
        L.caps_autotune_entry.argtypes = [ctypes.c_int, ip, ip, ip, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]
        L.caps_autotune_entry.restype = ctypes.c_int
        L.caps_autotune_entry_ex.argtypes = [ctypes.c_int, ip, ip, ip, ctypes.c_char_p, ip, ip,
                                             ctypes.POINTER(ctypes.c_double)]
        L.caps_autotune_entry_ex.restype = ctypes.c_int
        L.caps_rect_mm_dev.argtypes = [vp, vp, vp, i_, i_, i_, i_, ctypes.c_char_p, ip, vp]
        L.caps_rect_mm_dev.restype = ctypes.c_int
        L.caps_rect_mm_host.argtypes = [dp, dp, dp, i_, i_, i_, i_, ctypes.c_char_p, ip]
        L.caps_rect_mm_host.restype = ctypes.c_int
        L.caps_autotune_info.argtypes = [ctypes.c_int, ctypes.POINTER(TuneInfo)]
        L.caps_autotune_info.restype = ctypes.c_int
        L.caps_debug_tune_cache_line.argtypes = [ctypes.c_char_p, ctypes.c_char_p, i_, i_, i_, i_,
                                                 ctypes.POINTER(TuneInfo)]
        L.caps_debug_tune_cache_line.restype = ctypes.c_int
        _lib = L
    return _lib


def _check(status: int) -> None:
    if status != 0:
        L = lib()
        msg = L.caps_status_string(status).decode()
        extra = L.caps_last_cuda_error().decode()
        if status == 4 and extra:
            msg = msg + ": " + extra
        raise CapsError(status, msg)


SPLIT_SCHEMES = {"auto": 0, "digits": 1, "residues": 2}


PLAIN_TILES = {"64x64": 0, "32x32": 1, "128x64": 2}


def options(form: int | str = CAPS_FORM_PLAIN, slices: int = 0, diagonals: int = 0,
            workspace_limit: int = 0, scheme: int | str = 0, tile: int | str = 0,
            operand_bits: int = 0) -> Options:
    """caps_options.  tile: the plain form's DMMA tile ("64x64", "32x32",
    "128x64"); operand_bits: the residue scheme's operand-bit cap (0 = 55; -1:
    chosen by the library per leaf size under its accuracy gate)."""
    if isinstance(form, str):
        form = {"plain": CAPS_FORM_PLAIN, "split": CAPS_FORM_SPLIT}[form]
    if isinstance(scheme, str):
        scheme = SPLIT_SCHEMES[scheme]
    o = Options()
    lib().caps_options_init(ctypes.byref(o))
    o.form, o.slices, o.diagonals, o.workspace_limit = int(form), int(slices), int(diagonals), int(workspace_limit)
    o.split_scheme = int(scheme)
    o.plain_tile = PLAIN_TILES[tile] if isinstance(tile, str) else int(tile)
    o.operand_bits = int(operand_bits)
    return o


def _pat(pattern):
    if pattern is None:
        return None
    return pattern.encode() if isinstance(pattern, str) else bytes(pattern)


def _dev_ptr(t, name):
    import torch
    if not (isinstance(t, torch.Tensor) and t.is_cuda):
        raise TypeError("%s must be a CUDA tensor" % name)
    if t.dtype != torch.float64 or not t.is_contiguous():
        raise TypeError("%s must be contiguous float64" % name)
    return ctypes.c_void_p(t.data_ptr())


def _stream_ptr(stream):
    if stream is None:
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return ctypes.c_void_p(int(stream))


def multiply(A, B, C, desc: MatDescriptor, pattern=None, form: int | str = CAPS_FORM_PLAIN,
             slices: int = 0, diagonals: int = 0, workspace_limit: int = 0, stream=None,
             scheme: int | str = 0, tile: int | str = 0, operand_bits: int = 0) -> None:
    """C = A * B for CAPS-layout matrices (multiply.h:13).

    Torch CUDA tensors run asynchronously on `stream` (default: torch's
    current stream); numpy arrays go through the host entry point, which
    stages the copies and synchronises.  scheme: split-form operand cut
    ("auto", "digits" or "residues"); tile, operand_bits: see options().
    """
    opt = options(form, slices, diagonals, workspace_limit, scheme, tile, operand_bits)
    if isinstance(A, np.ndarray):
        for x in (A, B, C):
            if x.dtype != np.float64 or not x.flags.c_contiguous:
                raise TypeError("host arrays must be contiguous float64")
        dp = ctypes.POINTER(ctypes.c_double)
        _check(lib().caps_multiply_host(A.ctypes.data_as(dp), B.ctypes.data_as(dp), C.ctypes.data_as(dp),
                                        desc, _pat(pattern), ctypes.byref(opt)))
        return
    _check(lib().caps_multiply_dev(_dev_ptr(A, "A"), _dev_ptr(B, "B"), _dev_ptr(C, "C"), desc, _pat(pattern),
                                   ctypes.byref(opt), _stream_ptr(stream)))


def leaf_gemm(A, B, C, m: int, form: int | str = CAPS_FORM_PLAIN, slices: int = 0, diagonals: int = 0,
              stream=None, scheme: int | str = 0, tile: int | str = 0, operand_bits: int = 0) -> None:
    """Base case alone: column-major m x m C = A * B on the device."""
    opt = options(form, slices, diagonals, 0, scheme, tile, operand_bits)
    _check(lib().caps_leaf_gemm_dev(_dev_ptr(A, "A"), _dev_ptr(B, "B"), _dev_ptr(C, "C"), int(m),
                                    ctypes.byref(opt), _stream_ptr(stream)))


def chol_mult(C, A, B, n: int, r: int, alpha: float = 1.0, x: int = 1, pattern=None,
              form: int | str = CAPS_FORM_PLAIN, slices: int = 0, diagonals: int = 0, stream=None,
              scheme: int | str = 0, operand_bits: int = 0) -> None:
    """The Cholesky subproject's multiply (cholesky/mult.h:6, mult.cpp:11-28 on
    one rank): C = alpha C - A B^T on n x n matrices in its recursive layout
    with r levels (the CAPS layout with nrec = r, bs = 1).  The product runs
    as this library's Strassen-Winograd multiply with r levels.  alpha = 0
    leaves C unread.  Torch CUDA tensors run on `stream`; numpy arrays go
    through the host entry point.  operand_bits: see options()."""
    opt = options(form, slices, diagonals, 0, scheme, 0, operand_bits)
    if isinstance(A, np.ndarray):
        for t in (A, B, C):
            if t.dtype != np.float64 or not t.flags.c_contiguous:
                raise TypeError("host arrays must be contiguous float64")
        dp = ctypes.POINTER(ctypes.c_double)
        _check(lib().caps_chol_mult_host(C.ctypes.data_as(dp), A.ctypes.data_as(dp), B.ctypes.data_as(dp),
                                         int(n), int(x), int(r), float(alpha), _pat(pattern), ctypes.byref(opt)))
        return
    _check(lib().caps_chol_mult_dev(_dev_ptr(C, "C"), _dev_ptr(A, "A"), _dev_ptr(B, "B"), int(n), int(x), int(r),
                                    float(alpha), _pat(pattern), ctypes.byref(opt), _stream_ptr(stream)))


def rect_mm(A, B, C, m: int, n: int, k: int, r: int = 0, pattern: str = "", div=(), stream=None) -> None:
    """The rectangular subproject's rectMM on one rank (rect-class/rectmm.h:1):
    C = A B with A m x k, B k x n, C m x n in its block layout, r levels of
    'd' steps with the division triples `div` (3 r ints: m, n, k per level).
    Torch CUDA tensors run on `stream`; numpy arrays go through the host
    entry point (C is copied in too: blocks the one-rank walk never writes
    keep their entries)."""
    d = (ctypes.c_int * max(1, 3 * int(r)))(*[int(x) for x in div])
    pat = _pat(pattern) if r > 0 else b""
    if isinstance(A, np.ndarray):
        for t in (A, B, C):
            if t.dtype != np.float64 or not t.flags.c_contiguous:
                raise TypeError("host arrays must be contiguous float64")
        dp = ctypes.POINTER(ctypes.c_double)
        _check(lib().caps_rect_mm_host(A.ctypes.data_as(dp), B.ctypes.data_as(dp), C.ctypes.data_as(dp), int(m),
                                       int(n), int(k), int(r), pat, d))
        return
    _check(lib().caps_rect_mm_dev(_dev_ptr(A, "A"), _dev_ptr(B, "B"), _dev_ptr(C, "C"), int(m), int(n), int(k),
                                  int(r), pat, d, _stream_ptr(stream)))


NOALLOC_MAX_M = 512


def leaf_gemm_split_noalloc(A, B, C, m: int, slices: int = 0, diagonals: int = 0, stream=None) -> None:
    """Split-form base case that allocates nothing (scratch in a static device
    array; 1 <= m <= 512; synchronises the stream)."""
    _check(lib().caps_leaf_gemm_split_noalloc_dev(_dev_ptr(A, "A"), _dev_ptr(B, "B"), _dev_ptr(C, "C"), int(m),
                                                  int(slices), int(diagonals), _stream_ptr(stream)))


def to_caps_layout(colmajor, out, desc: MatDescriptor, stream=None) -> None:
    """distributeFrom1Proc (communication.cpp:612-657) on the device."""
    _check(lib().caps_to_caps_layout_dev(_dev_ptr(colmajor, "colmajor"), _dev_ptr(out, "out"), desc,
                                         _stream_ptr(stream)))


def from_caps_layout(caps, out, desc: MatDescriptor, stream=None) -> None:
    """collectTo1Proc (communication.cpp:661-708) on the device."""
    _check(lib().caps_from_caps_layout_dev(_dev_ptr(caps, "caps"), _dev_ptr(out, "out"), desc,
                                           _stream_ptr(stream)))


def multiply_batched(As, Bs, Cs, ns, form: int | str = CAPS_FORM_PLAIN, slices: int = 0, stream=None,
                     scheme: int | str = 0) -> None:
    """Independent column-major multiplies of uneven sizes (lists of CUDA tensors)."""
    count = len(As)
    arr = ctypes.c_void_p * count
    pa = arr(*[_dev_ptr(a, "A").value for a in As])
    pb = arr(*[_dev_ptr(b, "B").value for b in Bs])
    pc = arr(*[_dev_ptr(c, "C").value for c in Cs])
    nn = (ctypes.c_int * count)(*[int(n) for n in ns])
    opt = options(form, slices, 0, 0, scheme)
    _check(lib().caps_multiply_batched_dev(count, ctypes.cast(pa, ctypes.c_void_p), ctypes.cast(pb, ctypes.c_void_p),
                                           ctypes.cast(pc, ctypes.c_void_p), nn, ctypes.byref(opt),
                                           _stream_ptr(stream)))


def autotune_table() -> list:
    """The autotuner's choices so far (caps_autotune_info): dicts of n, form,
    nrec, pattern, the split scheme chosen ("residues" / "digits"; None for
    the plain form), the base-case tile, the residues' operand bits and
    moduli (0 otherwise), the bit caps the accuracy gate turned down, whether
    the entry came from the on-disk cache, and seconds per instance."""
    out = []
    i = 0
    while True:
        t = TuneInfo()
        if lib().caps_autotune_info(i, ctypes.byref(t)):
            return out
        out.append(_tune_dict(t))
        i += 1


def _tune_dict(t: TuneInfo) -> dict:
    names = {0: None, 1: "digits", 2: "residues"}
    return {"n": t.n, "form": "split" if t.form == 1 else "plain", "nrec": t.nrec,
            "pattern": t.pattern.decode(), "scheme": names.get(t.scheme, t.scheme),
            "tile": [t.tile_rows, t.tile_cols], "operand_bits": t.operand_bits, "moduli": t.moduli,
            "gate_rejected": t.gate_rejected, "leaf_gate": bool(t.leaf_gate),
            "from_cache": bool(t.from_cache),
            "seconds_per_instance": t.seconds}


def debug_tune_cache_line(line: str, device_key: str, n: int, form: int | str = CAPS_FORM_SPLIT,
                          slices: int = 0, scheme: int | str = 0):
    """caps_debug_tune_cache_line: the choice one line of the autotuner's
    on-disk cache gives for size n under (form, slices, scheme) on the device
    keyed `device_key`, as an autotune_table() entry, or None when the line
    does not apply or is damaged.  Host only: no device call."""
    if isinstance(form, str):
        form = {"plain": CAPS_FORM_PLAIN, "split": CAPS_FORM_SPLIT}[form]
    if isinstance(scheme, str):
        scheme = SPLIT_SCHEMES[scheme]
    t = TuneInfo()
    ok = lib().caps_debug_tune_cache_line(line.encode(), device_key.encode(), int(n), int(form), int(slices),
                                          int(scheme), ctypes.byref(t))
    return _tune_dict(t) if ok else None


def workspace_size(desc: MatDescriptor, pattern=None, form: int | str = CAPS_FORM_PLAIN,
                   workspace_limit: int = 0, scheme: int | str = 0) -> int:
    out = ctypes.c_longlong()
    opt = options(form, 0, 0, workspace_limit, scheme)
    _check(lib().caps_workspace_size(desc, _pat(pattern), ctypes.byref(opt), ctypes.byref(out)))
    return out.value


def resolve_pattern(desc: MatDescriptor, pattern=None, form: int | str = CAPS_FORM_PLAIN,
                    workspace_limit: int = 0, scheme: int | str = 0) -> str:
    buf = ctypes.create_string_buffer(desc.nrec + 8)
    opt = options(form, 0, 0, workspace_limit, scheme)
    _check(lib().caps_resolve_pattern(desc, _pat(pattern), ctypes.byref(opt), buf, len(buf)))
    return buf.value.decode()


def counters() -> dict:
    c = Counters()
    lib().caps_get_counters(ctypes.byref(c))
    return {f: getattr(c, f) for f, _ in Counters._fields_}


def reset_counters() -> None:
    lib().caps_reset_counters()


def set_phase_timing(enable: bool) -> None:
    lib().caps_set_phase_timing(1 if enable else 0)


def release_cache() -> None:
    lib().caps_release_cache()


def debug_fail_allocations(count: int) -> None:
    lib().caps_debug_fail_allocations(int(count))


def debug_starve_split_gemm(count: int) -> None:
    """The next `count` split GEMM launches issue no copies: their bounded
    waits give up and the call raises CapsError(CAPS_ERR_TIMEOUT)."""
    lib().caps_debug_starve_split_gemm(int(count))


@dataclass
class Flops:
    effective: float  # 2 n^3
    actual: float     # additions + multiplications as counters.cpp counts them


def digit_pairs(s: int, nd: int) -> int:
    """Digit-pair products of the split form: pairs (a, b), 1 <= a, b <= s, a + b <= nd + 1."""
    return sum(1 for a in range(1, s + 1) for b in range(1, s + 1) if a + b <= nd + 1)


def flop_counts(n: int, nrec: int) -> Flops:
    """Effective 2n^3 and the reference's counted flops (counters.cpp:65-69)."""
    m = n >> nrec
    adds = 0
    for l in range(nrec):
        q = (n >> (l + 1)) ** 2
        adds += 15 * q * 7 ** l
    leaves = 7 ** nrec
    muls = leaves * m ** 3
    adds += leaves * m ** 3
    return Flops(2.0 * n ** 3, float(adds + muls))
