"""CPU tests of the product library: it loads, exports every declared symbol,
and its host-side logic (validation, pattern choice, workspace sizing, error
codes) behaves like the reference's entry points.  No kernel runs here."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle.oracle import reference_dir  # noqa: E402

REF = reference_dir() or ""


def header_functions(path):
    txt = open(path).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(caps_[a-z_0-9]+)\s*\(", txt)))


def test_c_abi_exports_every_declared_symbol(caps):
    declared = header_functions(os.path.join(ROOT, "include", "caps_gb300.h"))
    assert set(caps.C_ABI_SYMBOLS) == set(declared)
    L = caps.lib()
    for name in declared:
        assert hasattr(L, name), name


def test_compat_header_symbols_exported(caps):
    out = subprocess.run(["nm", "-D", "--defined-only", caps.LIB_PATH], stdout=subprocess.PIPE, text=True).stdout
    for mangled in ["_Z8multiplyPdS_S_13MatDescriptorPc", "_Z8allocatex", "_Z10deallocatePdx",
                    "_Z18setAvailableMemoryx", "_Z12enoughMemoryx", "_Z16getMaxUsedMemoryv",
                    "_Z17numEntriesPerProc13MatDescriptor", "_Z19distributeFrom1Proc13MatDescriptorPdS0_",
                    "_Z14collectTo1Proc13MatDescriptorPdS0_", "_Z10initTimersv", "_Z13printCountersd13MatDescriptor",
                    "_Z17initCommunicationPiPPPci", "_Z20initCommunicationAltPiPPPci", "_Z7getRankv",
                    "_Z13getLog7nProcsv", "_Z10getPFactorv", "_Z10read_timerv", "_Z7getCommv",
                    "caps_compat_set_form"]:
        assert mangled in out, mangled
    for name in header_functions(os.path.join(ROOT, "include", "caps_compat.h")):
        assert name in out, name


def test_status_strings_and_validation(caps):
    L = caps.lib()
    assert L.caps_status_string(1).decode() == "Invalid pattern"
    d = caps.MatDescriptor.make(56, 2)
    assert caps.resolve_pattern(d, "db") == "db"
    with pytest.raises(caps.CapsError) as e:
        caps.resolve_pattern(d, "dx")
    assert str(e.value) == "Invalid pattern" and e.value.status == 1
    with pytest.raises(caps.CapsError) as e:
        caps.resolve_pattern(d, "d")          # shorter than nrec
    assert e.value.status == 1
    with pytest.raises(caps.CapsError) as e:
        caps.resolve_pattern(caps.MatDescriptor.make(54, 2))  # 54 % 4 != 0
    assert e.value.status == 2
    with pytest.raises(caps.CapsError) as e:
        caps.resolve_pattern(caps.MatDescriptor(56, 2, 7, 7, 1, 1, 1))  # multi-rank descriptor
    assert e.value.status == 7
    with pytest.raises(caps.CapsError) as e:
        caps.workspace_size(caps.MatDescriptor.make(56, 2), "dd", form=3)
    assert e.value.status == 8


def test_workspace_and_auto_pattern(caps):
    d = caps.MatDescriptor.make(16384, 3)
    q = (8192 ** 2) * 8
    ws_ddd = caps.workspace_size(d, "ddd")
    # a memory-lean 'd' level keeps 3 quarter buffers: 3 q (n/2) + 3 q/4 + 3 q/16
    assert 3 * q * (1 + 1 / 4 + 1 / 16) * 0.99 <= ws_ddd <= 3 * q * (1 + 1 / 4 + 1 / 16) * 1.01
    ws_bbb = caps.workspace_size(d, "bbb")
    assert ws_bbb > ws_ddd
    # a small budget forces 'd' everywhere, a large one allows 'b' at the bottom
    assert caps.resolve_pattern(d, None, workspace_limit=1 << 20) == "ddd"
    p = caps.resolve_pattern(d, None, workspace_limit=64 << 30)
    assert p.endswith("b")
    assert caps.workspace_size(d, None, workspace_limit=64 << 30) <= 64 << 30
    # 'h' behaves as 'd' on one GPU
    assert caps.workspace_size(d, "hhh") == ws_ddd


def test_split_workspace_bounded(caps):
    d = caps.MatDescriptor.make(16384, 3)
    ws = caps.workspace_size(d, "bbb", form="split")
    assert ws < 80 << 30
    # n = 32768, r = 4, 'bbdd' fits a 120 GB (-m 120000) budget in both forms
    d5 = caps.MatDescriptor.make(32768, 4)
    for form in ("split", "plain"):
        assert caps.workspace_size(d5, "bbdd", form=form) <= 120000 * 2 ** 20


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "randombenchmark.cpp")), reason="reference sources absent")
def test_reference_drivers_link_unmodified_against_library(caps, tmp_path):
    """The reference's own randombenchmark.cpp / fromfile1.cpp compile against
    the reference headers and link against libcaps_gb300.so alone (no
    multiply.o / communication.o / memory.o / counters.o / matrix.o / library.o)."""
    shim = os.path.join(ROOT, "oracle", "ref_shim", "mpi.h")
    libdir = os.path.dirname(caps.LIB_PATH)
    for drv in ("randombenchmark", "fromfile1"):
        out = tmp_path / drv
        cmd = ["g++", "-O1", "-w", "-include", shim, "-I" + os.path.dirname(shim), "-I" + REF,
               "-DNUM_THREADS=1", os.path.join(REF, "%s.cpp" % drv), "-o", str(out), "-L" + libdir, "-lcaps_gb300",
               "-Wl,-rpath," + libdir]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert r.returncode == 0, r.stdout


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "cholesky", "test-mult.cpp")),
                    reason="reference sources absent")
def test_cholesky_test_mult_links_against_library(caps, tmp_path):
    """The Cholesky subproject's own test-mult.cpp, with its sizes /
    communication / counters / library objects but without mult.o, links
    against libcaps_gb300.so: its mult() call resolves to the library's."""
    shim = os.path.join(ROOT, "oracle", "ref_shim")
    ref = os.path.join(REF, "cholesky")
    libdir = os.path.dirname(caps.LIB_PATH)
    import numpy
    npl = os.path.realpath(os.path.join(os.path.dirname(numpy.__file__), os.pardir, "numpy.libs"))
    blas = [os.path.join(npl, f) for f in (os.listdir(npl) if os.path.isdir(npl) else [])
            if f.startswith("libscipy_openblas64_")]
    if not blas:
        pytest.skip("numpy's OpenBLAS not found (test-mult checks itself with dgemm)")
    objs = []
    for src in ("test-mult", "sizes", "communication", "counters", "library"):
        o = str(tmp_path / (src + ".o"))
        cmd = ["g++", "-O1", "-w", "-fopenmp", "-DNUM_THREADS=1", "-include", os.path.join(shim, "mpi.h"),
               "-I" + shim, "-I" + ref, "-c", os.path.join(ref, src + ".cpp"), "-o", o]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert r.returncode == 0, r.stdout
        objs.append(o)
    bo = str(tmp_path / "blas_lp64.o")
    r = subprocess.run(["gcc", "-O1", "-c", os.path.join(shim, "blas_lp64.c"), "-o", bo],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    out = str(tmp_path / "test-mult")
    cmd = (["g++", "-fopenmp", "-o", out] + objs + [bo, blas[0], "-Wl,-rpath," + npl, "-L" + libdir, "-lcaps_gb300",
                                                    "-Wl,-rpath," + libdir])
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    syms = subprocess.run(["nm", out], stdout=subprocess.PIPE, text=True).stdout
    assert " U _Z4multPdS_S_iiid" in syms  # left to the shared library


def test_hybrid_step_workspace_between_d_and_b(caps):
    """An 'h' step with factor k (desc.nproc_summa) holds the workspace of k
    concurrent subproducts: more than 'd', less than 'b'; k = 1 runs as 'd'."""
    n = 16384

    def ws(pat, k=1):
        return caps.workspace_size(caps.MatDescriptor.make(n, len(pat), 1, k), pat, form="plain")

    assert ws("hhh", 1) == ws("ddd")
    sizes = [ws("ddd")] + [ws("hhh", k) for k in (2, 3, 4, 5, 6)] + [ws("bbb")]
    assert sizes == sorted(sizes) and len(set(sizes)) == len(sizes), sizes


def test_hybrid_factor_outside_reference_range_rejected(caps):
    for k in (0, 7):
        with pytest.raises(caps.CapsError) as e:
            caps.workspace_size(caps.MatDescriptor.make(1024, 2, 1, k), "hh")
        assert e.value.status == 7  # CAPS_ERR_UNSUPPORTED


def test_chol_mult_validation_before_any_device_work(caps):
    """The Cholesky mult() entry point rejects bad arguments before it touches
    the device: x > 1 (more than one rank), n not divisible by 2^r, a bad
    pattern char, NULL pointers."""
    L = caps.lib()
    p = ctypes.c_void_p(4096)  # never dereferenced: every call below fails its checks first
    opt = caps.options("plain")
    call = lambda C, A, B, n, x, r, pat=None: L.caps_chol_mult_dev(C, A, B, n, x, r, 1.0, pat, ctypes.byref(opt), None)
    assert call(p, p, p, 64, 2, 1) == 7
    assert call(p, p, p, 54, 1, 2) == 2
    assert call(p, p, p, 0, 1, 0) == 2
    assert call(p, p, p, 64, 1, 2, b"dx") == 1
    assert call(None, p, p, 64, 1, 2) == 8
    # the host entry point checks its pointers and size before any copy
    dp = ctypes.POINTER(ctypes.c_double)
    assert L.caps_chol_mult_host(None, None, None, 64, 1, 2, 1.0, None, ctypes.byref(opt)) == 8
    buf = (ctypes.c_double * 4)()
    hp = ctypes.cast(buf, dp)
    assert L.caps_chol_mult_host(hp, hp, hp, 0, 1, 0, 1.0, None, ctypes.byref(opt)) == 2


def test_struct_layouts_match_header(caps, tmp_path):
    """caps_options and caps_tune_info as a C compiler lays them out equal the
    ctypes mirrors (sizes and every field offset)."""
    structs = {"caps_options": caps.Options, "caps_tune_info": caps.TuneInfo}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "caps_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True, check=True).stdout.split("\n")
    got = {(a, b): int(c) for a, b, c in (ln.split() for ln in out if ln)}
    for cname, py in structs.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)


def test_tile_and_operand_bits_validated(caps):
    L = caps.lib()
    d = caps.MatDescriptor.make(512, 1)
    out = ctypes.c_longlong()
    for kw, status in (({"tile": 2}, 0), ({"tile": "32x32"}, 0), ({"tile": 3}, 8), ({"tile": -1}, 8),
                       ({"operand_bits": 48}, 0), ({"operand_bits": 55}, 0), ({"operand_bits": 56}, 8),
                       ({"operand_bits": -1}, 0), ({"operand_bits": -2}, 8)):
        opt = caps.options("split", **kw)
        assert L.caps_workspace_size(d, b"b", ctypes.byref(opt), ctypes.byref(out)) == status, kw
    # -1 (CAPS_OPERAND_BITS_TUNED) is the library's choice: accepted; sizing a
    # workspace tunes nothing, so the tuner's table stays empty
    assert caps.autotune_table() == []
    assert L.caps_autotune_info(0, None) == 8


def test_rect_mm_validation_before_any_device_work(caps):
    """rectMM on one rank: a BFS step (which the reference cannot take on one
    rank), an unknown step, and divisions that do not divide are refused
    before anything runs."""
    import ctypes as C
    L = caps.lib()
    z = C.c_void_p(256)

    def call(m, n, k, r, patt, div):
        d = (C.c_int * max(1, len(div)))(*div)
        return L.caps_rect_mm_dev(z, z, z, m, n, k, r, patt, d if div else None, None)

    assert call(64, 48, 32, 1, b"b", [2, 2, 1]) == 7
    assert "BFS" in L.caps_last_cuda_error().decode()
    assert call(64, 48, 32, 1, b"x", [2, 2, 1]) == 1
    assert call(64, 48, 32, 2, b"dB", [2, 2, 1, 1, 1, 1]) == 7
    assert call(64, 48, 32, 1, b"d", [3, 2, 1]) == 2   # 64 % 3
    assert call(64, 48, 32, 1, b"d", [2, 0, 1]) == 2
    assert call(0, 48, 32, 0, b"", []) == 2
    assert call(64, 48, 32, 1, b"d", []) == 8          # no division triples


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "rect-class", "bench-rect.cpp")),
                    reason="reference sources absent")
def test_rect_bench_links_against_library(caps, tmp_path):
    """The rectangular subproject's own bench-rect.cpp, with its
    communication / library / sizes objects but without rectmm.o, links
    against libcaps_gb300.so: its rectMM() call resolves to the library's."""
    shim = os.path.join(ROOT, "oracle", "ref_shim")
    ref = os.path.join(REF, "rect-class")
    libdir = os.path.dirname(caps.LIB_PATH)
    objs = []
    for src in ("bench-rect", "communication", "library", "rectsizes", "sizes"):
        o = str(tmp_path / (src + ".o"))
        cmd = ["g++", "-O1", "-w", "-fopenmp", "-DNUM_THREADS=1", "-include", os.path.join(shim, "mpi.h"),
               "-I" + shim, "-I" + ref, "-c", os.path.join(ref, src + ".cpp"), "-o", o]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert r.returncode == 0, r.stdout
        objs.append(o)
    out = str(tmp_path / "bench-rect")
    cmd = ["g++", "-fopenmp", "-o", out] + objs + ["-L" + libdir, "-lcaps_gb300", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    syms = subprocess.run(["nm", out], stdout=subprocess.PIPE, text=True).stdout
    assert " U _Z6rectMMPdS_S_iiiiiPcPi" in syms  # left to the shared library


def test_autotune_cache_lines_checked_one_by_one(caps):
    """The on-disk autotune cache's reader (host only): a line applies only to
    its own version, device, size and options; a damaged line is skipped on
    its own, whatever it holds."""
    dev = "NVIDIA_GB300/152"

    def line(*f):
        return "\t".join(str(x) for x in f) + "\n"

    # version, device, n, form, slices, scheme asked, nrec, pattern, scheme chosen, tile, bits, rejected, s
    split1792 = line("caps-tune-4", dev, 1792, 1, 0, 0, 0, "-", 2, 0, 55, 2, 0.0104)
    t = caps.debug_tune_cache_line(split1792, dev, 1792, "split")
    assert t == {"n": 1792, "form": "split", "nrec": 0, "pattern": "", "scheme": "residues", "tile": [128, 256],
                 "operand_bits": 55, "moduli": 17, "gate_rejected": 2, "leaf_gate": False, "from_cache": True,
                 "seconds_per_instance": 0.0104}
    t = caps.debug_tune_cache_line(line("caps-tune-4", dev, 3584, 1, 0, 0, 1, "b", 2, 0, 52, 1, 0.7), dev, 3584,
                                   "split")
    assert (t["pattern"], t["operand_bits"], t["moduli"]) == ("b", 52, 16)
    t = caps.debug_tune_cache_line(line("caps-tune-4", dev, 448, 1, 0, 0, 0, "-", 1, 0, 0, 0, 1e-3), dev, 448,
                                   "split")
    assert (t["scheme"], t["tile"], t["moduli"]) == ("digits", [128, 64], 0)
    t = caps.debug_tune_cache_line(line("caps-tune-4", dev, 1792, 0, 0, 0, 2, "bb", 0, 2, 0, 0, 0.4), dev, 1792,
                                   "plain")
    assert (t["form"], t["pattern"], t["scheme"], t["tile"]) == ("plain", "bb", None, [128, 64])
    # a single multiply's leaf-gate choice is kept under the scheme asked for plus 8
    t = caps.debug_tune_cache_line(line("caps-tune-4", dev, 2048, 1, 0, 10, 0, "-", 2, 0, 55, 2, 0.01), dev, 2048,
                                   "split", scheme=10)
    assert t["leaf_gate"] and t["moduli"] == 17
    # another version, device, size, form or scheme asked: not this choice
    assert caps.debug_tune_cache_line(split1792.replace("caps-tune-4", "caps-tune-3"), dev, 1792, "split") is None
    assert caps.debug_tune_cache_line(split1792, "NVIDIA_B200/148", 1792, "split") is None
    assert caps.debug_tune_cache_line(split1792, dev, 896, "split") is None
    assert caps.debug_tune_cache_line(split1792, dev, 1792, "plain") is None
    assert caps.debug_tune_cache_line(split1792, dev, 1792, "split", scheme="residues") is None
    # damaged lines
    for bad in [line("caps-tune-4", dev, 1792, 1, 0, 0, 2, "b", 2, 0, 55, 0, 0.1),     # pattern shorter than nrec
                line("caps-tune-4", dev, 1792, 1, 0, 0, 1, "x", 2, 0, 55, 0, 0.1),     # not a b/d step
                line("caps-tune-4", dev, 1792, 1, 0, 0, 0, "b", 2, 0, 55, 0, 0.1),     # steps at depth 0
                line("caps-tune-4", dev, 1792, 1, 0, 0, 4, "bbbb", 2, 0, 55, 0, 0.1),  # deeper than the tuner goes
                line("caps-tune-4", dev, 1792, 1, 0, 0, 0, "-", 2, 3, 55, 0, 0.1),     # no such tile
                line("caps-tune-4", dev, 1792, 1, 0, 0, 0, "-", 2, 0, 56, 0, 0.1),     # bits above 55
                line("caps-tune-4", dev, 1792, 1, 0, 0, 0, "-", 3, 0, 55, 0, 0.1),     # no such scheme
                line("caps-tune-4", dev, 1792, 1, 0, 0, 0, "-", 2, 0, 55, 0),          # a field missing
                ""]:
        assert caps.debug_tune_cache_line(bad, dev, 1792, "split") is None, bad
