"""GPU parity of the split (Ozaki-style, tcgen05) form, through the C ABI.

Digit scheme: the leaf kernel computes exact integer digit-pair products, so
for the same digit count s and diagonal count nd it must equal the oracle's
CPU model of the split arithmetic BIT FOR BIT.  Residue scheme: the leaf
product of the scaled integers is exact, so it must equal the oracle's
128-bit model bit for bit.  Whole multiplies are bit-exact on integer inputs
and, on float inputs, within the plain FP64 path's error."""
import numpy as np
import pytest

from helpers import caps_of, mat_of, gpu_multiply, dd_of, rel_err

pytestmark = pytest.mark.gpu


def _leaf(caps, cuda, A, B, s=0, nd=0, scheme="auto", operand_bits=0):
    import torch
    m = A.shape[0]
    C = torch.full((m * m,), float("nan"), dtype=torch.float64, device=cuda)
    caps.leaf_gemm(torch.from_numpy(A.T.copy().reshape(-1)).to(cuda),
                   torch.from_numpy(B.T.copy().reshape(-1)).to(cuda), C, m, form="split", slices=s, diagonals=nd,
                   scheme=scheme, operand_bits=operand_bits)
    torch.cuda.synchronize()
    return C.cpu().numpy().reshape(m, m).T, caps.counters()


@pytest.mark.parametrize("m", [128, 64, 14, 200, 512, 1100])
def test_split_leaf_bitexact_vs_model_uniform(caps, oracle_mod, cuda, m):
    rng = np.random.default_rng(m)
    A = rng.uniform(-1, 1, (m, m))
    B = rng.uniform(-1, 1, (m, m))
    C, cnt = _leaf(caps, cuda, A, B, scheme="digits")
    s, nd = cnt["split_slices"], cnt["split_diagonals"]
    assert (s, nd, cnt["split_moduli"]) == (8, 8, 0)
    ref = oracle_mod.split_gemm(A.T.copy().reshape(-1), B.T.copy().reshape(-1), m, s, nd).reshape(m, m).T
    assert np.array_equal(C, ref)


@pytest.mark.parametrize("s,nd", [(7, 7), (6, 8), (3, 5), (8, 6), (1, 1)])
def test_split_leaf_bitexact_forced_digits(caps, oracle_mod, cuda, s, nd):
    m = 192
    rng = np.random.default_rng(s * 10 + nd)
    A = rng.uniform(-1, 1, (m, m)) * 2.0 ** rng.integers(-20, 21, (m, m))
    B = rng.uniform(-1, 1, (m, m))
    C, cnt = _leaf(caps, cuda, A, B, s, nd)
    assert (cnt["split_slices"], cnt["split_diagonals"]) == (s, nd)
    ref = oracle_mod.split_gemm(A.T.copy().reshape(-1), B.T.copy().reshape(-1), m, s, nd).reshape(m, m).T
    assert np.array_equal(C, ref)


@pytest.mark.parametrize("scheme", ["auto", "digits"])
@pytest.mark.parametrize("m,lim", [(256, 1024), (640, 9), (2048, 1024)])
def test_split_leaf_integers_exact(caps, oracle_mod, cuda, m, lim, scheme):
    rng = np.random.default_rng(m)
    A = rng.integers(-lim, lim + 1, (m, m)).astype(np.float64)
    B = rng.integers(-lim, lim + 1, (m, m)).astype(np.float64)
    C, cnt = _leaf(caps, cuda, A, B, scheme=scheme)
    if scheme == "digits":
        assert 0 < cnt["split_slices"] <= 4
    else:
        assert 0 < cnt["split_moduli"] <= 8
    assert np.array_equal(C, (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64))


def test_split_leaf_zero_rows_and_tiny_values(caps, oracle_mod, cuda):
    m = 130
    rng = np.random.default_rng(9)
    A = rng.uniform(-1, 1, (m, m))
    A[3, :] = 0.0
    A[:, 5] = 0.0
    A[7, 11] = 1e-300
    B = rng.uniform(-1, 1, (m, m)) * 1e-200
    B[:, 2] = 0.0
    C, cnt = _leaf(caps, cuda, A, B, scheme="digits")
    ref = oracle_mod.split_gemm(A.T.copy().reshape(-1), B.T.copy().reshape(-1), m, cnt["split_slices"],
                                cnt["split_diagonals"]).reshape(m, m).T
    assert np.array_equal(C, ref)
    assert np.all(C[3, :] == 0) and np.all(C[:, 2] == 0)


@pytest.mark.parametrize("n", [28, 56, 196, 392])
def test_reference_known_answers_split(caps, oracle_mod, ref_tests, cuda, n):
    A = ref_tests["A%d" % n].astype(np.float64)
    B = ref_tests["B%d" % n].astype(np.float64)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    for bs, r in ref_tests["params%d" % n]:
        for pat in ("d" * r, "b" * r):
            for scheme in ("digits", "residues"):
                C = gpu_multiply(caps, oracle_mod, A, B, r, bs, pat, form="split", scheme=scheme)
                assert np.array_equal(C, exact), (n, bs, r, pat, scheme)


def test_config5_like_integers_bitexact(caps, oracle_mod, cuda):
    """Integers in [-1024, 1024], 'bbdd' (scaled down from n = 32768)."""
    n, r = 2048, 4
    rng = np.random.default_rng(5)
    A = rng.integers(-1024, 1025, (n, n)).astype(np.float64)
    B = rng.integers(-1024, 1025, (n, n)).astype(np.float64)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    for form, scheme in (("split", "auto"), ("split", "residues"), ("plain", "auto")):
        C = gpu_multiply(caps, oracle_mod, A, B, r, 1, "bbdd", form=form, scheme=scheme)
        assert np.array_equal(C, exact), (form, scheme)


@pytest.mark.parametrize("scheme", ["digits", "residues"])
@pytest.mark.parametrize("wide", [False, True])
def test_split_error_no_worse_than_plain(caps, oracle_mod, cuda, wide, scheme):
    n, r = 1024, 3
    rng = np.random.default_rng(33 + wide)
    A = rng.uniform(-1, 1, (n, n))
    B = rng.uniform(-1, 1, (n, n))
    if wide:
        A *= 2.0 ** rng.integers(-20, 21, (n, n))
        B *= 2.0 ** rng.integers(-20, 21, (n, n))
    hi, lo = dd_of(oracle_mod, A, B)
    Cp = gpu_multiply(caps, oracle_mod, A, B, r, 1, "ddb", form="plain")
    Cs = gpu_multiply(caps, oracle_mod, A, B, r, 1, "ddb", form="split", scheme=scheme)
    ew_p, nw_p = rel_err(Cp, hi, lo, A, B)
    ew_s, nw_s = rel_err(Cs, hi, lo, A, B)
    assert nw_s <= 1.25 * nw_p, (nw_s, nw_p)
    assert ew_s <= 1.25 * ew_p or ew_s < 1e-13, (ew_s, ew_p)


# ---------------------------------------------------------------- residue scheme
MODULI = [181, 180, 179, 173, 169, 167, 163, 161, 157, 151, 149, 139, 137, 131, 127, 121, 113]


def expected_moduli(ta, tb, m):
    """Fewest moduli whose product M has floor(log2 M) >= ta + tb + ceil(log2 Kp) + 1."""
    kp = (m + 15) // 16 * 16
    need = ta + tb + (kp - 1).bit_length() + 1
    prod = 1
    for L, p in enumerate(MODULI, 1):
        prod *= p
        if prod.bit_length() - 1 >= need:
            return L
    return None


def _residue_ref(oracle_mod, A, B, bits=55):
    m = A.shape[0]
    ref, t = oracle_mod.split_gemm_residues(A.T.copy().reshape(-1), B.T.copy().reshape(-1), m, bits)
    return ref.reshape(m, m).T, t


@pytest.mark.parametrize("bits", [52, 48, 30])
@pytest.mark.parametrize("m,wide", [(512, False), (200, True), (2048, False)])
def test_residue_leaf_operand_bit_cap_bitexact_vs_model(caps, oracle_mod, cuda, m, wide, bits):
    """A cap on the operand bits (the autotuner's modulus-count axis) takes
    fewer moduli and still equals the oracle's 128-bit model at that cap."""
    rng = np.random.default_rng(7 * m + bits)
    A = rng.uniform(-1, 1, (m, m))
    B = rng.uniform(-1, 1, (m, m))
    if wide:
        A *= 2.0 ** rng.integers(-20, 21, (m, m))
        B *= 2.0 ** rng.integers(-20, 21, (m, m))
    C, cnt = _leaf(caps, cuda, A, B, scheme="residues", operand_bits=bits)
    ref, (ta, tb) = _residue_ref(oracle_mod, A, B, bits)
    assert ta == tb == bits
    assert cnt["split_moduli"] == expected_moduli(bits, bits, m) < expected_moduli(55, 55, m)
    assert np.array_equal(C, ref)
    # integer data needing fewer bits than the cap stay exact
    Ai = rng.integers(-1024, 1025, (m, m)).astype(np.float64)
    Bi = rng.integers(-1024, 1025, (m, m)).astype(np.float64)
    C, _ = _leaf(caps, cuda, Ai, Bi, scheme="residues", operand_bits=bits)
    assert np.array_equal(C, (Ai.astype(np.int64) @ Bi.astype(np.int64)).astype(np.float64))


def test_residue_leaf_tuned_operand_bits(caps, oracle_mod, cuda):
    """operand_bits = -1: the library gates 55 / 52 / 48 bits once for leaves
    of 1024, records the choice (leaf_gate), and the product equals the
    oracle's 128-bit model at the chosen cap; a second call reuses it."""
    m = 1024
    rng = np.random.default_rng(17)
    A = rng.uniform(-1, 1, (m, m))
    B = rng.uniform(-1, 1, (m, m))
    C, cnt = _leaf(caps, cuda, A, B, operand_bits=-1)
    tab = [t for t in caps.autotune_table() if t["leaf_gate"] and t["n"] == m]
    assert len(tab) == 1 and tab[0]["scheme"] == "residues" and tab[0]["operand_bits"] in (55, 52, 48)
    bits = tab[0]["operand_bits"]
    assert cnt["split_moduli"] == expected_moduli(bits, bits, m)
    ref, _ = _residue_ref(oracle_mod, A, B, bits)
    assert np.array_equal(C, ref)
    C2, _ = _leaf(caps, cuda, A, B, operand_bits=-1)
    assert np.array_equal(C2, C)
    assert len([t for t in caps.autotune_table() if t["leaf_gate"] and t["n"] == m]) == 1


@pytest.mark.parametrize("m", [128, 64, 14, 200, 512, 1100, 2048])
def test_residue_leaf_bitexact_vs_model_uniform(caps, oracle_mod, cuda, m):
    rng = np.random.default_rng(100 + m)
    A = rng.uniform(-1, 1, (m, m))
    B = rng.uniform(-1, 1, (m, m))
    C, cnt = _leaf(caps, cuda, A, B, scheme="residues")
    ref, (ta, tb) = _residue_ref(oracle_mod, A, B)
    assert 53 <= ta <= 55 and 53 <= tb <= 55  # numpy's uniform doubles carry 53 bits
    assert cnt["split_moduli"] == expected_moduli(ta, tb, m)
    assert np.array_equal(C, ref)


def test_residue_leaf_wide_range_zero_rows_subnormal_results(caps, oracle_mod, cuda):
    m = 300
    rng = np.random.default_rng(17)
    A = rng.uniform(-1, 1, (m, m)) * 2.0 ** rng.integers(-20, 21, (m, m))
    A[3, :] = 0.0
    A[:, 5] = 0.0
    A[7, 11] = 1e-300
    B = rng.uniform(-1, 1, (m, m)) * 1e-200
    B[:, 2] = 0.0
    B[4, 9] = -3e-310  # subnormal operand
    C, cnt = _leaf(caps, cuda, A, B, scheme="residues")
    ref, t = _residue_ref(oracle_mod, A, B)
    assert cnt["split_moduli"] == expected_moduli(t[0], t[1], m)
    assert np.array_equal(C, ref)
    assert np.all(C[3, :] == 0) and np.all(C[:, 2] == 0)
    # products below the normal range: rounded once at 2^-1074
    A = rng.uniform(-1, 1, (m, m)) * 1e-160
    B = rng.uniform(-1, 1, (m, m)) * 1e-160
    C, cnt = _leaf(caps, cuda, A, B, scheme="residues")
    ref, t = _residue_ref(oracle_mod, A, B)
    assert np.array_equal(C, ref)
    assert np.any((C != 0) & (np.abs(C) < 2.2250738585072014e-308))


@pytest.mark.parametrize("m,lim", [(256, 1024), (640, 9), (2048, 1024), (96, 2 ** 26)])
def test_residue_leaf_integers_exact(caps, oracle_mod, cuda, m, lim):
    rng = np.random.default_rng(m + lim)
    A = rng.integers(-lim, lim + 1, (m, m)).astype(np.float64)
    B = rng.integers(-lim, lim + 1, (m, m)).astype(np.float64)
    C, cnt = _leaf(caps, cuda, A, B, scheme="residues")
    bits = max(int(np.max(np.abs(A))).bit_length(), int(np.max(np.abs(B))).bit_length()) + 1
    assert 0 < cnt["split_moduli"] <= expected_moduli(bits, bits, m)
    if m <= 640:
        ref, t = _residue_ref(oracle_mod, A, B)
        assert cnt["split_moduli"] == expected_moduli(t[0], t[1], m)
        assert np.array_equal(C, ref)
    if m * lim * lim < 2 ** 53:
        exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    else:  # Python integers, each rounded once to double
        ex = A.astype(np.int64).astype(object) @ B.astype(np.int64).astype(object)
        exact = np.array([[float(v) for v in row] for row in ex])
    assert np.array_equal(C, exact)


def test_auto_scheme_choice(caps, oracle_mod, cuda):
    """Residues wherever the leaves fit them (K <= 2048), integer data
    included: float data take 16-17 moduli, 11-bit integers 5; above 2048
    the digits run."""
    m = 512
    rng = np.random.default_rng(3)
    A = rng.uniform(-1, 1, (m, m))
    B = rng.uniform(-1, 1, (m, m))
    C, cnt = _leaf(caps, cuda, A, B)
    assert cnt["split_moduli"] >= 16 and cnt["split_slices"] == 0
    assert np.array_equal(C, _residue_ref(oracle_mod, A, B)[0])
    Ai = rng.integers(-1024, 1025, (m, m)).astype(np.float64)
    Bi = rng.integers(-1024, 1025, (m, m)).astype(np.float64)
    C, cnt = _leaf(caps, cuda, Ai, Bi)
    Cr, t = _residue_ref(oracle_mod, Ai, Bi)
    assert cnt["split_moduli"] == expected_moduli(t[0], t[1], m) <= 5 and cnt["split_slices"] == 0
    assert np.array_equal(C, Cr)
    assert np.array_equal(C, (Ai.astype(np.int64) @ Bi.astype(np.int64)).astype(np.float64))
    m = 2064
    Ai = rng.integers(-1024, 1025, (m, m)).astype(np.float64)
    Bi = rng.integers(-1024, 1025, (m, m)).astype(np.float64)
    C, cnt = _leaf(caps, cuda, Ai, Bi)
    assert cnt["split_moduli"] == 0 and cnt["split_slices"] == 2
    assert np.array_equal(C, (Ai.astype(np.int64) @ Bi.astype(np.int64)).astype(np.float64))


def test_residue_scheme_falls_back_to_digits_above_2048(caps, oracle_mod, cuda):
    m = 2064
    rng = np.random.default_rng(8)
    A = rng.uniform(-1, 1, (m, m))
    B = rng.uniform(-1, 1, (m, m))
    Cr, cnt_r = _leaf(caps, cuda, A, B, scheme="residues")
    Cd, cnt_d = _leaf(caps, cuda, A, B, scheme="digits")
    assert cnt_r["split_moduli"] == 0 and cnt_r["split_slices"] == 8
    assert np.array_equal(Cr, Cd)


@pytest.mark.parametrize("scheme", ["residues", "digits"])
def test_starved_gemm_wait_gives_up_then_next_call_runs(caps, oracle_mod, cuda, scheme):
    """The bounded device waits: a GEMM launch that is given no copies (test
    hook; nothing is in flight, no fault) gives up its waits, frees TMEM and
    returns CAPS_ERR_TIMEOUT; the context stays usable and the next call is
    exact against the oracle's model."""
    import time
    m = 256
    rng = np.random.default_rng(77)
    A = rng.uniform(-1, 1, (m, m))
    B = rng.uniform(-1, 1, (m, m))
    caps.debug_starve_split_gemm(1)
    t0 = time.perf_counter()
    with pytest.raises(caps.CapsError) as e:
        _leaf(caps, cuda, A, B, scheme=scheme)
    waited = time.perf_counter() - t0
    assert e.value.status == 6, e.value
    assert waited < 30.0
    C, cnt = _leaf(caps, cuda, A, B, scheme=scheme)
    if scheme == "residues":
        ref, _ = oracle_mod.split_gemm_residues(A.T.copy().reshape(-1), B.T.copy().reshape(-1), m)
    else:
        ref = oracle_mod.split_gemm(A.T.copy().reshape(-1), B.T.copy().reshape(-1), m, cnt["split_slices"],
                                    cnt["split_diagonals"])
    assert np.array_equal(C, ref.reshape(m, m).T)


def test_first_split_call_of_a_process_runs_residues(caps, cuda):
    """The scheme is chosen on the device from the moduli tables; a fresh
    process's very first split multiply must already see them and pick the
    same moduli count as a second call on the same data, not fall back to
    digits (moduli count 0)."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys, numpy as np, torch; sys.path.insert(0, %r); import caps_gb300 as cg; "
            "m = 256; rng = np.random.default_rng(1); "
            "A = torch.from_numpy(rng.uniform(-1, 1, m * m)).cuda(); B = torch.from_numpy(rng.uniform(-1, 1, m * m)).cuda(); "
            "C = torch.empty_like(A); cg.leaf_gemm(A, B, C, m, form='split'); first = cg.counters()['split_moduli']; "
            "cg.leaf_gemm(A, B, C, m, form='split'); torch.cuda.synchronize(); "
            "print(first, cg.counters()['split_moduli'])" % root)
    out = subprocess.run([sys.executable, "-c", code], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stdout
    first, second = (int(x) for x in out.stdout.strip().splitlines()[-1].split())
    assert first == second > 0, out.stdout


@pytest.mark.parametrize("n,r,pat,ref_pat,wide", [(1024, 2, "dd", "bb", False), (896, 2, "bd", "bb", True),
                                                  (2048, 2, "dd", "bb", True), (512, 1, "d", "b", False)])
def test_split_d_step_bit_identical_to_b(caps, oracle_mod, cuda, n, r, pat, ref_pat, wide):
    """A lean 'd' step over residue-scheme leaves combines its products with
    the reference's FP64 operations in its order (C22 = C12 = C11 + Q4,
    C22 += Q5, the U2 / Q3 triple, C21 -= Q7, C12 += Q6, C11 += Q2), as
    calcCij does for a 'b' step, so the two agree bit for bit on float data,
    wide-range data included."""
    import torch
    rng = np.random.default_rng(7 * n + r)
    A = rng.uniform(-1, 1, (n, n))
    B = rng.uniform(-1, 1, (n, n))
    if wide:
        A *= 2.0 ** rng.integers(-20, 21, (n, n))
        B *= 2.0 ** rng.integers(-20, 21, (n, n))
    dA = torch.from_numpy(caps_of(oracle_mod, A, r)).to(cuda)
    dB = torch.from_numpy(caps_of(oracle_mod, B, r)).to(cuda)
    out = {}
    for p in (pat, ref_pat):
        dC = torch.full_like(dA, float("nan"))
        caps.multiply(dA, dB, dC, caps.MatDescriptor.make(n, r), p, form="split")
        torch.cuda.synchronize()
        assert caps.counters()["split_moduli"] > 0  # the residues ran
        out[p] = dC.cpu().numpy()
    assert np.array_equal(out[pat], out[ref_pat])
