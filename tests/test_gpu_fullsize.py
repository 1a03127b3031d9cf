"""Parity at the workloads' full sizes, through the C ABI (about a minute of GPU time).

The smaller tests pin every path bit for bit against the oracle.  Here the
multiplies run at the sizes the benchmark quotes and are checked by
properties that do not need a full classical product:
  - n = 8192, r = 3, 'ddd', FP64 (plain) form on uniform[-1,1) inputs: error
    against the double-double classical product on 1024 sampled entries,
    within 4x of the oracle's own CPU Strassen of the same inputs (the
    reference's arithmetic, multiply.cpp:409-454, with OpenBLAS leaves);
  - n = 16384, r = 3, split and plain forms, on uniform[-1,1) inputs and on
    wide-range inputs u 2^k (k uniform in [-20, 20]): the split form's error
    is no worse than the plain form's, elementwise and normwise, over 1024
    sampled entries, with 55-bit operands and with the library's
    accuracy-gated operand bits;
  - n = 32768, r = 4, 'bbdd' under a 120 GB workspace budget (-m 120000),
    integers in [-1024, 1024]: 256 sampled entries of both forms equal the
    exact int64 dot products (fromfile1.cpp:124-145 checks its known answers
    the same way, entry by entry).
Error = |C - C_ref| / (|A||B|) per entry (max), and ||C - C_ref|| / ||C_ref||
over the sampled entries."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _uniform(n, seed, cuda, wide=False):
    import torch
    g = torch.Generator(device=cuda)
    g.manual_seed(seed)
    x = torch.rand(n * n, dtype=torch.float64, device=cuda, generator=g) * 2 - 1
    if wide:
        x *= torch.exp2(torch.randint(-20, 21, (n * n,), device=cuda, generator=g).to(torch.float64))
    return x


def _colmajor_host(caps, x, desc):
    import torch
    y = torch.empty_like(x)
    caps.from_caps_layout(x, y, desc)
    torch.cuda.synchronize()
    return y.cpu().numpy()


def _sampled_error(oracle_mod, C_cm, A_cm, B_cm, n, samples, seed):
    rng = np.random.default_rng(seed)
    rows, cols = rng.integers(0, n, samples), rng.integers(0, n, samples)
    hi, lo = oracle_mod.dd_entries(A_cm, B_cm, n, rows, cols)
    ab = oracle_mod.absprod_entries(A_cm, B_cm, n, rows, cols)
    C = C_cm.reshape(n, n)[cols, rows]  # column-major: C[i, j] at j * n + i
    m = oracle_mod.error_metrics(C, hi, lo, ab)
    return m["max_elementwise_rel"], m["normwise_rel"]


def test_fullsize_plain_n8192_ddd_error_with_cpu_strassen(caps, oracle_mod, cuda):
    import torch
    n, r, pat = 8192, 3, "ddd"
    d = caps.MatDescriptor.make(n, r)
    A, B = _uniform(n, 2, cuda), _uniform(n, 22, cuda)
    C = torch.empty_like(A)
    caps.multiply(A, B, C, d, pat, form="plain")
    torch.cuda.synchronize()
    A_cm, B_cm, C_cm = (_colmajor_host(caps, x, d) for x in (A, B, C))
    ew, nw = _sampled_error(oracle_mod, C_cm, A_cm, B_cm, n, 1024, 8)
    # the oracle's CPU Strassen of the same inputs (CAPS layout in and out)
    oracle_mod.use_blas(True)
    try:
        Co = oracle_mod.multiply(A.cpu().numpy(), B.cpu().numpy(), n, r, 1, pat)
    finally:
        oracle_mod.use_blas(False)
    del A, B, C
    Co_cm = oracle_mod.from_caps(Co, n, r)
    ew_o, nw_o = _sampled_error(oracle_mod, Co_cm, A_cm, B_cm, n, 1024, 8)
    assert ew <= 4 * ew_o and nw <= 4 * nw_o, (ew, ew_o, nw, nw_o)
    assert ew < 1e-14


@pytest.mark.parametrize("bits", [0, -1])
@pytest.mark.parametrize("wide", [False, True])
def test_fullsize_split_n16384_error_no_worse_than_plain(caps, oracle_mod, cuda, wide, bits):
    """bits 0: 55-bit operands (17 moduli); -1: the library's accuracy-gated
    choice for leaves of 2048, as the benchmark runs it."""
    import torch
    n, r = 16384, 3
    d = caps.MatDescriptor.make(n, r)
    A, B = _uniform(n, 3 + 10 * wide, cuda, wide), _uniform(n, 4 + 10 * wide, cuda, wide)
    C = torch.empty_like(A)
    A_cm, B_cm = _colmajor_host(caps, A, d), _colmajor_host(caps, B, d)
    err = {}
    for form in ("split", "plain"):
        caps.multiply(A, B, C, d, None, form=form, operand_bits=bits)
        torch.cuda.synchronize()
        if form == "split":
            assert caps.counters()["split_moduli"] == 17 if bits == 0 else caps.counters()["split_moduli"] in (15, 16, 17)
        err[form] = _sampled_error(oracle_mod, _colmajor_host(caps, C, d), A_cm, B_cm, n, 1024, 9)
    del A, B, C
    caps.release_cache()
    (ew_s, nw_s), (ew_p, nw_p) = err["split"], err["plain"]
    assert ew_s <= ew_p and nw_s <= nw_p, err


def test_fullsize_config5_n32768_bbdd_integers_exact(caps, cuda):
    import torch
    n, r, pat = 32768, 4, "bbdd"
    budget = 120000 * 2 ** 20
    d = caps.MatDescriptor.make(n, r)
    g = torch.Generator(device=cuda)
    g.manual_seed(9)
    A = torch.randint(-1024, 1025, (n * n,), dtype=torch.int32, device=cuda, generator=g).to(torch.float64)
    B = torch.randint(-1024, 1025, (n * n,), dtype=torch.int32, device=cuda, generator=g).to(torch.float64)
    C = torch.empty_like(A)
    Ac, Bc, Cc = torch.empty_like(A), torch.empty_like(B), torch.empty_like(A)
    caps.from_caps_layout(A, Ac, d)
    caps.from_caps_layout(B, Bc, d)
    rng = np.random.default_rng(1)
    rows = torch.from_numpy(rng.integers(0, n, 256)).to(cuda)
    cols = torch.from_numpy(rng.integers(0, n, 256)).to(cuda)
    Am, Bm = Ac.view(n, n), Bc.view(n, n)  # [column][row]
    exact = ((Am[:, rows].T.to(torch.int64)) * Bm[cols].to(torch.int64)).sum(dim=1)
    for form in ("split", "plain"):
        C.fill_(float("nan"))
        caps.multiply(A, B, C, d, pat, form=form, workspace_limit=budget)
        caps.from_caps_layout(C, Cc, d)
        torch.cuda.synchronize()
        got = Cc.view(n, n)[cols, rows]
        assert torch.equal(got, exact.to(torch.float64)), form
    del A, B, C, Ac, Bc, Cc
    caps.release_cache()
    torch.cuda.empty_cache()
