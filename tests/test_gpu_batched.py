"""GPU tests of the batched uneven-size path: grouping, autotuned depth,
CUDA-graph replay, both forms."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(cuda, sizes, seed, integer):
    import torch
    rng = np.random.default_rng(seed)
    As, Bs, Cs, host = [], [], [], []
    for n in sizes:
        if integer:
            A = rng.integers(-64, 65, (n, n)).astype(np.float64)
            B = rng.integers(-64, 65, (n, n)).astype(np.float64)
        else:
            A = rng.uniform(-1, 1, (n, n))
            B = rng.uniform(-1, 1, (n, n))
        host.append((A, B))
        As.append(torch.from_numpy(A.T.copy().reshape(-1)).to(cuda))
        Bs.append(torch.from_numpy(B.T.copy().reshape(-1)).to(cuda))
        Cs.append(torch.full((n * n,), float("nan"), dtype=torch.float64, device=cuda))
    return As, Bs, Cs, host


@pytest.mark.parametrize("form", ["split", "plain"])
def test_batched_uneven_integers_exact_and_replay(caps, cuda, form):
    import torch
    sizes = [448, 896, 448, 224, 896, 448]
    As, Bs, Cs, host = _batch(cuda, sizes, 4, True)
    for rep in range(2):  # second call replays the captured graph
        for c in Cs:
            c.fill_(float("nan"))
        caps.multiply_batched(As, Bs, Cs, sizes, form=form)
        torch.cuda.synchronize()
        for (A, B), C, n in zip(host, Cs, sizes):
            got = C.cpu().numpy().reshape(n, n).T
            assert np.array_equal(got, (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)), (form, n, rep)
    tab = caps.autotune_table()
    assert {t["n"] for t in tab if t["form"] == form} >= {224, 448, 896}


def test_batched_float_error(caps, cuda, oracle_mod):
    import torch
    from helpers import dd_of, rel_err
    sizes = [896, 448]
    As, Bs, Cs, host = _batch(cuda, sizes, 5, False)
    for form in ("split", "plain"):
        caps.multiply_batched(As, Bs, Cs, sizes, form=form)
        torch.cuda.synchronize()
        for (A, B), C, n in zip(host, Cs, sizes):
            got = C.cpu().numpy().reshape(n, n).T
            hi, lo = dd_of(oracle_mod, A, B)
            ew, nw = rel_err(got, hi, lo, A, B)
            assert nw < 1e-14 and ew < 1e-13, (form, n, ew, nw)


def test_batched_argument_errors(caps, cuda):
    import torch
    t = torch.zeros(16, dtype=torch.float64, device=cuda)
    with pytest.raises(caps.CapsError) as e:
        caps.multiply_batched([t], [t], [t], [0])
    assert e.value.status == 2


def test_autotune_choices_persist_on_disk(caps, cuda, tmp_path):
    """Two fresh processes with the same CAPS_AUTOTUNE_CACHE file: the first
    times the candidates and writes its choices, the second reads them back
    (from_cache) and makes the same ones; both give exact integer products."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cache = tmp_path / "autotune.tsv"
    code = (
        "import sys, json, numpy as np, torch; sys.path.insert(0, %r); import caps_gb300 as cg; "
        "sizes = [448, 224]; rng = np.random.default_rng(3); ok = True; As = []; Bs = []; Cs = []; ref = []\n"
        "for n in sizes:\n"
        "    A = rng.integers(-9, 10, (n, n)).astype(np.float64); B = rng.integers(-9, 10, (n, n)).astype(np.float64)\n"
        "    As.append(torch.from_numpy(A.T.copy().reshape(-1)).cuda()); Bs.append(torch.from_numpy(B.T.copy().reshape(-1)).cuda())\n"
        "    Cs.append(torch.empty(n * n, dtype=torch.float64, device='cuda')); ref.append(A.astype(np.int64) @ B.astype(np.int64))\n"
        "cg.multiply_batched(As, Bs, Cs, sizes, form='split'); torch.cuda.synchronize()\n"
        "for C, R, n in zip(Cs, ref, sizes): ok = ok and np.array_equal(C.cpu().numpy().reshape(n, n).T, R.astype(np.float64))\n"
        "print(json.dumps({'ok': bool(ok), 'tab': cg.autotune_table()}))\n" % root)
    env = dict(os.environ, CAPS_AUTOTUNE_CACHE=str(cache))
    runs = []
    for _ in range(2):
        out = subprocess.run([sys.executable, "-c", code], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                             text=True, timeout=600, env=env)
        assert out.returncode == 0, out.stdout
        runs.append(json.loads(out.stdout.strip().splitlines()[-1]))
    assert runs[0]["ok"] and runs[1]["ok"]
    assert cache.exists() and len(cache.read_text().strip().splitlines()) >= 2
    first = {t["n"]: t for t in runs[0]["tab"]}
    second = {t["n"]: t for t in runs[1]["tab"]}
    assert set(first) == set(second) == {448, 224}
    for n in first:
        assert not first[n]["from_cache"] and second[n]["from_cache"]
        for k in ("nrec", "pattern", "scheme", "tile", "operand_bits", "moduli"):
            assert first[n][k] == second[n][k], (n, k)


def _sampled_errors(oracle_mod, C_cm, A_cm, B_cm, n, seed):
    rng = np.random.default_rng(seed)
    rows, cols = rng.integers(0, n, 256), rng.integers(0, n, 256)
    hi, lo = oracle_mod.dd_entries(A_cm, B_cm, n, rows, cols)
    ab = oracle_mod.absprod_entries(A_cm, B_cm, n, rows, cols)
    m = oracle_mod.error_metrics(C_cm.reshape(n, n)[cols, rows], hi, lo, ab)
    return m["max_elementwise_rel"], m["normwise_rel"]


def test_autotuner_axes_and_split_no_worse_than_plain(caps, cuda, oracle_mod):
    """The tuner's table carries every axis (depth, pattern, scheme, tile,
    operand bits / moduli); whatever it chose for the split form, each
    batched split product is compared with the plain FP64 product at the same
    depth and pattern (the same Strassen sums, FP64 DMMA leaves; the plain
    batched form picks its own depth): no less accurate normwise, and per
    entry on uniform inputs and on wide-range inputs from K = 1024 on; at a
    shorter K on wide-range inputs, per entry within 16x (the bit cap's
    accuracy gate keeps a cap only if it adds nothing to these)."""
    import torch
    sizes = [1792, 448, 1792]
    rng = np.random.default_rng(21)
    for wide in (False, True):
        As, Bs, host = [], [], []
        for n in sizes:
            A = rng.uniform(-1, 1, n * n)
            B = rng.uniform(-1, 1, n * n)
            if wide:
                A *= 2.0 ** rng.integers(-20, 21, n * n)
                B *= 2.0 ** rng.integers(-20, 21, n * n)
            host.append((A, B))
            As.append(torch.from_numpy(A).to(cuda))
            Bs.append(torch.from_numpy(B).to(cuda))
        Cs = [torch.full((n * n,), float("nan"), dtype=torch.float64, device=cuda) for n in sizes]
        caps.multiply_batched(As, Bs, Cs, sizes, form="split")
        torch.cuda.synchronize()
        tab = {(t["n"], t["form"]): t for t in caps.autotune_table()}
        for i, ((A, B), C, n) in enumerate(zip(host, Cs, sizes)):
            ew_s, nw_s = _sampled_errors(oracle_mod, C.cpu().numpy(), A, B, n, 5 + i)
            s = tab[(n, "split")]
            r, pat = s["nrec"], s["pattern"] or None
            # the plain form at the split's depth and pattern (CAPS layout in between)
            d = caps.MatDescriptor.make(n, r)
            a, b = torch.empty_like(As[i]), torch.empty_like(Bs[i])
            caps.to_caps_layout(As[i], a, d)
            caps.to_caps_layout(Bs[i], b, d)
            c = torch.full_like(a, float("nan"))
            caps.multiply(a, b, c, d, pat, form="plain")
            cp = torch.empty_like(c)
            caps.from_caps_layout(c, cp, d)
            torch.cuda.synchronize()
            ew_p, nw_p = _sampled_errors(oracle_mod, cp.cpu().numpy(), A, B, n, 5 + i)
            # The split form rounds each entry to 55 bits of its row's (column's)
            # largest: on entries spread over 2^+-20 at a short inner dimension that
            # rounding exceeds the classical FP64 error per entry, while normwise it
            # stays below (the measured 448 leaf: 1.5e-14 against 1.3e-15 per entry,
            # 6.5e-16 normwise for both).  From K = 1024 on the FP64 rounding grows
            # past it on both measures, as at the headline's leaves of 2048.
            leaf = n >> r
            assert nw_s <= nw_p, (wide, n, s, nw_s, nw_p)
            if not wide or leaf >= 1024:
                assert ew_s <= ew_p, (wide, n, s, ew_s, ew_p)
            else:
                assert ew_s <= 16 * ew_p, (wide, n, s, ew_s, ew_p)
    caps.multiply_batched(As, Bs, Cs, sizes, form="plain")  # the plain form's choices too
    torch.cuda.synchronize()
    tab = {(t["n"], t["form"]): t for t in caps.autotune_table()}
    for n in (448, 1792):
        p = tab[(n, "plain")]
        assert p["tile"] in ([64, 64], [32, 32], [128, 64]) and p["operand_bits"] == 0 and p["scheme"] is None
        s = tab[(n, "split")]
        if s["scheme"] == "residues" and (n >> s["nrec"]) <= 2048:
            assert s["tile"] == [128, 256] and s["operand_bits"] in (55, 52, 48)
            assert s["moduli"] == {55: 17, 52: 16, 48: 15}[s["operand_bits"]]  # K of 448..2048
        else:
            assert s["tile"] == [128, 64] and s["operand_bits"] == 0 and s["moduli"] == 0
