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
    operand bits / moduli); whatever it chose, the batched split products are
    no less accurate than the batched plain FP64 ones, on uniform and on
    wide-range inputs (the promise its accuracy gate on the bit cap keeps)."""
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
        err = {}
        for form in ("split", "plain"):
            Cs = [torch.full((n * n,), float("nan"), dtype=torch.float64, device=cuda) for n in sizes]
            caps.multiply_batched(As, Bs, Cs, sizes, form=form)
            torch.cuda.synchronize()
            err[form] = [_sampled_errors(oracle_mod, C.cpu().numpy(), A, B, n, 5 + i)
                         for i, ((A, B), C, n) in enumerate(zip(host, Cs, sizes))]
        for (ew_s, nw_s), (ew_p, nw_p), n in zip(err["split"], err["plain"], sizes):
            assert ew_s <= ew_p and nw_s <= nw_p, (wide, n, ew_s, ew_p, nw_s, nw_p)
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
