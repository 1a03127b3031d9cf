"""GPU parity of the plain (FP64 DMMA) path and the layout reorder, through
the C ABI, against the oracle and the reference's own fixtures."""
import os

import numpy as np
import pytest

from helpers import caps_of, mat_of, gpu_multiply, dd_of, rel_err

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_layout_reorder_matches_reference_permutation(caps, oracle_mod, cuda):
    import torch
    g = np.load(os.path.join(ROOT, "tests", "golden", "ref_layout.npz"))
    for key in g.files:
        _, n, r, bs = key.split("_")
        n, r, bs = int(n), int(r), int(bs)
        d = caps.MatDescriptor.make(n, r, bs)
        cm = torch.arange(n * n, dtype=torch.float64, device=cuda)
        out = torch.empty_like(cm)
        caps.to_caps_layout(cm, out, d)
        back = torch.empty_like(cm)
        caps.from_caps_layout(out, back, d)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy().astype(np.int32), g[key]), key
        assert torch.equal(back, cm)


@pytest.mark.parametrize("n,r,bs", [(1024, 3, 1), (96, 2, 3), (4096, 2, 16), (112, 4, 1)])
def test_layout_reorder_matches_oracle(caps, oracle_mod, cuda, n, r, bs):
    import torch
    x = np.random.default_rng(n).uniform(-1, 1, n * n)
    d = caps.MatDescriptor.make(n, r, bs)
    t = torch.from_numpy(x).to(cuda)
    out = torch.empty_like(t)
    caps.to_caps_layout(t, out, d)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle_mod.to_caps(x, n, r, bs))


@pytest.mark.parametrize("m", [1, 7, 14, 64, 100, 256, 515])
def test_dmma_leaf_gemm(caps, oracle_mod, cuda, m):
    import torch
    rng = np.random.default_rng(m)
    Ai = rng.integers(-50, 51, (m, m)).astype(np.float64)
    Bi = rng.integers(-50, 51, (m, m)).astype(np.float64)
    C = torch.empty(m * m, dtype=torch.float64, device=cuda)
    caps.leaf_gemm(torch.from_numpy(Ai.T.copy().reshape(-1)).to(cuda),
                   torch.from_numpy(Bi.T.copy().reshape(-1)).to(cuda), C, m)
    torch.cuda.synchronize()
    got = C.cpu().numpy().reshape(m, m).T
    assert np.array_equal(got, (Ai.astype(np.int64) @ Bi.astype(np.int64)).astype(np.float64))
    Af = rng.uniform(-1, 1, (m, m))
    Bf = rng.uniform(-1, 1, (m, m))
    caps.leaf_gemm(torch.from_numpy(Af.T.copy().reshape(-1)).to(cuda),
                   torch.from_numpy(Bf.T.copy().reshape(-1)).to(cuda), C, m)
    torch.cuda.synchronize()
    got = C.cpu().numpy().reshape(m, m).T
    hi, lo = dd_of(oracle_mod, Af, Bf)
    ew, _ = rel_err(got, hi, lo, Af, Bf)
    # classical FP64 dot products: |error| <= m u |A||B| (u = 2^-53)
    assert ew <= m * 2.0 ** -53


@pytest.mark.parametrize("tile", ["32x32", "128x64"])
@pytest.mark.parametrize("m", [1, 20, 33, 100, 130, 515])
def test_dmma_leaf_tiles_bitidentical_to_default(caps, oracle_mod, cuda, m, tile):
    """The three DMMA tile shapes (an autotuner axis) accumulate every entry
    over k in the same order, so on float data they agree bit for bit; on
    integers they equal the exact product."""
    import torch
    rng = np.random.default_rng(3 * m)
    Af = torch.from_numpy(rng.uniform(-1, 1, m * m)).to(cuda)
    Bf = torch.from_numpy(rng.uniform(-1, 1, m * m)).to(cuda)
    C0 = torch.full_like(Af, float("nan"))
    C1 = torch.full_like(Af, float("nan"))
    caps.leaf_gemm(Af, Bf, C0, m)
    caps.leaf_gemm(Af, Bf, C1, m, tile=tile)
    torch.cuda.synchronize()
    assert torch.equal(C0, C1)
    Ai = rng.integers(-50, 51, (m, m)).astype(np.float64)
    Bi = rng.integers(-50, 51, (m, m)).astype(np.float64)
    caps.leaf_gemm(torch.from_numpy(Ai.T.copy().reshape(-1)).to(cuda),
                   torch.from_numpy(Bi.T.copy().reshape(-1)).to(cuda), C1, m, tile=tile)
    torch.cuda.synchronize()
    got = C1.cpu().numpy().reshape(m, m).T
    assert np.array_equal(got, (Ai.astype(np.int64) @ Bi.astype(np.int64)).astype(np.float64))


@pytest.mark.parametrize("tile", ["32x32", "128x64"])
def test_plain_multiply_tiles_on_reference_fixtures(caps, oracle_mod, ref_tests, cuda, tile):
    """Whole plain multiplies with a non-default tile on the reference's
    integer fixtures (n = 196 and 392, 'd' and 'b' steps): deviation 0; and on
    floats bit-identical to the default tile."""
    for n in (196, 392):
        A = ref_tests["A%d" % n].astype(np.float64)
        B = ref_tests["B%d" % n].astype(np.float64)
        exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
        for bs, r in ref_tests["params%d" % n]:
            for pat in ("d" * r, "b" * r):
                C = gpu_multiply(caps, oracle_mod, A, B, r, bs, pat, tile=tile)
                assert np.array_equal(C, exact), (n, bs, r, pat)
    rng = np.random.default_rng(11)
    Af, Bf = rng.uniform(-1, 1, (512, 512)), rng.uniform(-1, 1, (512, 512))
    C0 = gpu_multiply(caps, oracle_mod, Af, Bf, 2, 1, "bd")
    C1 = gpu_multiply(caps, oracle_mod, Af, Bf, 2, 1, "bd", tile=tile)
    assert np.array_equal(C0, C1)


@pytest.mark.parametrize("n", [28, 42, 56, 196, 294, 392])
def test_reference_known_answers_plain(caps, oracle_mod, ref_tests, cuda, n):
    """The reference's integer fixtures, every one-rank (-b, -r), 'd' and 'b' steps: deviation 0."""
    A = ref_tests["A%d" % n].astype(np.float64)
    B = ref_tests["B%d" % n].astype(np.float64)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    for bs, r in ref_tests["params%d" % n]:
        for pat in ("d" * r, "b" * r, ("bd" * r)[:r]):
            C = gpu_multiply(caps, oracle_mod, A, B, r, bs, pat)
            assert np.array_equal(C, exact), (n, bs, r, pat)


def test_config1_n56_dd_integers_bitexact(caps, oracle_mod, cuda):
    rng = np.random.default_rng(1)
    A = rng.integers(-9, 10, (56, 56)).astype(np.float64)
    B = rng.integers(-9, 10, (56, 56)).astype(np.float64)
    C = gpu_multiply(caps, oracle_mod, A, B, 2, 1, "dd")
    assert np.array_equal(C, (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64))


@pytest.mark.parametrize("n,r,pat", [(256, 2, "dd"), (512, 3, "bdb"), (1024, 3, "ddd"), (1024, 2, None)])
def test_plain_float_error_vs_double_double(caps, oracle_mod, cuda, n, r, pat):
    """Plain GPU Strassen against the double-double classical product; its
    error sits with the oracle's own Strassen (same additions, FP64 leaves)."""
    rng = np.random.default_rng(n + r)
    A = rng.uniform(-1, 1, (n, n))
    B = rng.uniform(-1, 1, (n, n))
    C = gpu_multiply(caps, oracle_mod, A, B, r, 1, pat)
    hi, lo = dd_of(oracle_mod, A, B)
    ew, nw = rel_err(C, hi, lo, A, B)
    oracle_mod.use_blas(False)
    Co = mat_of(oracle_mod, oracle_mod.multiply(caps_of(oracle_mod, A, r), caps_of(oracle_mod, B, r), n, r, 1,
                                                pat or "d" * r), n, r)
    ew_o, nw_o = rel_err(Co, hi, lo, A, B)
    # Strassen-Winograd normwise bound grows ~ 12^r n u; stay within 4x of the CPU oracle
    assert nw <= max(4 * nw_o, 1e-15)
    assert ew <= max(4 * ew_o, 1e-14)


def test_plain_wide_range_error(caps, oracle_mod, cuda):
    n, r = 512, 2
    rng = np.random.default_rng(77)
    A = rng.uniform(-1, 1, (n, n)) * 2.0 ** rng.integers(-20, 21, (n, n))
    B = rng.uniform(-1, 1, (n, n)) * 2.0 ** rng.integers(-20, 21, (n, n))
    C = gpu_multiply(caps, oracle_mod, A, B, r, 1, "dd")
    hi, lo = dd_of(oracle_mod, A, B)
    oracle_mod.use_blas(False)
    Co = mat_of(oracle_mod, oracle_mod.multiply(caps_of(oracle_mod, A, r), caps_of(oracle_mod, B, r), n, r, 1, "dd"),
                n, r)
    _, nw = rel_err(C, hi, lo, A, B)
    _, nw_o = rel_err(Co, hi, lo, A, B)
    assert nw <= max(4 * nw_o, 1e-15)


def test_host_entry_point_matches_device(caps, oracle_mod, cuda):
    n, r = 128, 2
    rng = np.random.default_rng(3)
    A = rng.integers(-5, 6, (n, n)).astype(np.float64)
    B = rng.integers(-5, 6, (n, n)).astype(np.float64)
    a, b = caps_of(oracle_mod, A, r), caps_of(oracle_mod, B, r)
    c = np.zeros(n * n)
    caps.multiply(a, b, c, caps.MatDescriptor.make(n, r), "db")
    assert np.array_equal(mat_of(oracle_mod, c, n, r), (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64))


@pytest.mark.parametrize("n,r", [(512, 3), (198, 1)])
@pytest.mark.parametrize("form", ["plain", "split"])
def test_host_entry_default_pattern_overlapped_copies(caps, oracle_mod, cuda, form, n, r):
    """No pattern: the library's choice, a top-level 'd' step with the copies
    overlapping the subproducts (C12 comes back in four parts).  Integer
    inputs, exact; and a second call with other inputs (the copy stream and
    events are reused).  n = 198: quadrants of 99^2, an odd element count,
    so the parts of C12 have uneven lengths."""
    for seed in (11, 12):
        rng = np.random.default_rng(seed)
        A = rng.integers(-100, 101, (n, n)).astype(np.float64)
        B = rng.integers(-100, 101, (n, n)).astype(np.float64)
        a, b = caps_of(oracle_mod, A, r), caps_of(oracle_mod, B, r)
        c = np.full(n * n, np.nan)
        caps.multiply(a, b, c, caps.MatDescriptor.make(n, r), None, form=form)
        assert np.array_equal(mat_of(oracle_mod, c, n, r), (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64))


def test_counters_after_multiply(caps, oracle_mod, cuda):
    n, r = 256, 2
    A = np.ones((n, n))
    gpu_multiply(caps, oracle_mod, A, A, r, 1, "dd")
    c = caps.counters()
    f = caps.flop_counts(n, r)
    assert c["additions"] + c["multiplications"] == f.actual
    assert c["kernel_launches"] > 0


def test_error_paths(caps, oracle_mod, cuda):
    import torch
    n, r = 64, 2
    t = torch.zeros(n * n, dtype=torch.float64, device=cuda)
    d = caps.MatDescriptor.make(n, r)
    with pytest.raises(caps.CapsError) as e:
        caps.multiply(t, t, t.clone(), d, "dz")
    assert e.value.status == 1 and str(e.value) == "Invalid pattern"
    with pytest.raises(caps.CapsError) as e:
        caps.multiply(t, t, t.clone(), caps.MatDescriptor.make(66, 2), "dd")
    assert e.value.status == 2
    with pytest.raises(caps.CapsError) as e:
        caps.multiply(t, t, t.clone(), d, "bb", workspace_limit=1024)
    assert e.value.status == 3
    # host-side fault injection: the workspace allocation fails, the call
    # reports it and the library stays usable afterwards
    caps.release_cache()
    caps.debug_fail_allocations(1)
    with pytest.raises(caps.CapsError) as e:
        caps.multiply(t, t, t.clone(), d, "dd")
    assert e.value.status == 5
    caps.debug_fail_allocations(0)
    out = t.clone()
    caps.multiply(t + 1, t + 1, out, d, "dd")
    torch.cuda.synchronize()
    assert float(out[0]) == n


def test_fromfile1_driver_on_reference_fixtures(caps, ref_tests, cuda, tmp_path):
    """bin/fromfile1 (the reference's flags and output) on the reference fixtures."""
    import subprocess
    exe = os.path.join(os.path.dirname(caps.LIB_PATH), "..", "bin", "fromfile1")
    for n in (28, 56):
        A, B = ref_tests["A%d" % n].astype(np.int64), ref_tests["B%d" % n].astype(np.int64)
        C = A @ B
        fin, fc = tmp_path / ("t%d.in" % n), tmp_path / ("t%d.correct" % n)
        with open(fin, "w") as f:
            f.write("%d\n" % n)
            for M in (A, B):
                for row in M:
                    f.write(" ".join(str(int(v)) for v in row) + "\n")
        with open(fc, "w") as f:
            for row in C:
                f.write(" ".join(str(int(v)) for v in row) + "\n")
        for bs, r in ref_tests["params%d" % n]:
            for form in ("plain", "split"):
                out = subprocess.run([exe, "-i", str(fin), "-b", str(bs), "-r", str(r), "-c", str(fc), "--form", form],
                                     stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
                assert out.returncode == 0, out.stdout
                assert "Maximum deviation 0.000000e+00" in out.stdout, (n, bs, r, form, out.stdout)


def test_randombenchmark_driver(caps, cuda):
    import subprocess
    exe = os.path.join(os.path.dirname(caps.LIB_PATH), "..", "bin", "randombenchmark")
    out = subprocess.run([exe, "-s", "1024", "-r", "2", "-p", "bd"], stdout=subprocess.PIPE,
                         stderr=subprocess.STDOUT, text=True, timeout=300)
    assert out.returncode == 0, out.stdout
    assert "Execution pattern BFS,DFS," in out.stdout
    assert "effective Gflop/s" in out.stdout
    bad = subprocess.run([exe, "-s", "1024", "-r", "2", "-p", "bx"], stdout=subprocess.PIPE,
                         stderr=subprocess.STDOUT, text=True, timeout=300)
    assert bad.returncode != 0 and "Invalid pattern" in bad.stdout


def test_fromfile1_on_generated_fixture(caps, cuda, tmp_path):
    """A 448 fixture from the fixture generator (signed entries, exact product)
    through bin/fromfile1 at every depth the reference's params would list."""
    import importlib.util
    import subprocess
    spec = importlib.util.spec_from_file_location(
        "caps_generate_test", os.path.join(ROOT, "caps_gb300", "drivers", "generate_test.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    n = 448
    base = str(tmp_path / "t448")
    gen.generate(n, base, lo=-9, hi=9, seed=11)
    exe = os.path.join(os.path.dirname(caps.LIB_PATH), "..", "bin", "fromfile1")
    params = gen.valid_params(n)
    picked = [(bs, r) for bs, r in params if bs in (1, 7, 14, 56) or bs == n >> r]
    assert any(r == 6 for _, r in picked)
    for bs, r in picked:
        for form, pat in (("plain", None), ("split", "bd" * 3)):
            cmd = [exe, "-i", base + ".in", "-b", str(bs), "-r", str(r), "-c", base + ".correct", "--form", form]
            if pat and r > 0:
                cmd += ["-p", pat[:r]]
            out = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
            assert out.returncode == 0, out.stdout
            assert "Maximum deviation 0.000000e+00" in out.stdout, (bs, r, form, out.stdout)


@pytest.mark.parametrize("pat,k,ref_pat", [("hhh", 2, "bbb"), ("hhh", 3, "bbb"), ("hhh", 6, "bbb"),
                                           ("hbd", 4, "bbd"), ("hhh", 1, "ddd")])
def test_hybrid_steps_match_bfs_and_dfs_bit_for_bit(caps, oracle_mod, cuda, pat, k, ref_pat):
    """strassenHybrid2..6 (multiply.cpp:458-1080) form a 'b' step's operands and
    combine its products, running the subproducts k at a time; factor 1 runs
    the step as 'd'.  Per element the arithmetic is the same, so the results
    are bit-identical on float data."""
    import torch
    n, r = 1024, 3
    rng = np.random.default_rng(40 + k)
    A = rng.uniform(-1, 1, (n, n))
    B = rng.uniform(-1, 1, (n, n))
    dA = torch.from_numpy(caps_of(oracle_mod, A, r)).to(cuda)
    dB = torch.from_numpy(caps_of(oracle_mod, B, r)).to(cuda)
    out = {}
    for key, p, kk in (("h", pat, k), ("ref", ref_pat, 1)):
        dC = torch.full_like(dA, float("nan"))
        caps.multiply(dA, dB, dC, caps.MatDescriptor.make(n, r, 1, kk), p, form="plain")
        torch.cuda.synchronize()
        out[key] = dC.cpu().numpy()
    assert np.array_equal(out["h"], out["ref"])


def test_hybrid_split_integers_exact(caps, oracle_mod, cuda):
    import torch
    n, r = 896, 2
    rng = np.random.default_rng(3)
    A = rng.integers(-50, 51, (n, n)).astype(np.float64)
    B = rng.integers(-50, 51, (n, n)).astype(np.float64)
    dA = torch.from_numpy(caps_of(oracle_mod, A, r)).to(cuda)
    dB = torch.from_numpy(caps_of(oracle_mod, B, r)).to(cuda)
    dC = torch.full_like(dA, float("nan"))
    caps.multiply(dA, dB, dC, caps.MatDescriptor.make(n, r, 1, 3), "hh", form="split")
    torch.cuda.synchronize()
    C = mat_of(oracle_mod, dC.cpu().numpy(), n, r)
    assert np.array_equal(C, (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64))


@pytest.mark.parametrize("k", [1, 2, 5])
def test_host_entry_hybrid_top_step(caps, oracle_mod, cuda, k):
    """Host arrays with a top-level 'h' step: factor 1 runs it as 'd' with the
    copies overlapped; factors 2..6 take the copies whole before the step."""
    n, r = 512, 3
    rng = np.random.default_rng(20 + k)
    A = rng.integers(-100, 101, (n, n)).astype(np.float64)
    B = rng.integers(-100, 101, (n, n)).astype(np.float64)
    a, b = caps_of(oracle_mod, A, r), caps_of(oracle_mod, B, r)
    for form in ("plain", "split"):
        c = np.full(n * n, np.nan)
        caps.multiply(a, b, c, caps.MatDescriptor.make(n, r, 1, k), "hbd", form=form)
        assert np.array_equal(mat_of(oracle_mod, c, n, r), (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64))


@pytest.mark.parametrize("n,r,pat,ref_pat", [(1024, 2, "dd", "bb"), (1024, 3, "ddd", "bbb"), (896, 2, "bd", "bb"),
                                             (448, 1, "d", "b"), (1024, 3, "bdd", "bbb")])
def test_plain_d_step_epilogue_folds_bit_identical_to_b(caps, oracle_mod, cuda, n, r, pat, ref_pat):
    """A lean 'd' step over plain-form leaves folds its combinations into the
    products' DMMA epilogues (C22 = C12 = C11 + Q4, C22 += Q5, the U2 / Q3
    triple, C21 -= Q7, C12 += Q6, C11 += Q2).  They are the reference's FP64
    operations in its order, as calcCij does them for a 'b' step, so the two
    results agree bit for bit on float data; the fold launches no combination
    pass of its own."""
    import torch
    rng = np.random.default_rng(n + r)
    A = rng.uniform(-1, 1, (n, n))
    B = rng.uniform(-1, 1, (n, n))
    dA = torch.from_numpy(caps_of(oracle_mod, A, r)).to(cuda)
    dB = torch.from_numpy(caps_of(oracle_mod, B, r)).to(cuda)
    out, launches = {}, {}
    for p in (pat, ref_pat):
        dC = torch.full_like(dA, float("nan"))
        caps.multiply(dA, dB, dC, caps.MatDescriptor.make(n, r), p, form="plain")
        torch.cuda.synchronize()
        out[p] = dC.cpu().numpy()
        launches[p] = caps.counters()["kernel_launches"]
    assert np.array_equal(out[pat], out[ref_pat])
    if pat == "d":
        # one 'd' step over 7 leaves: 5 operand-sum launches and 7 products, no folds
        assert launches[pat] == 5 + 7


@pytest.mark.parametrize("form", ["plain", "split"])
@pytest.mark.parametrize("n,r", [(1024, 3), (512, 2), (256, 1)])
def test_host_entry_float_bit_identical_to_device(caps, oracle_mod, cuda, form, n, r):
    """The host entry point's overlapped plan (a lean top step, its first
    subproduct a lean step on sub-quadrants, the operand sums formed in one
    pass once every input is in, C12 in four parts) computes the same FP64
    operations in the same order as the device entry point's 'b' steps:
    float results agree bit for bit."""
    import torch
    rng = np.random.default_rng(n + r + len(form))
    a = caps_of(oracle_mod, rng.uniform(-1, 1, (n, n)), r)
    b = caps_of(oracle_mod, rng.uniform(-1, 1, (n, n)), r)
    c = np.full(n * n, np.nan)
    caps.multiply(a, b, c, caps.MatDescriptor.make(n, r), None, form=form)
    dC = torch.full((n * n,), float("nan"), dtype=torch.float64, device=cuda)
    caps.multiply(torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda), dC, caps.MatDescriptor.make(n, r),
                  "b" * r, form=form)
    torch.cuda.synchronize()
    assert np.array_equal(c, dC.cpu().numpy())


@pytest.mark.parametrize("form", ["plain", "split"])
def test_host_entry_tight_budget_drops_overlap_extras(caps, oracle_mod, cuda, form):
    """A workspace budget that fits the overlapped host plan only without its
    extra buffers (the one-pass sums and the early Q5): the call still runs,
    with the lean passes, and gives the device path's bits."""
    import torch
    n, r = 512, 2
    d = caps.MatDescriptor.make(n, r)
    q_bytes = (n // 2) ** 2 * 8
    budget = caps.workspace_size(d, "dd", form=form) + 2 * q_bytes  # Q2's buffers, not ten more quarters
    rng = np.random.default_rng(77)
    a = caps_of(oracle_mod, rng.uniform(-1, 1, (n, n)), r)
    b = caps_of(oracle_mod, rng.uniform(-1, 1, (n, n)), r)
    c = np.full(n * n, np.nan)
    caps.multiply(a, b, c, d, "dd", form=form, workspace_limit=budget)
    assert caps.counters()["workspace_peak_bytes"] <= budget
    dC = torch.full((n * n,), float("nan"), dtype=torch.float64, device=cuda)
    caps.multiply(torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda), dC, d, "dd", form=form)
    torch.cuda.synchronize()
    assert np.array_equal(c, dC.cpu().numpy())
