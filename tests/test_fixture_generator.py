"""CPU tests of the known-answer fixture generator (caps_gb300/drivers/
generate_test.py): its parameter lines are the ones the reference's own
tests/*.params list, and its files read back as A, B and the exact A*B."""
import importlib.util
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def gen_module():
    path = os.path.join(ROOT, "caps_gb300", "drivers", "generate_test.py")
    spec = importlib.util.spec_from_file_location("caps_generate_test", path)
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_valid_params_match_reference_param_files():
    g = np.load(os.path.join(ROOT, "tests", "golden", "ref_tests.npz"))
    gen = gen_module()
    for key in g.files:
        if not key.startswith("params"):
            continue
        n = int(key[len("params"):])
        assert sorted(map(tuple, g[key].tolist())) == sorted(gen.valid_params(n)), n


def test_generated_files_read_back_exactly(tmp_path):
    gen = gen_module()
    n = 48
    A, B, C = gen.generate(n, str(tmp_path / "t48"), lo=-3, hi=7, seed=5)
    vals = np.array(open(tmp_path / "t48.in").read().split(), dtype=np.int64)
    assert vals[0] == n and vals.size == 1 + 2 * n * n
    assert np.array_equal(vals[1:1 + n * n].reshape(n, n), A)
    assert np.array_equal(vals[1 + n * n:].reshape(n, n), B)
    Cf = np.array(open(tmp_path / "t48.correct").read().split(), dtype=np.int64).reshape(n, n)
    assert np.array_equal(Cf, A @ B) and np.array_equal(C, A @ B)
    lines = open(tmp_path / "t48.params").read().splitlines()
    assert len(lines) == len(gen.valid_params(n))
    for line in lines:
        f = line.split()
        bs, r = int(f[f.index("-b") + 1]), int(f[f.index("-r") + 1])
        assert n % ((1 << r) * bs) == 0
