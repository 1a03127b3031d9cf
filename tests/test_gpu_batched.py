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
