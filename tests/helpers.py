"""Shared helpers for the tests: layout conversions through the oracle and
GPU runs through the C ABI."""
import numpy as np


def caps_of(oracle, M, r, bs=1):
    """CAPS layout (flat) of a square numpy matrix M."""
    n = M.shape[0]
    return oracle.to_caps(np.ascontiguousarray(M.T).reshape(-1), n, r, bs)


def mat_of(oracle, flat, n, r, bs=1):
    """Square numpy matrix from its CAPS layout."""
    return oracle.from_caps(flat, n, r, bs).reshape(n, n).T


def gpu_multiply(caps, oracle, A, B, r, bs=1, pattern=None, form="plain", slices=0, diagonals=0,
                 device="cuda:0", scheme="auto", tile=0, operand_bits=0):
    import torch
    n = A.shape[0]
    dA = torch.from_numpy(caps_of(oracle, A, r, bs)).to(device)
    dB = torch.from_numpy(caps_of(oracle, B, r, bs)).to(device)
    dC = torch.full_like(dA, float("nan"))
    caps.multiply(dA, dB, dC, caps.MatDescriptor.make(n, r, bs), pattern, form=form, slices=slices,
                  diagonals=diagonals, scheme=scheme, tile=tile, operand_bits=operand_bits)
    torch.cuda.synchronize()
    return mat_of(oracle, dC.cpu().numpy(), n, r, bs)


def dd_of(oracle, A, B):
    n = A.shape[0]
    hi, lo = oracle.dd_gemm(np.ascontiguousarray(A.T).reshape(-1), np.ascontiguousarray(B.T).reshape(-1), n)
    return hi.reshape(n, n).T, lo.reshape(n, n).T


def rel_err(C, hi, lo, A, B):
    """max |C - C_dd| / (|A||B|) elementwise, and normwise."""
    d = (C - hi) - lo
    ab = np.abs(A) @ np.abs(B)
    ew = float(np.max(np.abs(d) / np.where(ab > 0, ab, 1)))
    nw = float(np.linalg.norm(d) / max(np.linalg.norm(hi), 1e-300))
    return ew, nw
