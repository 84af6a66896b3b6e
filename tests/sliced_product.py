"""CPU reference of an FP64-accurate product built from exact low-precision
slice products (Ozaki's error-free splitting: Ozaki, Ogita, Oishi and Rump,
"Error-free transformations of matrix multiplication by using fast routines
of matrix multiplication and its applications", Numer. Algorithms 59, 2012).

Test infrastructure: it is the reference a tensor-core version of the FP64
H_eff*psi product is to be checked against, and it sizes that product (how
many slices give which accuracy).  No product path calls it.

A (m x k) is scaled per row and B (k x n) per column by powers of two so
that every entry lies in (-1, 1), then cut into S signed base-2^7 digits
(integers of magnitude <= 127, exact in BF16).  Digit products are exact
integers; a K chunk of at most 1024 of them sums exactly in FP32 (|sum| <=
1024 * 127^2 < 2^24).  The slice products with s + t < S are recombined in
FP64 and the scalings undone.
"""
from __future__ import annotations

import numpy as np

DIGIT_BITS = 7        # |digit| <= 127: exact in BF16 (8 significant bits)
EXACT_K_CHUNK = 1024  # digit products a FP32 accumulator sums exactly


def split(x: np.ndarray, n_slices: int, axis: int):
    """Digits (n_slices, *x.shape) as int64 and the power-of-two exponents
    (per row for axis=1, per column for axis=0) with
    x = 2**e * sum_s digits[s] * 2**(-7 (s + 1)) + a remainder below 2**(e - 7 S)."""
    mx = np.max(np.abs(x), axis=axis, keepdims=True)
    # 2**e strictly above the largest magnitude, so every digit stays within +-127
    e = np.where(mx > 0, np.floor(np.log2(np.where(mx > 0, mx, 1.0))) + 1.0, 0.0)
    r = x * np.exp2(-e)
    digits = np.empty((n_slices,) + x.shape, dtype=np.int64)
    for s in range(n_slices):
        r = r * 2.0 ** DIGIT_BITS
        d = np.trunc(r)
        digits[s] = d.astype(np.int64)
        r = r - d
    return digits, e


def sliced_matmul(a: np.ndarray, b: np.ndarray, n_slices: int) -> np.ndarray:
    """a @ b from the digit products with s + t < n_slices (each exact),
    recombined in FP64."""
    da, ea = split(a, n_slices, 1)
    db, eb = split(b, n_slices, 0)
    c = np.zeros((a.shape[0], b.shape[1]))
    for s in range(n_slices):
        for t in range(n_slices - s):
            c += (da[s] @ db[t]).astype(np.float64) * 2.0 ** (-DIGIT_BITS * (s + t + 2))
    return c * np.exp2(ea) * np.exp2(eb)


def _view(blob, off, rows, cols, ld, trans):
    if trans:
        return np.lib.stride_tricks.as_strided(blob[off:], shape=(cols, rows), strides=(ld * 8, 8)).T
    return np.lib.stride_tricks.as_strided(blob[off:], shape=(rows, cols), strides=(ld * 8, 8))


def sliced_heff(pairs: dict, ops: np.ndarray, psi: np.ndarray, sigma_size: int, n_slices: int) -> np.ndarray:
    """H_eff*psi over a recorded pair list with both GEMMs of every pair as
    sliced products (W recombined in FP64 and sliced again for GEMM1)."""
    sigma = np.zeros(sigma_size)
    for i in range(len(pairs["m0"])):
        m0, n0, k0 = int(pairs["m0"][i]), int(pairs["n0"][i]), int(pairs["k0"][i])
        m1, n1, k1 = int(pairs["m1"][i]), int(pairs["n1"][i]), int(pairs["k1"][i])
        if min(m0, n0, k0, m1, n1, k1) == 0:
            continue
        a0 = _view(psi, int(pairs["a0"][i]), m0, k0, int(pairs["lda0"][i]), False)
        b0 = _view(ops, int(pairs["b0"][i]), k0, n0, int(pairs["ldb0"][i]), bool(pairs["tb0"][i]))
        a1 = _view(ops, int(pairs["a1"][i]), m1, k1, int(pairs["lda1"][i]), bool(pairs["ta1"][i]))
        w = pairs["alpha0"][i] * sliced_matmul(a0, b0, n_slices)
        c = pairs["alpha1"][i] * sliced_matmul(a1, w, n_slices)
        ldc, c1 = int(pairs["ldc1"][i]), int(pairs["c1"][i])
        for r in range(m1):
            sigma[c1 + r * ldc: c1 + r * ldc + n1] += c[r]
    return sigma
