"""The slice arithmetic of an FP64-accurate tensor-core H_eff*psi
(tests/sliced_product.py): its digits are exact in BF16, a K chunk of digit
products is exact in FP32, and on the reference's H_eff fixtures the error
against the FP64 replay falls by about two decades per 7-bit slice (the
sizing of that product: 7 slices ~1e-13, 8 slices at FP64 level)."""
import numpy as np
import pytest

from oracle import oracle
from sliced_product import DIGIT_BITS, EXACT_K_CHUNK, sliced_heff, sliced_matmul, split

# relative error bound per slice count on the fixtures (measured: 4.6e-8..1.1e-7,
# 4.0e-12..1.2e-11, 3.7e-14..1.2e-13, 3.9e-16..1.1e-15)
BOUNDS = {4: 3e-7, 6: 3e-11, 7: 3e-13, 8: 3e-15}


def test_digits_are_exact_bf16_integers():
    rng = np.random.default_rng(3)
    x = rng.standard_normal((17, 23)) * np.exp2(rng.integers(-30, 30, size=(17, 1)))
    d, e = split(x, 8, 1)
    assert np.abs(d).max() <= 2 ** DIGIT_BITS - 1
    # an integer of magnitude <= 127 has at most 7 significant bits: exact in BF16 (8)
    f = d.astype(np.float64)
    assert np.all(np.frexp(f)[0] * 256 == np.round(np.frexp(f)[0] * 256))
    # the digits rebuild x to 2^-56 of each row's scale
    rebuilt = sum(d[s] * 2.0 ** (-DIGIT_BITS * (s + 1)) for s in range(8)) * np.exp2(e)
    assert np.all(np.abs(rebuilt - x) <= np.exp2(e) * 2.0 ** (-DIGIT_BITS * 8))


def test_power_of_two_entries_keep_digits_in_range():
    x = np.array([[1.0, -0.5, 0.25], [-4.0, 3.0, 0.0], [0.0, 0.0, 0.0]])
    d, e = split(x, 3, 1)
    assert np.abs(d).max() <= 2 ** DIGIT_BITS - 1
    rebuilt = sum(d[s] * 2.0 ** (-DIGIT_BITS * (s + 1)) for s in range(3)) * np.exp2(e)
    np.testing.assert_array_equal(rebuilt, x)


def test_k_chunk_of_digit_products_is_exact_in_fp32():
    worst = EXACT_K_CHUNK * (2 ** DIGIT_BITS - 1) ** 2
    assert worst < 2 ** 24
    # the largest chunk, summed one product at a time in FP32, stays exact
    prods = np.full(EXACT_K_CHUNK, 127 * 127, dtype=np.float32)
    acc = np.float32(0)
    for v in prods:
        acc = np.float32(acc + v)
    assert int(acc) == EXACT_K_CHUNK * 127 * 127


def test_sliced_matmul_converges_to_fp64():
    rng = np.random.default_rng(4)
    a, b = rng.standard_normal((30, 50)), rng.standard_normal((50, 20))
    ref = a @ b
    errs = [np.linalg.norm(sliced_matmul(a, b, s) - ref) / np.linalg.norm(ref) for s in (4, 6, 8)]
    assert errs[0] > errs[1] > errs[2] and errs[2] < 1e-15


@pytest.mark.parametrize("name", ["hub8_su2", "syn8_su2", "hub16_su2_M250"])
def test_sliced_heff_error_per_slice_count(problems, name):
    p = problems[name]
    ref = oracle.replay(p.seq(), p.ops, p.psi, p.sigma_size)
    for n_slices, bound in BOUNDS.items():
        out = sliced_heff(p.pairs, p.ops, p.psi, p.sigma_size, n_slices)
        assert np.linalg.norm(out - ref) / np.linalg.norm(ref) <= bound, (name, n_slices)
