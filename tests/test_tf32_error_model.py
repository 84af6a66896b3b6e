"""Where the split-TF32x3 form loses bits: an error model of the tensor-core
product, checked against the plain FP32 form and against the GPU.

The TF32x3 kernels (csrc/b2g_tc.cu, b2g_g1.cu, split_tf32 in
b2g_tcgen05.cuh) round each FP32 operand x to hi = tf32_rna(x) and
lo = tf32_rna(x - hi), issue hi*hi + hi*lo + lo*hi into an FP32 accumulator,
store the GEMM0 result W in FP32 and split it again for GEMM1.  A TF32 value
has 10 explicit mantissa bits, so hi + lo keeps 22 significant bits of x
(|x - hi - lo| <= 2^-22 |x|) where an FP32 operand keeps 24, and the dropped
lo*lo term is of the same order: each product carries about four times the
FP32 rounding error, which cancellation in sigma then amplifies as it does
for FP32.  The emulation below reproduces exactly those roundings on the CPU
(every TF32 product of 11-bit mantissas is exact in FP32; numpy's float32
matmul accumulates in FP32) and measures both forms against the FP64 oracle.
"""
import numpy as np
import pytest

from oracle import oracle


def tf32_rna(x32):
    """Round FP32 to TF32 (10 explicit mantissa bits), nearest, ties away from
    zero (the cvt.rna.tf32.f32 rounding): add half an ulp to the magnitude
    bits and clear the 13 low bits."""
    b = np.ascontiguousarray(x32, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x1000) & 0xFFFFE000).astype(np.uint32)
    return b.view(np.float32)


def split(x32):
    hi = tf32_rna(x32)
    lo = tf32_rna((x32 - hi).astype(np.float32))
    return hi, lo


def mm_tf32x3(a32, b32):
    ah, al = split(a32)
    bh, bl = split(b32)
    return (ah @ bh + ah @ bl + al @ bh).astype(np.float32)


def block(buf, off, rows, cols, ld, trans):
    """op(X) of shape rows x cols read from buf at off with leading dim ld."""
    if trans:
        idx = off + np.arange(cols)[None, :] * ld + np.arange(rows)[:, None]
    else:
        idx = off + np.arange(rows)[:, None] * ld + np.arange(cols)[None, :]
    return buf[idx]


def emulate(seq, ops, psi, sigma_size, form):
    """sigma = H_eff psi with the roundings of one arithmetic form:
    'fp32' (FP32 operands and accumulation) or 'tf32x3' (the split form)."""
    a = seq.arrays
    ops32 = ops.astype(np.float32)
    psi32 = psi.astype(np.float32)
    sig = np.zeros(sigma_size)
    for i in range(seq.n):
        m0, n0, k0 = int(a["m0"][i]), int(a["n0"][i]), int(a["k0"][i])
        m1, n1, k1 = int(a["m1"][i]), int(a["n1"][i]), int(a["k1"][i])
        if min(m0, n0, k0, m1, n1, k1) == 0:
            continue
        x = block(psi32, int(a["a0"][i]), m0, k0, int(a["lda0"][i]), False)
        r = block(ops32, int(a["b0"][i]), k0, n0, int(a["ldb0"][i]), bool(a["tb0"][i]))
        l_ = block(ops32, int(a["a1"][i]), m1, k1, int(a["lda1"][i]), bool(a["ta1"][i]))
        if form == "fp32":
            w = (np.float32(a["alpha0"][i]) * (x @ r)).astype(np.float32)
            t = (np.float32(a["alpha1"][i]) * (l_ @ w)).astype(np.float32)
        else:
            w = (np.float32(a["alpha0"][i]) * mm_tf32x3(x, r)).astype(np.float32)
            t = (np.float32(a["alpha1"][i]) * mm_tf32x3(l_, w)).astype(np.float32)
        c1, ldc = int(a["c1"][i]), int(a["ldc1"][i])
        idx = c1 + np.arange(m1)[:, None] * ldc + np.arange(n1)[None, :]
        np.add.at(sig, idx, t.astype(np.float64))
    return sig


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_tf32_rounding_keeps_22_bits():
    rng = np.random.default_rng(5)
    x = (rng.standard_normal(100000) * 10.0 ** rng.uniform(-6, 6, 100000)).astype(np.float32)
    hi, lo = split(x)
    # hi is a TF32 value (13 low bits clear) within half a TF32 ulp of x
    assert np.all((hi.view(np.uint32) & 0x1FFF) == 0) and np.all((lo.view(np.uint32) & 0x1FFF) == 0)
    assert np.all(np.abs(x.astype(np.float64) - hi) <= 2.0 ** -11 * np.abs(x) * 1.0000001)
    resid = np.abs(x.astype(np.float64) - hi.astype(np.float64) - lo.astype(np.float64))
    assert np.all(resid <= 2.0 ** -22 * np.abs(x) * 1.0000001)
    # the representation loses bits FP32 keeps: some residuals exceed half an
    # FP32 ulp (2^-24 relative), up to the 2^-22 bound
    assert np.max(resid / np.abs(x)) > 2.0 ** -24


@pytest.mark.parametrize("name", ["hub16_su2_M250", "syn8_su2", "hub8_sz"])
def test_split_tf32_error_is_a_few_times_fp32(problems, name):
    p = problems[name]
    seq = p.seq()
    ref = oracle.replay(seq, p.ops, p.psi, p.sigma_size)
    e32 = rel(emulate(seq, p.ops, p.psi, p.sigma_size, "fp32"), ref)
    e3 = rel(emulate(seq, p.ops, p.psi, p.sigma_size, "tf32x3"), ref)
    # 22 instead of 24 bits per operand, plus the dropped lo*lo term: a small
    # multiple of the FP32 error, far from TF32's own 11 bits
    assert 1.5 * e32 < e3 < 20 * e32, (e3, e32)
    assert e3 < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["hub16_su2_M250", "syn8_su2"])
def test_gpu_tf32x3_error_matches_the_model(problems, name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import b2g
    p = problems[name]
    seq = p.seq()
    ref = oracle.replay(seq, p.ops, p.psi, p.sigma_size)
    model = rel(emulate(seq, p.ops, p.psi, p.sigma_size, "tf32x3"), ref)
    ctx = b2g.Context(0)
    h = b2g.EffectiveHamiltonian(ctx, seq, p.ops, p.psi_size, p.sigma_size)
    out = {}
    for name_, form in (("tf32x3", b2g.TF32X3), ("fp32", b2g.FP32)):
        sig = np.zeros(p.sigma_size)
        h(p.psi.copy(), sig, 1.0, form)
        out[name_] = rel(sig, ref)
    h.close()
    ctx.close()
    # the GPU's split-K order and FP64 reduction differ from the emulation's
    # order; the error is the same size
    assert model / 3 < out["tf32x3"] < 3 * model, (out, model)
    assert out["tf32x3"] > out["fp32"]
