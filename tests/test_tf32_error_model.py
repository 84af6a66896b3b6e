"""Where the split-TF32x3 form loses bits: an error model of the tensor-core
product, checked against the plain FP32 form and against the GPU.

The TF32x3 kernels (csrc/b2g_tc.cu, b2g_g1.cu, split_tf32 in
b2g_tcgen05.cuh) round each FP32 operand x to hi = tf32_rna(x) and
lo = tf32_rna(x - hi), issue hi*hi + hi*lo + lo*hi into an FP32 accumulator in
TMEM (one MMA instruction sums 8 products of K), store the GEMM0 result W in
FP32 and split it again for GEMM1 (whose left operand image holds alpha*op(L)).

Two error sources, emulated on the CPU with exactly these roundings (TF32
products of 11-bit mantissas are exact in FP32 and in FP64):
  * the split keeps 22 significant bits of x (|x - hi - lo| <= 2^-22 |x|,
    against FP32's 2^-24) and drops lo*lo: with round-to-nearest FP32
    accumulation this alone is 1.5-2x the FP32 form's error;
  * the accumulation: each MMA's group of products is added to the FP32
    accumulator; if those adds truncate (round toward zero) instead of
    rounding to nearest, the error grows with the number of adds.
The GPU's TF32x3 error lies between two emulations: round-to-nearest adds
with each pair's result summed in FP64 (below it), and truncating adds with
every pair's result accumulated in FP32 (above it; the GPU holds GEMM1 tiles
in FP32 across the contributions of a split-K chunk).  So the accumulation,
not the split, is where most of the bits go, and shorter accumulation chains
(the GEMM1 split-K chunk) are the knob.
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


def round_toward_zero32(x64):
    f = np.asarray(x64, dtype=np.float64)
    r = f.astype(np.float32)
    away = np.abs(r.astype(np.float64)) > np.abs(f)
    return np.where(away, np.nextafter(r, np.float32(0)), r).astype(np.float32)


def mm_tf32x3_mma(a32, b32, group=8):
    """hi*hi, hi*lo, lo*hi issued as MMAs over K groups of `group` products:
    each group summed exactly, then added to the FP32 accumulator with a
    truncating add (the pessimistic accumulator model)."""
    ah, al = split(a32)
    bh, bl = split(b32)
    acc = np.zeros((a32.shape[0], b32.shape[1]), dtype=np.float32)
    for g0 in range(0, a32.shape[1], group):
        for x, y in ((ah, bh), (ah, bl), (al, bh)):
            part = x[:, g0:g0 + group].astype(np.float64) @ y[g0:g0 + group, :].astype(np.float64)
            acc = round_toward_zero32(acc.astype(np.float64) + part)
    return acc


def block(buf, off, rows, cols, ld, trans):
    """op(X) of shape rows x cols read from buf at off with leading dim ld."""
    if trans:
        idx = off + np.arange(cols)[None, :] * ld + np.arange(rows)[:, None]
    else:
        idx = off + np.arange(rows)[:, None] * ld + np.arange(cols)[None, :]
    return buf[idx]


def emulate(seq, ops, psi, sigma_size, form):
    """sigma = H_eff psi with the roundings of one arithmetic form: 'fp32'
    (FP32 operands and accumulation), 'tf32x3' (the split form, accumulation
    rounded to nearest, each pair's result added to sigma in FP64) or
    'tf32x3_rz' (the split form, truncating MMA-group adds, alpha folded into
    the left operand as in the GEMM1 images, and every pair's result added
    into an FP32 sigma with truncating adds: the GPU keeps GEMM1 tiles in FP32
    across the contributions of a split-K chunk, so this bounds it from above)."""
    a = seq.arrays
    ops32 = ops.astype(np.float32)
    psi32 = psi.astype(np.float32)
    sig = np.zeros(sigma_size)
    sig32 = np.zeros(sigma_size, dtype=np.float32)
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
        elif form == "tf32x3_rz":
            w = (np.float32(a["alpha0"][i]) * mm_tf32x3_mma(x, r)).astype(np.float32)
            t = mm_tf32x3_mma((np.float32(a["alpha1"][i]) * l_).astype(np.float32), w)
        else:
            w = (np.float32(a["alpha0"][i]) * mm_tf32x3(x, r)).astype(np.float32)
            t = (np.float32(a["alpha1"][i]) * mm_tf32x3(l_, w)).astype(np.float32)
        c1, ldc = int(a["c1"][i]), int(a["ldc1"][i])
        idx = c1 + np.arange(m1)[:, None] * ldc + np.arange(n1)[None, :]
        if form == "tf32x3_rz":
            idx = idx.ravel()
            sig32[idx] = round_toward_zero32(sig32[idx].astype(np.float64) + t.ravel().astype(np.float64))
        else:
            np.add.at(sig, idx, t.astype(np.float64))
    return sig32.astype(np.float64) if form == "tf32x3_rz" else sig


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
def test_gpu_tf32x3_error_lies_between_the_accumulator_models(problems, name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import b2g
    p = problems[name]
    seq = p.seq()
    ref = oracle.replay(seq, p.ops, p.psi, p.sigma_size)
    rn = rel(emulate(seq, p.ops, p.psi, p.sigma_size, "tf32x3"), ref)
    rz = rel(emulate(seq, p.ops, p.psi, p.sigma_size, "tf32x3_rz"), ref)
    ctx = b2g.Context(0)
    h = b2g.EffectiveHamiltonian(ctx, seq, p.ops, p.psi_size, p.sigma_size)
    out = {}
    for name_, form in (("tf32x3", b2g.TF32X3), ("fp32", b2g.FP32)):
        sig = np.zeros(p.sigma_size)
        h(p.psi.copy(), sig, 1.0, form)
        out[name_] = rel(sig, ref)
    h.close()
    ctx.close()
    # measured on GB300: 2.8e-7 (hub16) and 9.3e-7 (syn8) between the models
    # (6.5e-8 / 8.3e-8 round-to-nearest per pair; 5.5e-7 / 1.4e-6 truncating
    # FP32 accumulation across pairs)
    assert rn < out["tf32x3"] < rz, (out, rn, rz)
    assert out["tf32x3"] > out["fp32"]
