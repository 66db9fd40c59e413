"""CPU model of the tensor-core gridding arithmetic: FP16 hi/lo operands, three products
(hi*hi + hi*lo + lo*hi), FP32 accumulation.  This pins the error the GPU tests' FP32
tolerances rest on, without a GPU.

The kernels split an FP32 operand x as hi = fp16(x), lo = fp16(x - hi)
(tc_split2_f16 / tc_split8_f16, cunfft_gb300/csrc/kernels_spread_tc.cuh), after scaling
A = w0 w1 (taps in [0, 1]) by 2^10 and B = w2 f by 2^(14 - e), 2^e >= max |w2 f|, so
both stay below the FP16 maximum.  x - hi is exact in FP32, and |x - (hi + lo)| is at
most 2^-22 |x| plus 2^-25 where lo is subnormal; the dropped lo*lo term adds at most
2^-22 |a b|.  A product then carries at most about 3 x 2^-22 relative error, and a
cell's sum adds FP32 rounding over its chain of nodes.  The reference's own gridding
(src/cunfft_kernel.cu:918-972, 1098-1149) is FP64 throughout; these tests measure the
model against FP64 sums of the same FP32 operands."""
import numpy as np

SCALE_A = 2.0 ** 10  # kTcScaleA
LOG_B = 14           # kTcLogB


def split(x):
    """FP32 array -> FP16 hi, lo with hi + lo ~ x (round to nearest even, subnormals kept)."""
    x = np.asarray(x, dtype=np.float32)
    hi = x.astype(np.float16)
    lo = (x - hi.astype(np.float32)).astype(np.float16)
    return hi, lo


def product3(a, b):
    """hi_a hi_b + hi_a lo_b + lo_a hi_b, each FP16 x FP16 product exact in FP32."""
    ah, al = split(a)
    bh, bl = split(b)
    f = lambda u: u.astype(np.float64)
    return f(ah) * f(bh) + f(ah) * f(bl) + f(al) * f(bh)


def b_scale(bmax):
    e = int(np.frexp(np.float32(bmax))[1])  # 2^e > bmax
    return np.float32(2.0 ** (LOG_B - e))


def mma_sums(a, b, k=16):
    """Cell sums of a[..., j] b[..., j] over j with the three products of each k-step of
    k nodes accumulated in FP32, k-step after k-step (sequential FP32: no wider internal
    sum assumed)."""
    p = product3(a, b)
    acc = np.zeros(p.shape[:-1], dtype=np.float32)
    for s in range(0, p.shape[-1], k):
        acc = (acc + p[..., s:s + k].sum(axis=-1).astype(np.float32)).astype(np.float32)
    return acc


def test_single_products_within_the_split_bound():
    rng = np.random.default_rng(1)
    a = (rng.uniform(0, 1, 200000) * SCALE_A).astype(np.float32)
    f = rng.uniform(-1, 1, 200000)
    s = b_scale(np.abs(f).max())
    b = (f * s).astype(np.float32)
    exact = a.astype(np.float64) * b.astype(np.float64)
    err = np.abs(product3(a, b) - exact)
    floor = 2.0 ** -25 * (np.abs(a) + np.abs(b)) + 2.0 ** -48
    assert np.all(err <= 3 * 2.0 ** -22 * np.abs(exact) + floor)
    # typical products sit well inside the bound
    rel = err[exact != 0] / np.abs(exact[exact != 0])
    assert np.median(rel) < 2.0 ** -23


def test_operands_spanning_many_binades_keep_the_row_relative_error():
    """Grid values far below the row maximum: their lo parts go subnormal in FP16, which
    costs absolute error relative to the row's scale, not to the value."""
    rng = np.random.default_rng(2)
    f = rng.uniform(-1, 1, 100000) * 2.0 ** rng.uniform(-24, 0, 100000)
    s = b_scale(np.abs(f).max())
    b = (f * s).astype(np.float32)
    a = (rng.uniform(0, 1, 100000) * SCALE_A).astype(np.float32)
    exact = a.astype(np.float64) * b.astype(np.float64)
    err = np.abs(product3(a, b) - exact)
    assert np.all(err <= 3 * 2.0 ** -22 * np.abs(exact) + 2.0 ** -25 * (np.abs(a) + np.abs(b)) * SCALE_A)
    assert np.linalg.norm(err) / np.linalg.norm(exact) < 5e-7


def test_cell_sums_match_the_measured_kernel_error():
    """Gaussian taps of m = 6 (W = 14) over chains of 256 nodes per cell, as one
    work item of the 2D spreading gives a cell: relative l2 against FP64 sums of the same
    FP32 operands about 1.1e-7 (7e-8 over 16 nodes, 1.6e-7 over 1024), far below the FP32
    forms' 1e-5.  The kernels' measured error against the FP64 gridding (2.7e-7
    interpolation, 6.1e-7 spreading at 3D) adds the taps' ex2.approx rounding and the FP32
    tap products to this."""
    rng = np.random.default_rng(3)
    cells, chain = 4096, 256
    b_gauss = 2 * 2 * 6 / ((2 * 2 - 1) * np.pi)  # sigma = 2, m = 6
    y0 = rng.uniform(-7, 7, (cells, chain))
    y1 = rng.uniform(-7, 7, (cells, chain))
    w0 = np.exp(-(y0 ** 2) / b_gauss)
    w1 = np.exp(-(y1 ** 2) / b_gauss)
    a = (w0 * w1 * SCALE_A).astype(np.float32)
    f = rng.uniform(-1, 1, (cells, chain))
    s = b_scale(np.abs(f).max())
    b = (f * s).astype(np.float32)
    exact = (a.astype(np.float64) * b.astype(np.float64)).sum(axis=-1)
    got = mma_sums(a, b).astype(np.float64)
    rel = np.linalg.norm(got - exact) / np.linalg.norm(exact)
    assert rel < 1e-6, rel
    assert rel > 1e-9  # the model does round


def test_dropping_the_lo_terms_is_visible():
    """The hi*lo and lo*hi products are what take the error from FP16's 2^-11 to 2^-22:
    hi*hi alone misses the FP32 bound by orders of magnitude."""
    rng = np.random.default_rng(4)
    a = (rng.uniform(0, 1, 50000) * SCALE_A).astype(np.float32)
    b = (rng.uniform(-1, 1, 50000) * 2.0 ** 13).astype(np.float32)
    exact = a.astype(np.float64) * b.astype(np.float64)
    ah, _ = split(a)
    bh, _ = split(b)
    hh = ah.astype(np.float64) * bh.astype(np.float64)
    rel_hh = np.linalg.norm(hh - exact) / np.linalg.norm(exact)
    rel_3 = np.linalg.norm(product3(a, b) - exact) / np.linalg.norm(exact)
    assert rel_hh > 1e-4
    assert rel_3 < 1e-6
