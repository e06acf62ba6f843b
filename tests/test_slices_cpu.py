"""The fixed-point fp16 slicing of the tensor-core stage, emulated in numpy float32
(round to nearest, as the kernels' __f*_rn intrinsics): the slices are fp16
integers, the anti-diagonal sums D2 and D3 of the slice products are exact in
FP32, D4 and D5 round only beyond 2^24, and the recombined product matches the
FP64 dot product to ~2^-35 of the row and column scales (the slices hold 40
bits, but the float-float operand enters them through one float32 remainder,
|r| <= 1/2 of the leading slice: ~2^-25 absolute, 2^-35 of the row scale).

This checks the arithmetic argument of the mixed path on the CPU; the kernels
themselves are compared with the FP64 path in the GPU tests."""
import numpy as np

SLB, NSL, K = 10, 4, 16
f32 = np.float32


def exp_of(m):
    """e with m = f 2^e, f in [0.5, 1) (m > 0, float32)."""
    return int((np.array(m, dtype=f32).view(np.int32) >> 23) & 0xFF) - 126


def to_ff(x):
    hi = x.astype(f32)
    lo = (x - hi.astype(np.float64)).astype(f32)
    return hi, lo


def slice_scaled(hi, lo, scale):
    """The kernel's slice_scaled: NSL slices of (hi + lo) * scale, base 2^10."""
    h = (hi * f32(scale)).astype(f32)
    l = (lo * f32(scale)).astype(f32)
    out = [np.rint(h).astype(f32)]
    r = ((h - out[0]).astype(f32) + l).astype(f32)
    for _ in range(1, NSL):
        r = (r * f32(1024.0)).astype(f32)
        s = np.rint(r).astype(f32)
        out.append(s)
        r = (r - s).astype(f32)
    return out


def slice_rows(x):
    """Rows of x (float64) -> slices with a power-of-two scale per row."""
    hi, lo = to_ff(x)
    sl = np.zeros((NSL,) + x.shape, dtype=f32)
    scl = np.zeros(x.shape[0])
    for r in range(x.shape[0]):
        e = exp_of(np.max(np.abs(hi[r])))
        s = slice_scaled(hi[r], lo[r], 2.0 ** (SLB - e))
        for q in range(NSL):
            sl[q, r] = s[q]
        scl[r] = 2.0 ** (e - SLB)
    return sl, scl


def fp32_accumulate(terms):
    """Sum of products in a float32 accumulator, one rounding per addition."""
    acc = np.zeros(terms[0].shape[:-1], dtype=f32)
    for t in terms:
        for k in range(t.shape[-1]):
            acc = (acc + t[..., k]).astype(f32)
    return acc


def test_slices_are_fp16_integers_and_reconstruct():
    rng = np.random.default_rng(3)
    x = rng.standard_normal((64, K)) * np.exp(rng.uniform(-20, 20, (64, 1)))
    sl, scl = slice_rows(x)
    assert np.all(sl == np.rint(sl))
    assert np.all(np.abs(sl[0]) <= 2 ** SLB) and np.all(np.abs(sl[1:]) <= 2 ** (SLB - 1))
    assert np.all(sl.astype(np.float16).astype(f32) == sl)
    rec = sum(sl[q].astype(np.float64) * 2.0 ** (-SLB * q) for q in range(NSL)) * scl[:, None]
    rowmax = np.max(np.abs(x), axis=1, keepdims=True)
    assert np.max(np.abs(rec - x) / rowmax) < 2.0 ** -34


def test_diagonal_sums_and_recombination():
    rng = np.random.default_rng(4)
    M, N = 48, 32
    a = rng.standard_normal((M, K)) * np.exp(rng.uniform(-10, 10, (M, 1)))
    b = rng.standard_normal((N, K)) * np.exp(rng.uniform(-10, 10, (N, 1)))
    A, sa = slice_rows(a)
    B, sb = slice_rows(b)
    D = {}
    for s in range(NSL):  # D_{s+2} = sum_{i+j=s} A_i B_j^T, slices numbered from 0 here
        prods = [A[i][:, None, :].astype(f32) * B[s - i][None, :, :].astype(f32) for i in range(s + 1)]
        exact = sum(p.astype(np.int64) for p in prods).sum(axis=-1)
        got = fp32_accumulate(prods)
        if s <= 1:  # D2, D3: every partial sum stays within 2^24
            assert np.array_equal(got.astype(np.int64), exact)
        else:  # D4, D5: rounding only where a partial sum passes 2^24
            assert np.max(np.abs(got.astype(np.float64) - exact)) <= 2.0
        D[s] = got
    # recombination as in the readout: D2 + D3 2^-10 + D4 2^-20 + D5 2^-30
    val = sum(D[s].astype(np.float64) * 2.0 ** (-SLB * s) for s in range(NSL)) * sa[:, None] * sb[None, :]
    ref = a @ b.T
    scale = np.max(np.abs(a), axis=1)[:, None] * np.max(np.abs(b), axis=1)[None, :] * K
    assert np.max(np.abs(val - ref) / scale) < 2.0 ** -33
