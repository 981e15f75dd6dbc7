"""Bit-level arithmetic of the kernels, restated on the host and checked against IEEE:

- the exact power-of-two scaling of the FP64 kernels (pow2_scale in
  cans_gb300/csrc/cans_internal.cuh): for an FP64 x whose biased exponent e satisfies
  S < e < 0x7ff, x / 2^S is the bit pattern of x with e lowered by S; every other x (zero,
  results that would be subnormal, infinities, NaN) takes the multiply;
- the FP64 <-> FP32 conversions by integer operations (cans_gb300/csrc/fpconv.cuh):
  d2f_rn / d2f_split (hi = RN(v), lo = RN(v - hi)) and the exact widening f2d, each on its
  fast range, the conversion instructions elsewhere.

Each restatement must equal the IEEE result bit for bit on every class of input (ties of
the rounding included), which is what lets the kernels replace the FP64-pipe instruction."""
import numpy as np
import pytest


def pow2_scale_model(x, s):
    b = x.view(np.int64)
    e = (b >> 52) & 0x7FF
    fast = (e > s) & (e < 0x7FF)
    out = x * (1.0 / (1 << s))
    out_bits = out.view(np.int64).copy()
    out_bits[fast] = b[fast] - (np.int64(s) << 52)
    return out_bits.view(np.float64), fast


@pytest.mark.parametrize("s", [1, 2])
def test_pow2_scale_matches_multiply(s):
    rng = np.random.default_rng(7 + s)
    # random signs, mantissas and exponents over the whole normal range
    mant = rng.random(200000) + 1.0
    expo = rng.integers(-1022, 1024, 200000)
    x = np.ldexp(mant, expo) * rng.choice([-1.0, 1.0], 200000)
    edge = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324,
                     np.ldexp(1.0, -1022), np.ldexp(1.0, -1021), np.ldexp(1.0, -1020),
                     np.ldexp(1.5, -1020), np.ldexp(1.0, -1019), np.finfo(np.float64).max,
                     -np.finfo(np.float64).max, np.ldexp(1.0, -1074 + 52)])
    x = np.concatenate([x, edge])
    got, fast = pow2_scale_model(x, s)
    want = x * (1.0 / (1 << s))
    same = (got.view(np.int64) == want.view(np.int64)) | (np.isnan(got) & np.isnan(want))
    assert same.all(), x[~same][:5]
    # the integer path covers all but the edge classes
    assert fast[:200000].mean() > 0.99


# ---- FP64 <-> FP32 conversions by integer operations (cans_gb300/csrc/fpconv.cuh) ----------
M52 = np.uint64(0xFFFFFFFFFFFFF)


def d2f_model(v):
    """d2f_rn / d2f_split restated: (hi, lo, fast) with hi = RN(v), lo = RN(v - hi) on the fast
    range, the conversions themselves elsewhere"""
    b = v.view(np.uint64)
    e = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    m = (b & M52) | (np.uint64(1) << np.uint64(52))
    q = (m >> np.uint64(29)).astype(np.int64)
    rb = (m & np.uint64(0x1FFFFFFF)).astype(np.int64)
    q = q + ((rb > 0x10000000) | ((rb == 0x10000000) & ((q & 1) == 1))).astype(np.int64)
    r = m.astype(np.int64) - (q << 29)
    ef = e - 1023 + 127
    over = (q >> 24) > 0
    qq = np.where(over, q >> 1, q)
    ef = np.where(over, ef + 1, ef)
    sign = (b >> np.uint64(63)).astype(np.int64)
    hi_bits = (sign << 31) | (ef << 23) | (qq & 0x7FFFFF)
    fast_hi = (e >= 1023 - 125) & (e <= 1023 + 126)
    hi = np.where(fast_hi, (hi_bits & 0xFFFFFFFF).astype(np.uint32).view(np.float32), v.astype(np.float32))
    scale = np.where(fast_hi, e - 1075 + 127, 127)
    scale_f = ((np.clip(scale, 1, 254).astype(np.uint32)) << np.uint32(23)).view(np.float32)
    rf = r.astype(np.float32) * scale_f
    lo_fast = np.where(sign == 1, -rf, rf)
    fast_lo = (e >= 1075 - 126) & (e <= 1023 + 126)
    lo = np.where(fast_lo, lo_fast, (v - hi.astype(np.float64)).astype(np.float32))
    return hi, lo, fast_hi, fast_lo


def test_d2f_split_matches_conversions():
    rng = np.random.default_rng(11)
    n = 400000
    x = np.ldexp(rng.random(n) + 1.0, rng.integers(-140, 140, n)) * rng.choice([-1.0, 1.0], n)
    # ties of the first rounding (the 29 dropped bits exactly one half), both parities of q
    t = np.ldexp(1.0 + (rng.integers(0, 1 << 23, 2000) * 2 + rng.integers(0, 2, 2000)) * 2.0 ** -23
                 + 2.0 ** -24, rng.integers(-100, 100, 2000))
    edge = np.array([0.0, -0.0, np.ldexp(1.0, -126), np.ldexp(1.0, -125), np.ldexp(1.0, -149),
                     np.ldexp(1.0, 127), np.ldexp(1.9999999999, 127), 3.4e38, -3.4e38, 1e-300, 1e300])
    x = np.concatenate([x, t, -t, edge])
    with np.errstate(over="ignore", under="ignore", invalid="ignore"):
        hi, lo, fast_hi, fast_lo = d2f_model(x)
        want_hi = x.astype(np.float32)
        want_lo = (x - want_hi.astype(np.float64)).astype(np.float32)
    assert (hi.view(np.uint32) == want_hi.view(np.uint32)).all()
    assert (lo.view(np.uint32) == want_lo.view(np.uint32)).all()
    assert fast_lo[:n].mean() > 0.6  # exponents -74..126 of the -140..140 drawn take the integer path


def test_f2d_exact_widening():
    rng = np.random.default_rng(12)
    f = rng.integers(0, 1 << 32, 400000, dtype=np.uint64).astype(np.uint32).view(np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    ef = (b >> np.uint64(23)) & np.uint64(0xFF)
    fast = (ef != 0) & (ef != 0xFF)
    d_bits = ((b >> np.uint64(31)) << np.uint64(63)) | ((ef + np.uint64(896)) << np.uint64(52)) | \
             ((b & np.uint64(0x7FFFFF)) << np.uint64(29))
    got = d_bits.view(np.float64)[fast]
    want = f[fast].astype(np.float64)
    assert (got.view(np.uint64) == want.view(np.uint64)).all()
