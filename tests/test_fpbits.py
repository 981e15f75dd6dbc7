"""The exact power-of-two scaling of the FP64 kernels (pow2_scale in
cans_gb300/csrc/cans_internal.cuh), restated on the host: for an FP64 x whose biased exponent
e satisfies S < e < 0x7ff the result x / 2^S is the bit pattern of x with e lowered by S;
every other x (zero, values whose result would be subnormal, infinities, NaN) takes the
multiply.  The restatement must equal the IEEE multiply bit for bit on every class of
input, which is what lets the kernels replace the multiply."""
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
