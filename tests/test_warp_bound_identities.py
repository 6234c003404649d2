"""The 1-D warp kernel applies a one-operation boundary chain whose factor is exactly
+1 or +0 without the multiplication (lane_bound in csrc/warp_1d.cuh); its results must
be the table chain's, xadd(xmul(mul, v), sample + scalar), bit for bit. The identities
it relies on, checked in IEEE float64 (numpy rounds to nearest even like the device's
__dmul_rn / __dadd_rn) over signed zeros, subnormals, infinities and ordinary values:
  - 1 * v is v;
  - 0 * v is a zero with v's sign for finite v;
  - a zero z plus a constant c is c, or for a zero c a zero that is negative only when
    z and c both are (the integer path for held constants);
  - a sample plus a scalar of +0 is the sample with a negative zero made positive."""
import numpy as np

SIGN = np.int64(-0x8000000000000000)
SPECIAL = [0.0, -0.0, 5e-324, -5e-324, 1.0, -1.0, 2.5e-310, 1e308, -1e308, np.inf, -np.inf,
           3.0, -7.25, 1e-300]


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)[()]


def held_constant(z, c):
    """z + c for a zero z without the addition (the kernel's integer path)."""
    zb, cb = bits(z), bits(c)
    if (int(cb) << 1) & 0xFFFFFFFFFFFFFFFF:
        return np.float64(c)
    return np.float64(-0.0) if (zb < 0 and cb < 0) else np.float64(0.0)


def plus_zero(x):
    return np.float64(0.0) if bits(x) == bits(-0.0) else np.float64(x)


def test_identities():
    rng = np.random.default_rng(5)
    vals = np.concatenate([SPECIAL, rng.standard_normal(300) *
                           10.0 ** rng.integers(-300, 300, 300).astype(np.float64)])
    with np.errstate(all="ignore"):
        for v in vals.astype(np.float64):
            assert bits(np.float64(1.0) * v) == bits(v)
            if np.isfinite(v):
                assert bits(np.float64(0.0) * v) == (bits(v) & SIGN)
            assert bits(v + np.float64(0.0)) == bits(plus_zero(v))
            for z in (np.float64(0.0), np.float64(-0.0)):
                assert bits(z + v) == bits(held_constant(z, v)), (z, v)
