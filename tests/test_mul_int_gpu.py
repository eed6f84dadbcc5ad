"""Arbitrary factors (neither +-1 nor +-2^k) must give the bits of one
rounded FP64 multiply (round to nearest, ties to even) for every input:
random bit patterns over the whole exponent range, products that are exact
ties, products at the edges of the normal range (overflow to infinity by
rounding, underflow), zeros, subnormals, infinities; NaN inputs give NaN.
The flat kernel (identity permutation) computes them with its 32-bit
integer multiply, the staged kernels with the rounded FP64 multiply; both
are checked against numpy's IEEE multiply (the oracle), sort and sortacc,
through the flat, the default transpose and forced TMA-staged plans."""
import numpy as np
import pytest

from oracle import oracle as O
from spaghetty_gb300 import sort_generic
from tests._util import first_mismatch

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MAX = np.finfo(np.float64).max
TINY = np.finfo(np.float64).tiny


def factors():
    rng = np.random.default_rng(5)
    bits = rng.integers(1, 2046, 6, dtype=np.uint64) << np.uint64(52)
    bits |= rng.integers(0, 1 << 52, 6, dtype=np.uint64)
    bits[::2] |= np.uint64(1) << np.uint64(63)
    rnd = list(bits.view(np.float64))
    return [0.3, -1.25, 0.75, 1.5, -3.0, 1.0 + 2.0 ** -52, 2.0 - 2.0 ** -52, 7.0 / 3.0,
            -(1.0 + 2.0 ** -30), 1e-300, 3e300, 1.5 * TINY, MAX] + rnd


def inputs(n, f, seed):
    """Random bit patterns (every exponent), values whose product with f is
    a tie or lands at the top or bottom of the normal range, and the IEEE
    special classes."""
    rng = np.random.default_rng(seed)
    allbits = rng.integers(0, np.iinfo(np.int64).max, n // 4, dtype=np.int64).view(np.uint64)
    allbits |= rng.integers(0, 2, n // 4, dtype=np.uint64) << np.uint64(63)
    x1 = allbits.view(np.float64)
    # exponents placed so that x*f sits near 2^1024 or 2^-1022
    m = rng.uniform(1.0, 2.0, n // 4) * rng.choice([-1.0, 1.0], n // 4)
    _, ef = np.frexp(abs(f))
    e_top = 1024 - int(ef) - rng.integers(-2, 2, n // 8)
    e_bot = -1022 - int(ef) + rng.integers(-2, 3, n // 4 - n // 8)
    with np.errstate(all="ignore"):
        x2 = np.ldexp(m, np.concatenate([e_top, e_bot]).astype(np.int64))
    # ties: significands whose exact product ends in a single 1 just below
    # the last kept bit for f = 1.5 (odd significand times 3, halved) and
    # random significands otherwise
    k = rng.integers(0, 1 << 52, n // 4, dtype=np.uint64) | np.uint64(1)
    e = rng.integers(900, 1100, n // 4, dtype=np.uint64)
    x3 = ((e << np.uint64(52)) | k).view(np.float64)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -TINY, TINY, MAX, -MAX,
                        1.0, -1.0, 2.0 ** -1074 * 3])
    x = np.concatenate([x1, x2, x3, special])
    return np.resize(x, n)


def same_bits(a, b):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    nan = np.isnan(a) | np.isnan(b)
    return bool(np.all(np.isnan(a) == np.isnan(b)) and
                np.array_equal(a[~nan].view(np.uint64), b[~nan].view(np.uint64)))


@pytest.mark.parametrize("fi", range(len(factors())))
@pytest.mark.parametrize("acc", [False, True])
def test_integer_multiply_bits(cuda, fi, acc):
    f = factors()[fi]
    dims = (64, 48, 32)
    n = int(np.prod(dims))
    x = inputs(n, f, 100 + fi)
    rng = np.random.default_rng(7 + fi)
    y = rng.uniform(-1, 1, n)
    y[::97] = x[::97]          # some sums that cancel or overflow
    g = 1.0 if acc else 0.0
    for perm in [(1, 2, 3), (3, 2, 1), (2, 3, 1)]:
        with np.errstate(all="ignore"):
            want = O.np_sort(x, dims, perm, f, g, out=y)
        du = torch.from_numpy(x).to(cuda)
        ds = torch.from_numpy(y.copy()).to(cuda)
        sort_generic(du, ds, dims, perm, f, g)
        got = ds.cpu().numpy()
        assert same_bits(got, want), (f, acc, perm, first_mismatch(got, want))


@pytest.mark.parametrize("acc", [False, True])
def test_integer_multiply_bits_tma(cuda, acc):
    """The same through forced TMA-staged plans."""
    from spaghetty_gb300._lib import int_array, lib
    from spaghetty_gb300.autotune import candidates, clear
    dims = (16, 12, 10, 32)
    n = int(np.prod(dims))
    L = lib()
    ran = 0
    g = 1.0 if acc else 0.0
    try:
        for fi, f in enumerate(factors()[:8]):
            x = inputs(n, f, 300 + fi)
            y = np.random.default_rng(fi).uniform(-1, 1, n)
            for perm in [(4, 3, 2, 1), (2, 4, 1, 3)]:
                with np.errstate(all="ignore"):
                    want = O.np_sort(x, dims, perm, f, g, out=y)
                _, cands = candidates(dims, perm, int(acc))
                for box, nt, ept, st in [c for c in cands if c[3] >= 12][:2]:
                    if L.spaghetty_tune_set(4, int_array(dims), int_array(perm), int(acc),
                                            int_array(box), nt, ept, st) != 0:
                        continue
                    du = torch.from_numpy(x).to(cuda)
                    ds = torch.from_numpy(y.copy()).to(cuda)
                    sort_generic(du, ds, dims, perm, f, g)
                    got = ds.cpu().numpy()
                    assert same_bits(got, want), (f, acc, perm, box, st, first_mismatch(got, want))
                    ran += 1
                clear()
    finally:
        clear()
    assert ran > 0
