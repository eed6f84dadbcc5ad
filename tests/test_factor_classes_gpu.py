"""The factor classes (f = 1, -1, +-2^k, any) give the bits of one rounded
multiply (and one rounded add for sortacc) on every IEEE class of input:
zeros, subnormals, the normal range edges, values whose scaled result
overflows or underflows, infinities.  NaN inputs give NaN (payloads are not
part of the contract)."""
import numpy as np
import pytest

from oracle import oracle as O
from spaghetty_gb300 import sort_generic
from tests._util import first_mismatch

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TINY = np.finfo(np.float64).tiny          # 2^-1022
MAX = np.finfo(np.float64).max


def edge_values(n_random=4000, seed=3):
    vals = [0.0, -0.0, 5e-324, -5e-324, 1e-310, -3e-315, TINY, -TINY, 2 * TINY, TINY * 1.5,
            MAX, -MAX, MAX / 2, MAX / 4, 2.0 ** 1023, 2.0 ** -1021, 2.0 ** -1000, 1e-300,
            1e300, -1e308, np.inf, -np.inf, 1.0, -1.0, 0.5, 3.0, 2.0 ** 600, 2.0 ** -600]
    rng = np.random.default_rng(seed)
    r = rng.uniform(-1, 1, n_random)
    scale = 2.0 ** rng.integers(-1074, 1023, n_random).astype(np.float64)
    with np.errstate(over="ignore", under="ignore"):
        return np.concatenate([np.array(vals), r, r * scale])


def same_bits(a, b):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    nan = np.isnan(a) | np.isnan(b)
    return bool(np.all(np.isnan(a) == np.isnan(b)) and
                np.array_equal(a[~nan].view(np.uint64), b[~nan].view(np.uint64)))


@pytest.mark.parametrize("f", [1.0, -1.0, 0.5, -0.5, 2.0, 2.0 ** -10, -(2.0 ** 600),
                               2.0 ** -1030, 0.3, -37.0, 0.0])
@pytest.mark.parametrize("acc", [False, True])
def test_factor_class_bits(cuda, f, acc):
    x = edge_values()
    n = x.size
    # a rank-2 transpose so the tiled kernel (not only the flat one) runs
    a = 4
    while n % a:
        a += 1
    dims = (a, n // a)
    y = np.flip(edge_values(seed=9)[:n]).copy()
    with np.errstate(all="ignore"):
        want = O.np_sort(x, dims, (2, 1), f, 1.0 if acc else 0.0, out=y)
    for perm, wnt in [((2, 1), want), ((1, 2), None)]:
        du = torch.from_numpy(x).to(cuda)
        ds = torch.from_numpy(y.copy()).to(cuda)
        sort_generic(du, ds, dims, perm, f, 1.0 if acc else 0.0)
        got = ds.cpu().numpy()
        if wnt is None:
            with np.errstate(all="ignore"):
                wnt = O.np_sort(x, dims, perm, f, 1.0 if acc else 0.0, out=y)
        assert same_bits(got, wnt), (f, acc, perm, first_mismatch(got, wnt))
