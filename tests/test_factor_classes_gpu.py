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


@pytest.mark.parametrize("density", ["dense", "sparse"])
def test_factor_class_bits_tma(cuda, density):
    """The same bits through forced TMA-staged plans, whose permute threads
    take the integer path and fall back to the rounded multiply behind a
    warp vote: edge values everywhere (most votes take the multiply) or
    sprinkled among ordinary values (a few do), zeros on the integer path.
    Plain sorts (f = 1) on a tuned TMA plan run that path as f = 2^0."""
    from spaghetty_gb300._lib import int_array, lib
    from spaghetty_gb300.autotune import candidates, clear
    dims = (8, 12, 10, 16)
    n = int(np.prod(dims))
    rng = np.random.default_rng(17)
    edges = edge_values()
    if density == "dense":
        x = np.resize(edges, n)
        y = np.resize(np.flip(edge_values(seed=9)), n)
    else:
        x = rng.uniform(-2, 2, n)
        y = rng.uniform(-2, 2, n)
        pos = rng.choice(n, 40, replace=False)
        x[pos] = rng.choice(edges[:28], 40)
        y[pos[:10]] = rng.choice(edges[:28], 10)
    L = lib()
    ran = 0
    try:
        for perm in [(4, 3, 2, 1), (2, 3, 4, 1), (1, 3, 4, 2)]:
            for f in (1.0, -1.0, 0.5, -(2.0 ** 600), 2.0 ** -1030, 2.0 ** 1000):
                for acc in (False, True):
                    g = 1.0 if acc else 0.0
                    with np.errstate(all="ignore"):
                        want = O.np_sort(x, dims, perm, f, g, out=y)
                    _, cands = candidates(dims, perm, int(acc))
                    tma = [c for c in cands if c[3] >= 12][:2]
                    for box, nt, ept, st in tma:
                        if L.spaghetty_tune_set(4, int_array(dims), int_array(perm), int(acc),
                                                int_array(box), nt, ept, st) != 0:
                            continue
                        du = torch.from_numpy(x).to(cuda)
                        ds = torch.from_numpy(y.copy()).to(cuda)
                        sort_generic(du, ds, dims, perm, f, g)
                        got = ds.cpu().numpy()
                        assert same_bits(got, want), (f, acc, perm, box, nt, ept, st,
                                                      first_mismatch(got, want))
                        ran += 1
                clear()
    finally:
        clear()
    assert ran > 0


def test_plain_sort_large_tuned_tma_bits(cuda):
    """A plain sort (f = 1) of 2^25 elements on a tuned TMA plan, which runs
    the power-of-two path as f = 2^0: the input's bits, edge values
    included."""
    from spaghetty_gb300._lib import int_array, lib
    from spaghetty_gb300.autotune import candidates, clear
    dims = (32, 32, 128, 256)
    n = int(np.prod(dims))
    rng = np.random.default_rng(23)
    x = rng.uniform(-2, 2, n)
    pos = rng.choice(n, 2000, replace=False)
    x[pos] = rng.choice(edge_values()[:28], 2000)
    L = lib()
    ran = 0
    try:
        for perm in [(4, 3, 2, 1), (2, 1, 4, 3)]:
            want = O.np_sort(x, dims, perm, 1.0, 0.0)
            _, cands = candidates(dims, perm, 0)
            box, nt, ept, st = [c for c in cands if c[3] >= 12][0]
            assert L.spaghetty_tune_set(4, int_array(dims), int_array(perm), 0,
                                        int_array(box), nt, ept, st) == 0
            du = torch.from_numpy(x).to(cuda)
            ds = torch.empty_like(du)
            sort_generic(du, ds, dims, perm, 1.0, 0.0)
            got = ds.cpu().numpy()
            assert same_bits(got, want), (perm, first_mismatch(got, want))
            ran += 1
            clear()
    finally:
        clear()
    assert ran == 2
