"""The oracle against the reference (CPU only).

* every committed golden digest (made by the reference's own generated C
  nests, tests/golden/make_golden.py) is reproduced by the C restatement of
  trunk/old_sort.f and by the numpy restatement;
* where the reference nests can be built here, the oracle matches them bit
  for bit directly, including the full 24-loop-order space of rank 4;
* the known-answer fixture of trunk/tester_futil.F:139-185.
"""
import itertools

import numpy as np
import pytest

from oracle import oracle as O
from tests._util import bits_equal, golden, golden_inputs, parse_key


def test_golden_digests_old_sort_restatement():
    cases = golden()
    assert len(cases) == 4032
    done = 0
    for key, digest in cases.items():
        dims, inp, perm, f, g = parse_key(key)
        u, s0 = golden_inputs(dims, inp)
        out = O.old_sort(u, dims, perm, f, out=(s0.copy() if g else None), acc=bool(g))
        assert O.digest(out)[:16] == digest, key
        done += 1
    assert done == len(cases)


def test_golden_digests_numpy_restatement():
    for key, digest in golden().items():
        dims, inp, perm, f, g = parse_key(key)
        u, s0 = golden_inputs(dims, inp)
        out = O.np_sort(u, dims, perm, f, g, out=s0)
        assert O.digest(out)[:16] == digest, key


def test_init_array_known_answer():
    # x(i,j,k,l) = i + j*a + k*a*b + l*a*b*c over the Fortran array x(a,b,c,d)
    a, b, c, d = 3, 4, 2, 5
    x = O.init_array((a, b, c, d)).reshape((d, c, b, a))  # C view of x(a,b,c,d)
    for (i, j, k, l) in [(1, 1, 1, 1), (3, 4, 2, 5), (2, 3, 1, 4)]:
        assert x[l - 1, k - 1, j - 1, i - 1] == i + j * a + k * a * b + l * a * b * c


def test_factor_semantics_match_reference_formula():
    # s = f * u.permute(p-1): e.g. b(i,j,k,l) = f*a(l,k,j,i) for perm 4321
    dims = (2, 3, 4, 5)
    u = O.fixture_values(120, 7)
    s = O.old_sort(u, dims, (4, 3, 2, 1), -0.5).reshape(5, 4, 3, 2)
    x = u.reshape(dims)
    for (i, j, k, l) in [(0, 0, 0, 0), (1, 2, 3, 4), (1, 0, 2, 3)]:
        assert s[l, k, j, i] == -0.5 * x[i, j, k, l]


def test_rank2_rank8_restatements_agree_with_numpy():
    rng = np.random.default_rng(5)
    for dims, perm in [((7, 9), (2, 1)), ((3, 2, 2, 3, 2, 1, 2, 3), (8, 1, 7, 2, 6, 3, 5, 4))]:
        n = int(np.prod(dims))
        u = rng.uniform(-1, 1, n)
        y = rng.uniform(-1, 1, n)
        assert bits_equal(O.old_sort(u, dims, perm, 0.3), O.np_sort(u, dims, perm, 0.3))
        assert bits_equal(O.old_sort(u, dims, perm, 0.3, out=y.copy(), acc=True),
                          O.np_sort(u, dims, perm, 0.3, 1.0, out=y))


def test_general_acc_factor():
    dims = (3, 4, 5)
    u = O.fixture_values(60, 3)
    y = O.fixture_values(60, 4)
    got = O.sort_generic(u, dims, (3, 1, 2), 0.7, -2.5, out=y.copy())
    want = O.np_sort(u, dims, (3, 1, 2), 0.7, -2.5, out=y)
    assert bits_equal(got, want)


@pytest.fixture(scope="module")
def refnests():
    from oracle import refnests as R
    if not R.available():
        pytest.skip("reference nests not built (no reference checkout or generated C)")
    return R


def test_reference_nests_all_loop_orders_rank4(refnests):
    dims = (3, 5, 4, 7)
    n = int(np.prod(dims))
    u = O.fixture_values(n, 11)
    y = O.fixture_values(n, 12)
    for perm in itertools.permutations((1, 2, 3, 4)):
        want = O.old_sort(u, dims, perm, -0.5)
        want_acc = O.old_sort(u, dims, perm, 37.0, out=y.copy(), acc=True)
        loops = refnests.loops_for(4, perm)
        assert len(loops) == 24
        for lo in loops:
            s = np.zeros(n)
            refnests.call(perm, lo, u, s, dims, -0.5, 0.0)
            assert bits_equal(s, want), (perm, lo)
            s = y.copy()
            refnests.call(perm, lo, u, s, dims, 37.0, 1.0)
            assert bits_equal(s, want_acc), (perm, lo)


def test_reference_nests_rank6_all_perms(refnests):
    dims = (2, 3, 2, 3, 2, 2)
    n = int(np.prod(dims))
    u = O.fixture_values(n, 13)
    y = O.fixture_values(n, 14)
    for perm in itertools.permutations(range(1, 7)):
        lo = refnests.loops_for(6, perm)[0]
        s = np.zeros(n)
        refnests.call(perm, lo, u, s, dims, 0.3, 0.0)
        assert bits_equal(s, O.old_sort(u, dims, perm, 0.3)), perm
        s = y.copy()
        refnests.call(perm, lo, u, s, dims, 0.3, 1.0)
        assert bits_equal(s, O.old_sort(u, dims, perm, 0.3, out=y.copy(), acc=True)), perm
