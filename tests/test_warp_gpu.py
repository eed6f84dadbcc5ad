"""The warp-shuffle transpose (plan kind "warp"): transposes whose input
and output stride-1 extents are at most 32 with a product of at most 128
move each inner tile through one warp's registers with warp shuffles.
Forced on (SPAGHETTY_OPT_WARP_TR = 2) at small shapes of ranks 2 to 8, every
permutation (a seeded sample at ranks 6 and 8), every factor case, against
the oracle bit for bit; also misaligned buffers (the kernel uses plain
8-byte loads and stores) and the default rule at 10^6 (2^22 elements or
fewer take it)."""
import itertools
import random

import numpy as np
import pytest

from oracle import oracle as O
from spaghetty_gb300 import plan, sort_generic
from spaghetty_gb300._lib import lib
from tests._util import bits_equal, first_mismatch

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

OPT_WARP_TR = 4
CASES = [(1.0, 0.0), (-1.0, 0.0), (0.5, 0.0), (-1.25, 0.0), (1.0, 1.0), (-1.0, 1.0),
         (0.75, 1.0), (0.3, -2.5)]


@pytest.fixture
def warp_forced():
    L = lib()
    assert L.spaghetty_set_option(OPT_WARP_TR, 2) == 0
    yield
    assert L.spaghetty_set_option(OPT_WARP_TR, 1) == 0


def perms_of(rank, k, seed):
    allp = list(itertools.permutations(range(1, rank + 1)))
    return allp if len(allp) <= k else random.Random(seed).sample(allp, k)


@pytest.mark.parametrize("dims", [(7, 9), (32, 4), (3, 5, 7, 2), (10, 10, 10, 10), (8, 16, 4, 12),
                                  (6, 5, 4, 7, 3, 9), (10, 3, 4, 5, 6, 11), (2, 3, 2, 5, 3, 2, 4, 3)])
def test_warp_transpose_bits(cuda, warp_forced, dims):
    n = int(np.prod(dims))
    rng = np.random.default_rng(n)
    u = rng.uniform(-1, 1, n)
    y0 = rng.uniform(-1, 1, n)
    du = torch.from_numpy(u).to(cuda)
    ran = 0
    for perm in perms_of(len(dims), 60, n):
        kind = plan(dims, perm, 0)["kind"]
        for f, g in CASES:
            ds = torch.from_numpy(y0.copy()).to(cuda)
            sort_generic(du, ds, dims, perm, f, g)
            got = ds.cpu().numpy()
            want = O.np_sort(u, dims, perm, f, g, out=y0)
            assert bits_equal(got, want), (dims, perm, f, g, kind, first_mismatch(got, want))
        ran += kind == "warp"
    assert ran > 0


def test_warp_transpose_misaligned(cuda, warp_forced):
    """Buffers offset by one element (8 bytes): the kernel has no 16-byte rule."""
    dims, perm = (10, 10, 10, 10), (4, 3, 2, 1)
    assert plan(dims, perm, 0)["kind"] == "warp"
    n = int(np.prod(dims))
    rng = np.random.default_rng(3)
    u = rng.uniform(-1, 1, n)
    y0 = rng.uniform(-1, 1, n)
    bu = torch.zeros(n + 1, dtype=torch.float64, device=cuda)
    bs = torch.zeros(n + 1, dtype=torch.float64, device=cuda)
    bu[1:] = torch.from_numpy(u).to(cuda)
    for f, g in [(0.5, 0.0), (-1.25, 1.0)]:
        bs[1:] = torch.from_numpy(y0).to(cuda)
        sort_generic(bu[1:], bs[1:], dims, perm, f, g)
        got = bs[1:].cpu().numpy()
        want = O.np_sort(u, dims, perm, f, g, out=y0)
        assert bits_equal(got, want), (f, g, first_mismatch(got, want))


def test_warp_default_rule_10_6(cuda):
    """At 10^6 (10^6 elements) the default plans take the warp kernel for
    transposes of the two stride-1 dims, and match the oracle."""
    dims = (10,) * 6
    n = 10 ** 6
    u = O.seeded_uniform(n, 61)
    y0 = O.seeded_uniform(n, 62)
    du = torch.from_numpy(u).to(cuda)
    kinds = set()
    for perm in perms_of(6, 24, 7):
        kinds.add(plan(dims, perm, 1)["kind"])
        ds = torch.from_numpy(y0.copy()).to(cuda)
        sort_generic(du, ds, dims, perm, -1.0, 1.0)
        got = ds.cpu().numpy()
        want = O.np_sort(u, dims, perm, -1.0, 1.0, out=y0)
        assert bits_equal(got, want), (perm, first_mismatch(got, want))
    assert "warp" in kinds
