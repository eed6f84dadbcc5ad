"""Seeded random problems across every kernel the planner can pick: ranks 2
to 8, random extents (odd ones included), random permutations, every
factor class (1, -1, +-2^k, any other value, the general acc_factor),
sort and sortacc, device buffers aligned and offset by one element (no
bulk tensor copies then), against the oracle bit for bit.  The plan kinds
the cases reached are checked too, so that the sample keeps covering the
flat, direct, tiled, TMA-staged and warp-shuffle kernels."""
import random

import numpy as np
import pytest

from oracle import oracle as O
from spaghetty_gb300 import plan, sort_generic
from tests._util import bits_equal, first_mismatch

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FACTORS = [(1.0, 0.0), (-1.0, 0.0), (0.5, 0.0), (-4.0, 0.0), (0.3, 0.0), (1.0, 1.0),
           (-1.0, 1.0), (0.25, 1.0), (-1.7, 1.0), (0.6, -2.0)]


def cases(seed, n):
    rnd = random.Random(seed)
    out = []
    for _ in range(n):
        r = rnd.choice((2, 3, 4, 4, 5, 6, 6, 7, 8))
        cap = {2: 600, 3: 90, 4: 40, 5: 18, 6: 12, 7: 8, 8: 6}[r]
        dims = [rnd.randint(1, cap) for _ in range(r)]
        while int(np.prod(dims)) > 400_000:
            dims[rnd.randrange(r)] //= 2
            dims = [max(1, d) for d in dims]
        perm = list(range(1, r + 1))
        rnd.shuffle(perm)
        out.append((tuple(dims), tuple(perm), rnd.choice(FACTORS), rnd.random() < 0.25))
    return out


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_problems_bits(cuda, seed):
    kinds = set()
    for dims, perm, (f, g), offset in cases(seed, 120):
        n = int(np.prod(dims))
        rng = np.random.default_rng(n * 7 + len(dims))
        u = rng.uniform(-1, 1, n)
        y0 = rng.uniform(-1, 1, n)
        bu = torch.zeros(n + 1, dtype=torch.float64, device=cuda)
        bs = torch.zeros(n + 1, dtype=torch.float64, device=cuda)
        o = 1 if offset else 0
        bu[o:o + n] = torch.from_numpy(u).to(cuda)
        bs[o:o + n] = torch.from_numpy(y0).to(cuda)
        sort_generic(bu[o:o + n], bs[o:o + n], dims, perm, f, g)
        got = bs[o:o + n].cpu().numpy()
        with np.errstate(all="ignore"):
            want = O.np_sort(u, dims, perm, f, g, out=y0)
        assert bits_equal(got, want), (dims, perm, f, g, offset, first_mismatch(got, want))
        if not offset:
            kinds.add(plan(dims, perm, 0 if g == 0.0 else (1 if g == 1.0 else 2))["kind"])
    assert {"tiled", "tma", "warp"} <= kinds, kinds
