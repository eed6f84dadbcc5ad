"""Fused sortaccs (spaghetty_sortacc_fused): the nine CCSD(T) triples
sortaccs of each group in branches/spaghetty2/ccsd_t_tce_sort_list.txt
applied to one t3 tile in one kernel, bit-identical to applying them one
after another (the oracle's sequential old_sortacc_6 chain)."""
import random

import numpy as np
import pytest

from oracle import oracle as O
from spaghetty_gb300.workloads import TRIPLES_SORTACC6
from tests._util import bits_equal, first_mismatch

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def source_shape(out_shape, perm):
    # permute(x, p) has out.shape[q] = x.shape[p_q - 1]
    shp = [0] * len(perm)
    for q, p in enumerate(perm):
        shp[p - 1] = out_shape[q]
    return tuple(shp)


def run_group(cuda, out_shape, perms, factors, seed, share=False):
    from spaghetty_gb300 import sortacc_fused
    n = int(np.prod(out_shape))
    t3 = O.fixture_values(n, seed)
    srcs_h = []
    for k, p in enumerate(perms):
        if share and k > 0 and source_shape(out_shape, p) == source_shape(out_shape, perms[0]):
            srcs_h.append(srcs_h[0])
        else:
            srcs_h.append(O.fixture_values(n, seed + 100 + k))
    want = t3.copy()
    for x, p, f in zip(srcs_h, perms, factors):
        want = O.np_sort(x, source_shape(out_shape, p), p, f, 1.0, out=want)
    dsrc = [torch.from_numpy(x).to(cuda).reshape(source_shape(out_shape, p))
            for x, p in zip(srcs_h, perms)]
    dout = torch.from_numpy(t3.copy()).to(cuda).reshape(out_shape)
    sortacc_fused(dout, dsrc, perms, factors)
    got = dout.cpu().numpy().reshape(-1)
    assert bits_equal(got, want), (out_shape, first_mismatch(got, want))


@pytest.mark.parametrize("group", [0, 1, 2])
def test_triples_groups(cuda, group):
    perms = TRIPLES_SORTACC6[group]
    rnd = random.Random(group)
    factors = [rnd.choice([1.0, -1.0]) for _ in perms]
    run_group(cuda, (8, 10, 6, 8, 10, 6), perms, factors, 10 * group)
    run_group(cuda, (16, 16, 16, 16, 16, 16), perms, factors, 10 * group + 3)


def test_general_factors_odd_extents_and_rank4(cuda):
    rnd = random.Random(7)
    perms6 = TRIPLES_SORTACC6[1][:5]
    run_group(cuda, (5, 7, 3, 9, 2, 11), perms6, [rnd.uniform(-2, 2) for _ in perms6], 500)
    perms4 = [(4, 3, 2, 1), (2, 1, 4, 3), (1, 2, 3, 4), (3, 4, 1, 2)]
    run_group(cuda, (30, 30, 30, 30), perms4, [0.5, -1.0, 0.3, 1.0], 600)
    run_group(cuda, (17, 29, 6, 10), [(1, 2, 3, 4), (1, 2, 4, 3)], [0.25, -0.75], 700)


def test_shared_source(cuda):
    perms = [TRIPLES_SORTACC6[0][0]] * 3 + list(TRIPLES_SORTACC6[0][1:4])
    run_group(cuda, (10, 12, 8, 10, 12, 8), perms, [1.0, -1.0, 0.5, 1.0, 1.0, -1.0], 800, share=True)


@pytest.mark.parametrize("group", [0, 2])
def test_triples_partial_boxes(cuda, group):
    """Shapes whose TMA boxes (16 along the sources' stride-1 dim, up to 64
    along the output's) end in partial boxes, and an odd extent that sends
    some passes to the cp.async kernel."""
    perms = TRIPLES_SORTACC6[group]
    rnd = random.Random(40 + group)
    factors = [rnd.choice([1.0, -1.0, 0.5]) for _ in perms]
    run_group(cuda, (20, 12, 18, 20, 12, 18), perms, factors, 900 + group)
    run_group(cuda, (18, 6, 20, 18, 6, 19), perms, factors, 950 + group)


def run_sort_group(cuda, out_shape, perms, factors, seed, same_source=False):
    """spaghetty_sort_fused: the first term overwrites (as tce_sort), the
    rest accumulate (as tce_sortacc); the output starts as NaN garbage,
    which must never be read, and the first source holds signed zeros."""
    from spaghetty_gb300 import sort_fused
    n = int(np.prod(out_shape))
    srcs_h = []
    for k, p in enumerate(perms):
        if same_source and k > 0:
            srcs_h.append(srcs_h[0])
            continue
        x = O.fixture_values(n, seed + 100 + k)
        if k == 0:
            x[::7] = -0.0
        srcs_h.append(x)
    want = O.np_sort(srcs_h[0], source_shape(out_shape, perms[0]), perms[0], factors[0], 0.0)
    for x, p, f in zip(srcs_h[1:], perms[1:], factors[1:]):
        want = O.np_sort(x, source_shape(out_shape, p), p, f, 1.0, out=want)
    dsrc = [torch.from_numpy(x).to(cuda).reshape(source_shape(out_shape, p))
            for x, p in zip(srcs_h, perms)]
    dout = torch.full(out_shape, float("nan"), dtype=torch.float64, device=cuda)
    sort_fused(dout, dsrc, perms, factors)
    got = dout.cpu().numpy().reshape(-1)
    assert bits_equal(got, want), (out_shape, first_mismatch(got, want))


@pytest.mark.parametrize("group", [0, 1, 2])
def test_sort_fused_first_term_overwrites(cuda, group):
    perms = TRIPLES_SORTACC6[group]
    rnd = random.Random(60 + group)
    factors = [1.0] + [rnd.choice([1.0, -1.0, 0.5, -0.3]) for _ in perms[1:]]
    run_sort_group(cuda, (8, 10, 6, 8, 10, 6), perms, factors, 70 * group)
    run_sort_group(cuda, (16, 16, 16, 16, 16, 16), perms, factors, 70 * group + 5)
    # a lone term is a plain sort (signed zeros kept)
    run_sort_group(cuda, (8, 10, 6, 8, 10, 6), perms[:1], [1.0], 70 * group + 9)


@pytest.mark.parametrize("shape", [(24, 24, 24, 24), (12, 12, 12, 12, 12, 12), (46, 46, 46, 46)])
def test_sort_fused_repeated_source(cuda, shape):
    """The differentiable sort's pattern: one source under several perms
    whose stride-1 indices differ (one cp.async pass for L2-sized outputs,
    TMA passes above 2^22 elements)."""
    r = len(shape)
    perms = [tuple(range(r, 0, -1)), tuple([2, 1] + list(range(3, r + 1))),
             tuple(list(range(2, r + 1)) + [1])]
    run_sort_group(cuda, shape, perms, [0.75, -1.25, 0.3], 31 + r, same_source=True)
