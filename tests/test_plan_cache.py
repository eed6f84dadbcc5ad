"""The host planner's cache under load (no GPU needed): plans queried from
several threads at once agree with the same plans queried alone, and a
working set larger than the cache (16384 entries, half dropped when full)
still returns the right plans afterwards."""
import itertools
import random
import threading

from spaghetty_gb300 import plan
from spaghetty_gb300._lib import lib

OPT_WARP_TR = 4


def problems(n, seed):
    rnd = random.Random(seed)
    out = []
    for _ in range(n):
        r = rnd.choice((2, 3, 4, 5, 6))
        dims = tuple(rnd.randint(2, 24) for _ in range(r))
        perm = list(range(1, r + 1))
        rnd.shuffle(perm)
        out.append((dims, tuple(perm), rnd.randint(0, 1)))
    return out


def test_plans_from_many_threads_agree():
    probs = problems(240, 1)
    want = {p: plan(*p) for p in probs}
    errors = []

    def worker(k):
        try:
            rnd = random.Random(k)
            for _ in range(3):
                order = probs[:]
                rnd.shuffle(order)
                for p in order:
                    if plan(*p) != want[p]:
                        errors.append(p)
        except Exception as e:  # noqa: BLE001 -- reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(8)]
    for t in threads:
        t.start()
    # an option change in the middle drops every cached plan
    assert lib().spaghetty_set_option(OPT_WARP_TR, 1) == 0
    for t in threads:
        t.join()
    assert not errors, errors[:5]


def test_cache_eviction_keeps_plans_right():
    first = problems(64, 2)
    want = {p: plan(*p) for p in first}
    # more distinct shapes than the cache holds
    filler = [((a, b, c, d), perm, 0)
              for (a, b, c, d), perm in zip(itertools.product(range(3, 14), range(3, 14), range(3, 14),
                                                                range(3, 17)),
                                            itertools.cycle(itertools.permutations((1, 2, 3, 4))))]
    assert len(filler) > 17000
    for p in filler[:17000]:
        plan(*p)
    for p in first:
        assert plan(*p) == want[p], p
