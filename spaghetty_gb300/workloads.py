"""Workload descriptions: the CCSD(T) permutation lists and the seeded
synthetic configurations the tests and the benchmark run.

The permutation lists are the reference's data:
  * TRIPLES_SORT6 -- the 54 TCE_SORT_6 permutations NWChem's perturbative
    triples code calls (background/nwchem-perturbative-triples-usage:5-58;
    the same list plus identity is trunk/generator6.py:15-17).
  * TRIPLES_SORTACC6 -- the 27 sortacc permutations applied to triples tiles,
    three groups of nine in call order
    (branches/spaghetty2/ccsd_t_tce_sort_list.txt:1-27).
No public benchmark or dataset is involved: the sizes below are the seeded
synthetic stand-ins for NWChem tile traffic (README.md:30-34 of the
reference: CCSD tiles ~30, up to 100; CCSD(T) ~20).
"""
from __future__ import annotations

import itertools
import random

_TRIPLES_TEXT = """
261543 265431 326541 362154 362514 362541 421653 431652 432165 432651
436215 436251 436521 463215 463251 463521 521643 531642 532164 532641
541632 542136 542163 542631 543162 543216 543261 543621 621543 625431
631542 632154 632514 632541 641532 642153 642531 643152 643215 643251
643521 651432 652143 652413 652431 653142 653214 653241 653421 654132
654213 654231 654312 654321
"""
TRIPLES_SORT6 = [tuple(int(c) for c in w) for w in _TRIPLES_TEXT.split()]

_SORTACC_TEXT = """
326154 326514 326541 362154 362514 362541 365241 365214 365421
436215 436251 436521 463215 463251 463521 643215 643251 643521
653214 653241 653421 635214 635241 635421 632154 632514 632541
"""
_acc = [tuple(int(c) for c in w) for w in _SORTACC_TEXT.split()]
TRIPLES_SORTACC6 = [_acc[0:9], _acc[9:18], _acc[18:27]]

PERMS4 = list(itertools.permutations((1, 2, 3, 4)))
PERMS6 = list(itertools.permutations((1, 2, 3, 4, 5, 6)))

# tce_sort_4 sweep: sizes and factors of the sweep configuration
SORT4_DIMS = [(20,) * 4, (30,) * 4, (50,) * 4, (100,) * 4, (17, 29, 64, 100)]
SORT4_FACTORS = (1.0, -1.0, 0.5)
# tce_sort_6 sweep
SORT6_DIMS = [(10,) * 6, (16,) * 6, (20,) * 6, (12, 20, 16, 20, 12, 16)]


def batched_mix(n: int = 4096, seed: int = 2024, frac4: float = 0.7,
                ext4=(8, 40), ext6=(6, 20)):
    """Seeded list of n sort jobs: 70% rank 4 with extents uniform in [8,40],
    30% rank 6 with extents uniform in [6,20]; random permutation, factor
    uniform(-1,1), half sort and half sortacc."""
    rnd = random.Random(seed)
    jobs = []
    for _ in range(n):
        if rnd.random() < frac4:
            dims = tuple(rnd.randint(*ext4) for _ in range(4))
            perm = list(range(1, 5))
        else:
            dims = tuple(rnd.randint(*ext6) for _ in range(6))
            perm = list(range(1, 7))
        rnd.shuffle(perm)
        f = rnd.uniform(-1.0, 1.0)
        acc = rnd.random() < 0.5
        jobs.append({"dims": dims, "perm": tuple(perm), "factor": f, "acc": acc})
    return jobs
