"""Generate tests/golden/golden.json from the REFERENCE's own loop nests.

Runs the C code that the reference's emitters write (generate_cfunction in
trunk/generator2.py:48-130 and trunk/generator6.py:61-134, built by
oracle/make_ref.py from the reference checkout) on deterministic inputs and
records the SHA-256 of every output.  The committed JSON is what pins the
oracle (tests/test_oracle.py) and the GPU kernels
(tests/test_sort_gpu.py::test_golden_digests_all_perms)
to the reference without needing the reference checkout at test time.

Cases (every permutation; small shapes that hit odd extents and unit dims):
  * rank 4, dims (3,5,4,7) and (2,1,9,4): 24 perms x factors {1, -1, 37, 0.5, -0.5}
    x {sort, sortacc}, plus the tester's integer fixture (init_4d_array,
    trunk/tester_futil.F:139-159) with factors {1, 37} (trunk/generator2.py:488).
  * rank 6, dims (2,3,2,3,2,2): 720 perms x factors {1, -0.5} x {sort, sortacc}
    and the integer fixture (init_6d_array, trunk/tester_futil.F:161-185).
Inputs come from oracle.fixture_values (splitmix64, exact in binary64) so the
same bytes are produced on any machine.

The factor-0.5 cases rely on the generated-artefact patch documented in
oracle/make_ref.py (the emitters truncate factors to int).

Usage: python tests/golden/make_golden.py  (needs the reference checkout)
"""
from __future__ import annotations

import itertools
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import numpy as np  # noqa: E402

from oracle import oracle as O  # noqa: E402
from oracle import refnests as R  # noqa: E402

CASES4 = [((3, 5, 4, 7), (1.0, -1.0, 37.0, 0.5, -0.5)), ((2, 1, 9, 4), (1.0, -0.5))]
CASES6 = [((2, 3, 2, 3, 2, 2), (1.0, -0.5))]


def inputs(dims, tag):
    n = int(np.prod(dims))
    return O.fixture_values(n, 1000 + tag), O.fixture_values(n, 2000 + tag)


def run_ref(perm, dims, u, s0, f, g):
    s = s0.copy() if g else np.zeros_like(u)
    loops = R.loops_for(len(dims), perm)
    R.call(perm, loops[0], u, s, dims, f, g)
    return s


def main():
    if R.load() is None:
        raise SystemExit("reference nests unavailable (need the reference checkout)")
    out = {"generator": "tests/golden/make_golden.py",
           "key": "dims|input|perm|factor|acc_factor -> first 16 hex of sha256(output)",
           "cases": {}}

    def add(dims, inp, perm, f, g, s):
        key = "%s|%s|%s|%r|%r" % (",".join(map(str, dims)), inp, "".join(map(str, perm)), f, g)
        out["cases"][key] = O.digest(s)[:16]

    for tag, (dims, factors) in enumerate(CASES4):
        u, s0 = inputs(dims, tag)
        for perm in itertools.permutations((1, 2, 3, 4)):
            for f in factors:
                for g in (0.0, 1.0):
                    s = run_ref(perm, dims, u, s0, f, g)
                    add(dims, "fixture%d" % tag, perm, f, g, s)
        ui = O.init_array(dims)
        for perm in itertools.permutations((1, 2, 3, 4)):
            for f in (1.0, 37.0):
                s = run_ref(perm, dims, ui, np.zeros_like(ui), f, 0.0)
                add(dims, "init_array", perm, f, 0.0, s)
    for tag, (dims, factors) in enumerate(CASES6, start=10):
        u, s0 = inputs(dims, tag)
        ui = O.init_array(dims)
        for perm in itertools.permutations((1, 2, 3, 4, 5, 6)):
            for f in factors:
                for g in (0.0, 1.0):
                    s = run_ref(perm, dims, u, s0, f, g)
                    add(dims, "fixture%d" % tag, perm, f, g, s)
            s = run_ref(perm, dims, ui, np.zeros_like(ui), 1.0, 0.0)
            add(dims, "init_array", perm, 1.0, 0.0, s)
    path = os.path.join(HERE, "golden.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=0, sort_keys=True)
    print(path, len(out["cases"]), "cases")


if __name__ == "__main__":
    main()
