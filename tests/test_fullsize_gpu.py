"""GPU parity at the configurations' full sizes, against the oracle, bit for bit.

* tce_sort_4 at 100^4 (800 MB per tensor): all 24 permutations x factors
  {1, -1, 0.5} x {sort, sortacc}, through the drop-ins on the shipped tune
  table (large plain sorts with f = +-1 run the power-of-two path there, and
  sortaccs with f = -1 the voted sign flip);
* tce_sort_6 at 16^6 and at (12,20,16,20,12,16): all 720 permutations, sort
  (f = -0.5) and sortacc (f = 1);
* tce_sort_6 at 20^6 (512 MB per tensor): the 54 CCSD(T) permutations, sort
  and sortacc;
* the batched configuration's full mix (4096 sorts, rank-4 extents 8..40,
  rank-6 extents 6..20) in one graph-replayed batch, with a seeded sample of
  64 sorts checked.

The expected outputs are the oracle's (oracle.np_permuted for the index map
of trunk/old_sort.f:54-58, then numpy's rounded multiply and add as in
old_sort/old_sortacc), computed on the host -- the permutation once per
perm, in a thread pool ahead of the GPU -- uploaded, and compared with the
GPU's output as 64-bit patterns on the device.
"""
import concurrent.futures as cf
import itertools
import random

import numpy as np
import pytest

from oracle import oracle as O
from spaghetty_gb300._lib import lib
from spaghetty_gb300.workloads import TRIPLES_SORT6, batched_mix
from tests._util import call_dropin

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _permuted_ahead(uh, dims, perms, workers):
    """Yield (perm, O.np_permuted(uh, dims, perm)), computed `workers` ahead
    in threads (numpy's copy loops release the GIL)."""
    with cf.ThreadPoolExecutor(workers) as ex:
        futs = [ex.submit(O.np_permuted, uh, dims, p) for p in perms[:workers]]
        for i, p in enumerate(perms):
            t = futs[i].result()
            futs[i] = None
            if i + workers < len(perms):
                futs.append(ex.submit(O.np_permuted, uh, dims, perms[i + workers]))
            yield p, t


class _Expect:
    """Host-computed expected output, uploaded and compared on the device."""

    def __init__(self, n, cuda):
        self.pin = torch.empty(n, dtype=torch.float64, pin_memory=True)
        self.dev = torch.empty(n, dtype=torch.float64, device=cuda)

    def set(self, t, f, y0=None):
        out = self.pin.numpy()
        np.multiply(t, np.float64(f), out=out)          # x(ia)*s, rounded once
        if y0 is not None:
            np.add(y0, out, out=out)                     # y(ib) + x(ia)*s, rounded once
        self.dev.copy_(self.pin)

    def check(self, got, what):
        a, b = got.view(torch.int64), self.dev.view(torch.int64)
        if not torch.equal(a, b):
            bad = torch.nonzero(a != b)
            i = int(bad[0, 0])
            pytest.fail("%s: %d elements differ, first at %d: got %r want %r"
                        % (what, bad.shape[0], i, float(got[i]), float(self.dev[i])))


def _dropin(acc, du, ds, dims, perm, f):
    name = "tce_sort%s_%d" % ("acc" if acc else "", len(dims))
    call_dropin(name, du.data_ptr(), ds.data_ptr(), dims, perm, f)
    rc = lib().spaghetty_last_error()
    assert rc == 0, (name, dims, perm, f, rc)


def _sweep(cuda, dims, perms, cases, seed, workers):
    """Every perm x (factor, acc) case through the drop-ins, against the oracle."""
    n = int(np.prod(dims))
    uh = O.seeded_uniform(n, seed)
    y0 = O.seeded_uniform(n, seed + 1)
    du = torch.from_numpy(uh).to(cuda)
    dy0 = torch.from_numpy(y0).to(cuda)
    ds = torch.empty_like(du)
    want = _Expect(n, cuda)
    for perm, t in _permuted_ahead(uh, dims, perms, workers):
        for f, acc in cases:
            if acc:
                ds.copy_(dy0)
            _dropin(acc, du, ds, dims, perm, f)
            want.set(t, f, y0 if acc else None)
            want.check(ds, (dims, perm, f, "sortacc" if acc else "sort"))
    del du, dy0, ds, want
    torch.cuda.empty_cache()


def test_sort4_100_every_perm_factor_and_form(cuda):
    cases = [(f, acc) for f in (1.0, -1.0, 0.5) for acc in (False, True)]
    _sweep(cuda, (100,) * 4, list(itertools.permutations((1, 2, 3, 4))), cases, 41, 3)


def test_sort6_16_every_perm(cuda):
    _sweep(cuda, (16,) * 6, list(itertools.permutations(range(1, 7))),
           [(-0.5, False), (1.0, True)], 43, 8)


def test_sort6_noncubic_every_perm(cuda):
    _sweep(cuda, (12, 20, 16, 20, 12, 16), list(itertools.permutations(range(1, 7))),
           [(0.5, False), (1.0, True)], 45, 8)


def test_sort6_20_triples(cuda):
    _sweep(cuda, (20,) * 6, list(TRIPLES_SORT6), [(-1.0, False), (-0.5, True)], 47, 4)


def test_batched_config_mix_sample(cuda):
    """The batched configuration's own mix, all 4096 sorts in one
    graph-replayed batch (about 109 GB of tensors); 64 seeded sorts of it
    checked against the oracle."""
    from spaghetty_gb300.batched import Batch
    mix = batched_mix(4096, seed=2024)
    gen = torch.Generator(device=cuda)
    gen.manual_seed(2024)
    jobs, olds = [], []
    for m in mix:
        k = int(np.prod(m["dims"]))
        u = torch.rand(k, dtype=torch.float64, device=cuda, generator=gen) - 0.5
        s = torch.rand(k, dtype=torch.float64, device=cuda, generator=gen) - 0.5
        jobs.append((u, s, m["dims"], m["perm"], m["factor"], 1.0 if m["acc"] else 0.0))
    rnd = random.Random(64)
    sample = sorted(rnd.sample(range(len(mix)), 64))
    b = Batch(jobs)
    b.capture()                 # runs the batch once (warm-up) before capturing it
    torch.cuda.synchronize()
    olds = {i: jobs[i][1].cpu().numpy() for i in sample if mix[i]["acc"]}
    b.replay()
    assert b.status() == 0
    torch.cuda.synchronize()
    for i in sample:
        u, s, dims, perm, f, g = jobs[i]
        want = O.np_sort(u.cpu().numpy(), dims, perm, f, g, out=olds.get(i))
        got = s.cpu().numpy()
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (i, dims, perm, f, g)
    b.close()
    del jobs, b
    torch.cuda.empty_cache()
