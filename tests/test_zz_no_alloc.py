"""The no-allocation batched entry point, spaghetty_sort_batch_noalloc.

It is meant for callers that cannot allocate device memory (code running
while a CUDA graph is being captured, or inside an application that owns the
device memory budget): its work list lives in a fixed device array inside the
library.  Checked here through the C ABI against the allocating batched entry
point (spaghetty_batch_create + spaghetty_batch_launch) on two calls in a
row with different sorts, bit for bit -- the tolerance of every parity test
in this suite -- so a stale work list left in the shared array by the first
call would show up in the second.  This file is collected last on purpose.
"""
import ctypes
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _specs(seed, n):
    rnd = random.Random(seed)
    out = []
    for _ in range(n):
        if rnd.random() < 0.7:
            dims = tuple(rnd.randint(3, 17) for _ in range(4))
        else:
            dims = tuple(rnd.randint(2, 7) for _ in range(6))
        perm = list(range(1, len(dims) + 1))
        rnd.shuffle(perm)
        out.append((dims, tuple(perm), rnd.uniform(-1, 1), rnd.choice([0.0, 1.0, -0.5])))
    return out


def _entries(specs, ins, outs):
    from spaghetty_gb300._lib import BatchEntry
    arr = (BatchEntry * len(specs))()
    for e, (dims, perm, f, g), u, s in zip(arr, specs, ins, outs):
        e.unsorted = u.data_ptr()
        e.sorted = s.data_ptr()
        e.rank = len(dims)
        for q, d in enumerate(dims):
            e.dims[q] = d
        for q, p in enumerate(perm):
            e.perm[q] = p
        e.factor = f
        e.acc_factor = g
    return arr


def _run_both(cuda, seed, n):
    from spaghetty_gb300._lib import lib
    L = lib()
    specs = _specs(seed, n)
    gen = torch.Generator(device=cuda)
    gen.manual_seed(seed)
    ins, out_ref, out_new = [], [], []
    for dims, _, _, _ in specs:
        k = int(np.prod(dims))
        ins.append(torch.rand(k, dtype=torch.float64, device=cuda, generator=gen) - 0.5)
        y = torch.rand(k, dtype=torch.float64, device=cuda, generator=gen) - 0.5
        out_ref.append(y.clone())
        out_new.append(y.clone())
    stream = torch.cuda.current_stream().cuda_stream
    # existing entry point (allocates its work list)
    h = ctypes.c_void_p()
    ref = _entries(specs, ins, out_ref)
    assert L.spaghetty_batch_create(ctypes.cast(ref, ctypes.c_void_p), n, ctypes.byref(h)) == 0
    assert L.spaghetty_batch_launch(h, ctypes.c_void_p(stream)) == 0
    assert L.spaghetty_batch_status(h, ctypes.c_void_p(stream)) == 0
    L.spaghetty_batch_destroy(h)
    # the no-allocation entry point
    new = _entries(specs, ins, out_new)
    rc = L.spaghetty_sort_batch_noalloc(ctypes.cast(new, ctypes.c_void_p), n, ctypes.c_void_p(stream))
    assert rc == 0
    torch.cuda.synchronize()
    for a, b, sp in zip(out_ref, out_new, specs):
        assert torch.equal(a, b), sp


def test_noalloc_matches_allocating_entry_two_calls(cuda):
    _run_both(cuda, 101, 96)
    _run_both(cuda, 202, 57)     # different sorts: stale scratch would show


def test_noalloc_rejects_oversized_batch(cuda):
    from spaghetty_gb300._lib import lib
    from spaghetty_gb300._lib import BatchEntry
    arr = (BatchEntry * 1025)()
    rc = lib().spaghetty_sort_batch_noalloc(ctypes.cast(arr, ctypes.c_void_p), 1025, None)
    assert rc == 13
