"""The no-allocation batched entry point, spaghetty_sort_batch_noalloc.

Some callers cannot allocate device memory: an application that has handed
the whole device memory to its own pool allocator, or code that must not
cause the device-wide synchronisation cudaMalloc/cudaFree may trigger while
other streams run.  This entry point keeps its work list in a fixed device
array inside the library instead.  Checked here through the C ABI on two
calls in a row with different sorts, so that a stale work list left in the
shared array by the first call would show up in the second: bit for bit (the
tolerance of every parity test in this suite) against the allocating batched
entry point (spaghetty_batch_create + spaghetty_batch_launch) and against the
oracle.  One test runs the entry point as the first library call of a fresh
process, where it does its per-device set-up.  This file is collected last on
purpose.
"""
import ctypes
import os
import random
import subprocess
import sys

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


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


def _inputs(cuda, specs, seed):
    gen = torch.Generator(device=cuda)
    gen.manual_seed(seed)
    ins, olds = [], []
    for dims, _, _, _ in specs:
        k = int(np.prod(dims))
        ins.append(torch.rand(k, dtype=torch.float64, device=cuda, generator=gen) - 0.5)
        olds.append(torch.rand(k, dtype=torch.float64, device=cuda, generator=gen) - 0.5)
    return ins, olds


def _check_oracle(specs, ins, olds, outs):
    for (dims, perm, f, g), u, y0, got in zip(specs, ins, olds, outs):
        want = O.sort_generic(u.cpu().numpy(), dims, perm, f, g, out=y0.cpu().numpy().copy())
        assert np.array_equal(got.cpu().numpy().view(np.uint64), want.view(np.uint64)), (dims, perm, f, g)


def _run_both(cuda, seed, n):
    from spaghetty_gb300._lib import lib
    L = lib()
    specs = _specs(seed, n)
    ins, olds = _inputs(cuda, specs, seed)
    out_ref = [y.clone() for y in olds]
    out_new = [y.clone() for y in olds]
    stream = torch.cuda.current_stream().cuda_stream
    # the allocating entry point
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
    _check_oracle(specs, ins, olds, out_new)


def test_noalloc_matches_allocating_entry_two_calls(cuda):
    _run_both(cuda, 101, 96)
    _run_both(cuda, 202, 57)     # different sorts: stale scratch would show


def test_noalloc_rejects_oversized_batch(cuda):
    from spaghetty_gb300._lib import lib
    from spaghetty_gb300._lib import BatchEntry
    arr = (BatchEntry * 1025)()
    rc = lib().spaghetty_sort_batch_noalloc(ctypes.cast(arr, ctypes.c_void_p), 1025, None)
    assert rc == 13


_FIRST_CALL = r"""
import sys
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[2])
import torch
import test_zz_no_alloc as T
from spaghetty_gb300._lib import lib
cuda = torch.device("cuda", 0)
for seed, n in ((303, 40), (404, 33)):
    specs = T._specs(seed, n)
    ins, olds = T._inputs(cuda, specs, seed)
    outs = [y.clone() for y in olds]
    arr = T._entries(specs, ins, outs)
    rc = lib().spaghetty_sort_batch_noalloc(T.ctypes.cast(arr, T.ctypes.c_void_p), n,
                                           T.ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, rc
    torch.cuda.synchronize()
    T._check_oracle(specs, ins, olds, outs)
print("first-call ok")
"""


def test_noalloc_first_call_in_fresh_process(cuda):
    """The entry point as the first library call of a process (its per-device
    set-up runs inside it), twice in a row, against the oracle."""
    res = subprocess.run([sys.executable, "-c", _FIRST_CALL, ROOT, os.path.join(ROOT, "tests")],
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "first-call ok" in res.stdout
