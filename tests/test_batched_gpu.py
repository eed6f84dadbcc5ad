"""Batched persistent kernel through the C ABI: bit-exact against the oracle
and against the one-launch-per-sort path, CUDA-graph replay, and host-side
fault injection (a poisoned work-list entry is flagged, skipped, and leaves
every other sort correct)."""
import random

import numpy as np
import pytest

from oracle import oracle as O
from spaghetty_gb300 import plan
from spaghetty_gb300._lib import lib
from spaghetty_gb300.workloads import batched_mix
from tests._util import bits_equal, first_mismatch

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def make_jobs(specs, cuda, seed=0):
    """Device tensors + host copies for a list of job specs."""
    jobs, host = [], []
    for i, sp in enumerate(specs):
        n = int(np.prod(sp["dims"]))
        u = O.fixture_values(n, seed + 2 * i)
        y = O.fixture_values(n, seed + 2 * i + 1)
        du = torch.from_numpy(u).to(cuda)
        ds = torch.from_numpy(y).to(cuda)
        g = sp.get("g", 1.0 if sp.get("acc") else 0.0)
        jobs.append((du, ds, sp["dims"], sp["perm"], sp["factor"], g))
        host.append((u, y, g))
    return jobs, host


def small_specs(n, seed):
    rnd = random.Random(seed)
    specs = []
    for _ in range(n):
        if rnd.random() < 0.7:
            dims = tuple(rnd.randint(3, 13) for _ in range(4))
        else:
            dims = tuple(rnd.randint(2, 6) for _ in range(6))
        perm = list(range(1, len(dims) + 1))
        rnd.shuffle(perm)
        g = rnd.choice([0.0, 1.0, 1.0, -0.75])
        specs.append({"dims": dims, "perm": tuple(perm), "factor": rnd.uniform(-1, 1), "g": g})
    return specs


def expect(spec, u, y, g, times=1):
    out = y
    for _ in range(times):
        out = O.np_sort(u, spec["dims"], spec["perm"], spec["factor"], g, out=out)
    return out


def test_batched_matches_oracle(cuda):
    from spaghetty_gb300.batched import Batch
    specs = small_specs(160, 1)
    jobs, host = make_jobs(specs, cuda, 100)
    b = Batch(jobs)
    info = b.info()
    assert info["jobs"] == 160 and info["units"] >= 160
    b.launch()
    assert b.status() == 0
    for sp, (du, ds, *_), (u, y, g) in zip(specs, jobs, host):
        got = ds.cpu().numpy()
        want = expect(sp, u, y, g)
        assert bits_equal(got, want), (sp, first_mismatch(got, want))


def test_batched_equals_plain_and_graph_replay(cuda):
    from spaghetty_gb300.batched import Batch
    specs = small_specs(96, 2)
    jobs_a, host = make_jobs(specs, cuda, 300)
    jobs_b, _ = make_jobs(specs, cuda, 300)
    ba = Batch(jobs_a)
    bb = Batch(jobs_b)
    ba.capture()            # warm-up launch inside capture() runs once
    ba.replay()             # ... and the replay a second time
    bb.launch_plain()
    bb.launch_plain()
    assert ba.status() == 0
    torch.cuda.synchronize()
    for sp, ja, jb, (u, y, g) in zip(specs, jobs_a, jobs_b, host):
        a = ja[1].cpu().numpy()
        assert bits_equal(a, jb[1].cpu().numpy()), sp
        assert bits_equal(a, expect(sp, u, y, g, times=2)), sp


def test_poisoned_entry_is_flagged_and_skipped(cuda):
    from spaghetty_gb300.batched import Batch
    specs = small_specs(40, 3)
    jobs, host = make_jobs(specs, cuda, 500)
    b = Batch(jobs)
    b.poison(7)
    b.launch()
    assert b.status() == 11          # SPAGHETTY_ERR_DEVICE
    assert b.status() == 0           # the status word was cleared by the read
    for i, (sp, (du, ds, *_), (u, y, g)) in enumerate(zip(specs, jobs, host)):
        got = ds.cpu().numpy()
        if i == 7:
            assert bits_equal(got, y)        # untouched
        else:
            assert bits_equal(got, expect(sp, u, y, g)), i


def test_invalid_entries_rejected_on_host(cuda):
    from spaghetty_gb300 import SpaghettyError
    from spaghetty_gb300.batched import Batch
    a = torch.zeros(16, dtype=torch.float64, device=cuda)
    c = torch.zeros(16, dtype=torch.float64, device=cuda)
    with pytest.raises(SpaghettyError) as ei:
        Batch([(a, c, (2, 2, 2, 2), (1, 2, 3, 4), 1.0, 0.0),
               (a, c, (2, 2, 2, 2), (1, 1, 3, 4), 1.0, 0.0)])
    assert ei.value.code == 2 and "entry 1" in str(ei.value)
    with pytest.raises(SpaghettyError) as ei:           # two outputs overlap
        Batch([(a, c, (2, 2, 2, 2), (2, 1, 3, 4), 1.0, 0.0),
               (a, c, (2, 2, 2, 2), (4, 3, 2, 1), 1.0, 0.0)])
    assert ei.value.code == 6
    h = torch.zeros(16, dtype=torch.float64)
    with pytest.raises(SpaghettyError) as ei:           # host pointer
        Batch([(h, c, (2, 2, 2, 2), (2, 1, 3, 4), 1.0, 0.0)])
    assert ei.value.code == 8


def test_shared_input_is_allowed(cuda):
    """The nine triples sortaccs read different sources, but one source may
    feed several sorts: inputs may be shared, outputs may not."""
    from spaghetty_gb300.batched import Batch
    dims = (5, 6, 4, 7, 3, 5)
    n = int(np.prod(dims))
    u = O.fixture_values(n, 900)
    du = torch.from_numpy(u).to(cuda)
    perms = [(3, 2, 6, 1, 5, 4), (6, 5, 4, 3, 2, 1), (2, 6, 1, 5, 4, 3)]
    outs = [torch.zeros(n, dtype=torch.float64, device=cuda) for _ in perms]
    b = Batch([(du, o, dims, p, -0.5, 0.0) for o, p in zip(outs, perms)])
    b.launch()
    assert b.status() == 0
    for o, p in zip(outs, perms):
        assert bits_equal(o.cpu().numpy(), O.np_sort(u, dims, p, -0.5))


def test_mix_4096_reduced_extents(cuda):
    """The batched configuration's shape (4096 sorts, 70% rank 4 / 30% rank 6,
    random perms and factors, half sortacc) at reduced extents: batched ==
    plain bitwise on every sort, and 64 sorts checked against the oracle."""
    from spaghetty_gb300.batched import Batch
    mix = batched_mix(4096, seed=11, ext4=(4, 14), ext6=(3, 7))
    specs = [{"dims": m["dims"], "perm": m["perm"], "factor": m["factor"],
              "g": 1.0 if m["acc"] else 0.0} for m in mix]
    ja, host = make_jobs(specs, cuda, 7000)
    jb = [(u, s.clone(), d, p, f, g) for (u, s, d, p, f, g) in ja]
    Batch(ja).launch()
    pb = Batch(jb)
    pb.launch_plain()
    torch.cuda.synchronize()
    for x, y in zip(ja, jb):
        assert torch.equal(x[1], y[1])
    rnd = random.Random(5)
    for i in rnd.sample(range(4096), 64):
        u, y, g = host[i]
        assert bits_equal(ja[i][1].cpu().numpy(), expect(specs[i], u, y, g)), i


@pytest.mark.parametrize("rule", [(8, 8, 256), (64, 16, 1024), (16, 64, 512)])
def test_size_bucket_rules(cuda, rule):
    """Tuned per-size-bucket tile shapes (spaghetty_batch_tune_set) change
    the boxes, never the bits."""
    from spaghetty_gb300._lib import lib
    from spaghetty_gb300.batched import Batch
    L = lib()
    specs = small_specs(96, 5)
    jobs, host = make_jobs(specs, cuda, 300)
    try:
        assert L.spaghetty_batch_tune_set(4, 1, 64, *rule) == 0
        assert L.spaghetty_batch_tune_set(6, 1, 64, *rule) == 0
        b = Batch(jobs)
        b.launch()
        assert b.status() == 0
        b.close()
    finally:
        L.spaghetty_batch_tune_set(0, 0, 0, 0, 0, 0)
    for sp, (du, ds, *_), (u, y, g) in zip(specs, jobs, host):
        got = ds.cpu().numpy()
        want = expect(sp, u, y, g)
        assert bits_equal(got, want), (sp, rule, first_mismatch(got, want))


OPT_BATCH_OWN_MIN = 5
OWN_MIN_DEFAULT = 1 << 24


def test_large_sorts_run_as_their_own_launches(cuda):
    """Large sorts (SPAGHETTY_OPT_BATCH_OWN_MIN = 2^22 elements and more
    here) that the single-sort planner puts on the TMA-staged kernel leave
    the work list and run as their own launches inside the same launch (and
    the same captured graph); every sort still matches the oracle.  At the
    default threshold (2^24) the same sorts stay on the work list."""
    from spaghetty_gb300.batched import Batch
    L = lib()
    assert L.spaghetty_set_option(OPT_BATCH_OWN_MIN, 1 << 22) == 0
    try:
        _own_launches(cuda, Batch)
    finally:
        L.spaghetty_set_option(OPT_BATCH_OWN_MIN, OWN_MIN_DEFAULT)


def _own_launches(cuda, Batch):
    specs = small_specs(40, 9)
    big = [{"dims": (64, 40, 40, 48), "perm": (2, 4, 3, 1), "factor": -0.5, "g": 0.0},
           {"dims": (16, 12, 12, 16, 8, 16), "perm": (6, 5, 4, 3, 2, 1), "factor": 1.0, "g": 1.0},
           {"dims": (40, 64, 48, 40), "perm": (1, 3, 2, 4), "factor": 0.75, "g": -0.25},
           # odd extents only: no bulk tensor copy can describe its rows,
           # so it is planned on another kernel and stays on the work list
           {"dims": (15, 17, 13, 11, 9, 13), "perm": (3, 2, 6, 1, 5, 4), "factor": 1.0, "g": 1.0}]
    specs = specs[:20] + big + specs[20:]
    jobs, host = make_jobs(specs, cuda, 400)
    b = Batch(jobs)
    info = b.info()
    opclass = {0.0: 0, 1.0: 1}
    direct = [sp for sp in big if int(np.prod(sp["dims"])) >= 1 << 22 and
              plan(sp["dims"], sp["perm"], opclass.get(sp["g"], 2))["kind"] == "tma"]
    assert len(direct) == 3 and big[3] not in direct
    assert info["jobs"] == 44 - len(direct) and info["launches"] == len(direct) + 1
    lib().spaghetty_set_option(OPT_BATCH_OWN_MIN, OWN_MIN_DEFAULT)
    dflt = Batch(jobs)              # planned only: nothing above 2^24 elements
    assert dflt.info()["jobs"] == 44 and dflt.info()["launches"] == 1
    dflt.close()
    lib().spaghetty_set_option(OPT_BATCH_OWN_MIN, 1 << 22)
    b.capture()          # warm-up launch, then capture
    b.replay()           # the sorts ran twice: sortaccs accumulate twice
    assert b.status() == 0
    for sp, (du, ds, *_), (u, y, g) in zip(specs, jobs, host):
        got = ds.cpu().numpy()
        want = expect(sp, u, y, g, times=2)
        assert bits_equal(got, want), (sp, first_mismatch(got, want))


OPT_BATCH_OWN_KINDS = 6


def test_own_launches_of_every_plan_kind(cuda):
    """With SPAGHETTY_OPT_BATCH_OWN_KINDS = 1 the large sorts leave the work
    list whatever their single-sort plan (here also an odd-extent sort on the
    register-staged kernel and one that keeps its stride-1 index); the batch
    still matches the oracle, replayed from a graph."""
    from spaghetty_gb300.batched import Batch
    L = lib()
    specs = small_specs(24, 17)
    big = [{"dims": (15, 17, 13, 11, 9, 13), "perm": (3, 2, 6, 1, 5, 4), "factor": 0.3, "g": 1.0},
           {"dims": (40, 33, 21, 41), "perm": (3, 1, 2, 4), "factor": -1.0, "g": 0.0},
           {"dims": (64, 40, 40, 48), "perm": (2, 4, 3, 1), "factor": 0.5, "g": 0.0}]
    specs = specs[:12] + big + specs[12:]
    jobs, host = make_jobs(specs, cuda, 500)
    assert L.spaghetty_set_option(OPT_BATCH_OWN_MIN, 1 << 20) == 0
    assert L.spaghetty_set_option(OPT_BATCH_OWN_KINDS, 1) == 0
    try:
        b = Batch(jobs)
    finally:
        L.spaghetty_set_option(OPT_BATCH_OWN_MIN, OWN_MIN_DEFAULT)
        L.spaghetty_set_option(OPT_BATCH_OWN_KINDS, 0)
    big_n = [sp for sp in specs if int(np.prod(sp["dims"])) >= 1 << 20]
    info = b.info()
    assert len(big_n) >= 3
    assert info["jobs"] == len(specs) - len(big_n) and info["launches"] == len(big_n) + 1
    b.capture()
    b.replay()
    assert b.status() == 0
    for sp, (du, ds, *_), (u, y, g) in zip(specs, jobs, host):
        got = ds.cpu().numpy()
        want = expect(sp, u, y, g, times=2)
        assert bits_equal(got, want), (sp, first_mismatch(got, want))
    b.close()
