"""Host-side bookkeeping of the fused and differentiable sorts (CPU only):
the per-signature caches validate shapes once and give back the same
arrays and inverse permutations; bad signatures raise, and are not cached."""
import pytest

torch = pytest.importorskip("torch")

import importlib  # noqa: E402

# the modules themselves (the package re-exports functions of the same names)
S = importlib.import_module("spaghetty_gb300.sort")
A = importlib.import_module("spaghetty_gb300.autograd")


def test_fused_arrays_are_built_once_per_signature():
    shapes = ((2, 3, 4, 5),) * 3
    perms = ((4, 3, 2, 1), (4, 2, 3, 1), (4, 3, 1, 2))
    out = (5, 4, 3, 2)
    with pytest.raises(ValueError):
        S._fused_arrays(shapes, perms, out)      # (4,2,3,1) gives (5,3,4,2)
    perms = ((4, 3, 2, 1), (4, 3, 2, 1), (4, 3, 2, 1))
    a = S._fused_arrays(shapes, perms, out)
    b = S._fused_arrays(shapes, perms, out)
    assert a is b
    rank, dims, pp = a
    assert rank == 4 and list(dims) == [2, 3, 4, 5] * 3 and list(pp) == [4, 3, 2, 1] * 3


def test_fused_arrays_reject_rank_mismatch():
    with pytest.raises(ValueError):
        S._fused_arrays(((2, 3, 4, 5), (2, 3, 4)), ((1, 2, 3, 4), (1, 2, 3)), (2, 3, 4, 5))


def test_fused_rejects_cpu_tensors():
    x = torch.zeros(2, 3, dtype=torch.float64)
    y = torch.zeros(3, 2, dtype=torch.float64)
    with pytest.raises(TypeError):
        S.sort_fused(y, [x], [(2, 1)], [1.0])
    with pytest.raises(ValueError):
        S.sort_fused(y, [x, x], [(2, 1)], [1.0])


def test_autograd_signature_and_inverse():
    norm, out_shape, inv = A._signature((2, 3, 4), ((3, 1, 2), (3, 1, 2)))
    assert norm == ((3, 1, 2), (3, 1, 2)) and out_shape == (4, 2, 3)
    assert inv == ((2, 3, 1), (2, 3, 1))
    for p, q in zip(norm, inv):
        # the inverse undoes the permutation of the shape
        assert S.permuted_shape(S.permuted_shape((2, 3, 4), p), q) == (2, 3, 4)
    assert A._signature((2, 3, 4), ((3, 1, 2), (3, 1, 2))) is A._SIGS[((2, 3, 4), ((3, 1, 2), (3, 1, 2)))]
    with pytest.raises(ValueError):
        A._signature((2, 3, 4), ((3, 1, 2), (1, 2, 3)))
    assert ((2, 3, 4), ((3, 1, 2), (1, 2, 3))) not in A._SIGS
