"""Differentiable tensor sorts.

``permute_sum(x, perms, factors)`` computes y = sum_k f_k * permute_k(x)
with the rounding of one sort followed by sortaccs, in k order (each term's
product rounded, then each sum rounded), in ONE fused kernel launch
(spaghetty_sort_fused: x read once per term, y written once, y never read).
Its backward is the adjoint of a permutation: dx = sum_k f_k *
permute_{p_k^-1}(dy) -- the reference's sortacc (trunk/old_sort.f:512-575)
applied to the incoming gradient -- again one fused launch with the inverse
permutations.  ``permute_k`` follows the reference convention: the output
holds x's index p_q in position q, i.e. ``x.permute(p - 1)`` (1-based p).
Ranks above 6 (or more than 16 terms) run the same arithmetic as one sort
and sortacc launches.
"""
from __future__ import annotations

from typing import Sequence

import torch

from .sort import permuted_shape, sort_fused, sort_generic


def inverse(perm: Sequence[int]) -> tuple:
    inv = [0] * len(perm)
    for q, p in enumerate(perm):
        inv[p - 1] = q + 1
    return tuple(inv)


# (input shape, perms as given) -> (perms as int tuples, output shape,
# inverse perms): checked and derived once per signature, since at small
# sizes the host work of a step is most of its time
_SIGS: dict = {}


def _signature(shape: tuple, perms: tuple):
    key = (shape, perms)
    sig = _SIGS.get(key)
    if sig is None:
        norm = tuple(tuple(int(v) for v in p) for p in perms)
        shapes = {permuted_shape(shape, p) for p in norm}
        if len(shapes) != 1:
            raise ValueError("every permuted shape must agree, got %s" % sorted(shapes))
        if len(_SIGS) > 4096:
            _SIGS.clear()
        sig = _SIGS[key] = (norm, shapes.pop(), tuple(inverse(p) for p in norm))
    return sig


def _chain(x: torch.Tensor, perms, factors, out_shape) -> torch.Tensor:
    """sum_k f_k * permute_k(x) with the rounding of one sort and len-1
    sortaccs: one fused launch where the fused kernels take the rank."""
    y = torch.empty(out_shape, dtype=x.dtype, device=x.device)
    xs = x.contiguous()
    if xs.dim() <= 6 and len(perms) <= 16:
        return sort_fused(y, [xs] * len(perms), perms, factors)
    for k, (p, f) in enumerate(zip(perms, factors)):
        sort_generic(xs, y, tuple(xs.shape), p, float(f), 0.0 if k == 0 else 1.0)
    return y


class PermuteSum(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, perms, factors):
        in_shape = tuple(x.shape)
        perms, out_shape, inv = _signature(in_shape, tuple(tuple(p) for p in perms))
        factors = tuple(float(f) for f in factors)
        ctx.inv = inv
        ctx.factors = factors
        ctx.in_shape = in_shape
        return _chain(x, perms, factors, out_shape)

    @staticmethod
    def backward(ctx, dy):
        dx = _chain(dy.contiguous(), ctx.inv, ctx.factors, ctx.in_shape)
        return dx, None, None


def permute_sum(x: torch.Tensor, perms, factors) -> torch.Tensor:
    """y = sum_k factors[k] * x.permute(perms[k] - 1), differentiable."""
    return PermuteSum.apply(x, perms, factors)


def permute(x: torch.Tensor, perm: Sequence[int], factor: float = 1.0) -> torch.Tensor:
    """factor * x.permute(perm - 1) materialised by the GPU kernels,
    differentiable (the backward is the inverse-permutation sort)."""
    return PermuteSum.apply(x, [tuple(perm)], [factor])
