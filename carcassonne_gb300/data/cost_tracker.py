"""Static cost model: a fake Data object that counts complex multiply-adds.

Restates carcassonne/data/cost_tracker.py:8-39.  The counts define the
algorithmic work that throughput figures are quoted on, and they drive
Multiplier.isCheaperToFormMatrix exactly as in the reference.
"""
from __future__ import annotations

import numpy as np

from . import Data


class CostTracker(Data):
    def __init__(self, shape, cost=0):
        self.shape = tuple(int(x) for x in shape)
        self.ndim = len(self.shape)
        self.cost = int(cost)

    def __repr__(self):
        return "CostTracker({},{})".format(self.shape, self.cost)

    def contractWith(self, other, self_axes, other_axes):
        self_axes, other_axes = list(self_axes), list(other_axes)
        shape = tuple(x for i, x in enumerate(self.shape) if i not in self_axes) + \
            tuple(x for i, x in enumerate(other.shape) if i not in other_axes)
        summed = int(np.prod([x for i, x in enumerate(self.shape) if i in self_axes], dtype=np.int64))
        cost = self.cost + other.cost + int(np.prod(shape, dtype=np.int64)) * summed
        return CostTracker(shape, cost)

    def extractScalar(self):
        assert len(self.shape) == 0
        return self

    def transpose(self, *perm):
        perm = perm[0] if len(perm) == 1 and isinstance(perm[0], (tuple, list)) else perm
        return CostTracker(tuple(self.shape[i] for i in perm), self.cost)

    def join(self, *groups):
        groups = [[g] if isinstance(g, (int, np.integer)) else list(g) for g in groups]
        return CostTracker(tuple(int(np.prod([self.shape[i] for i in g], dtype=np.int64)) for g in groups), self.cost)


def computeCostOfContracting(contractor, *tensors):
    return contractor(*(CostTracker(t.shape) if not isinstance(t, tuple) else CostTracker(t) for t in tensors)).cost


def stage3_multiply_cost(s0_shape, s1_shape, d, identity_op):
    """Cost of formDenseStage3 / formNormalizationStage3 multiply (tensors/_2d/dense.py:114-174)
    as the reference's CostTracker counts it on the joined stage-2 tensors."""
    x = s0_shape[0] * s0_shape[1]
    k0, k1, l0, l1 = s0_shape[2:6]
    k2, k3, l2, l3 = s1_shape[2:6]
    c = x * l0 * l1 * k0 * k1 * k2 * k3 * d + x * l0 * l1 * l2 * l3 * k2 * k3 * d
    if not identity_op:
        c += k0 * k1 * k2 * k3 * d * d
    return int(c)


def stage3_form_matrix_cost(s0_shape, s1_shape, d):
    """Cost of formDenseStage3_formMatrix (tensors/_2d/dense.py:175-195)."""
    x = s0_shape[0] * s0_shape[1]
    k0, k1, l0, l1 = s0_shape[2:6]
    k2, k3, l2, l3 = s1_shape[2:6]
    g = l0 * l1 * k0 * k1 * l2 * l3 * k2 * k3
    return int(g * x + g * d * d)


__all__ = ["CostTracker", "computeCostOfContracting", "stage3_multiply_cost", "stage3_form_matrix_cost"]
