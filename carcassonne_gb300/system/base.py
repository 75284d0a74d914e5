"""Driver of the center-site path: policies, sweeps and bandwidth increase
(carcassonne/system/base.py:15-160), unchanged in behaviour, over the GPU
System.  The loop is host control flow; every step it calls runs on the GPU.
"""
from __future__ import annotations

import logging

from ..utils import O, RelaxFailed, computeNewDimension

log = logging.getLogger(__name__)

POLICY_NAMES = ("bandwidth increase", "contraction", "operator compression", "run convergence",
                "post-contraction hook", "pre-optimization hook", "post-optimization hook", "state compression",
                "sweep convergence")


class BaseSystem:
    def __init__(self):
        self._policies = {name: None for name in POLICY_NAMES}

    # -- policy registry (base.py:15-57, :77-84) ---------------------------
    def _bound(self, name, optional=False):
        if name not in self._policies:
            raise ValueError("No such policy name " + name)
        policy = self._policies[name]
        if policy is None:
            if optional:
                return None
            raise ValueError("Policy " + name + " has not been set.")
        return policy

    def _applyPolicy(self, name, optional=False):
        p = self._bound(name, optional)
        if p is not None:
            p.apply()

    def _hasConverged(self, name):
        return self._bound(name).converged()

    def _resetPolicy(self, name, optional=False):
        p = self._bound(name, optional)
        if p is not None:
            p.reset()

    def _updatePolicy(self, name, optional=False):
        p = self._bound(name, optional)
        if p is not None:
            p.update()

    def setPolicy(self, policy_name, policy):
        if policy_name not in self._policies:
            raise ValueError("No such policy name " + policy_name)
        if self._policies[policy_name] is not None:
            raise ValueError("Policy " + policy_name + " has already been set.")
        self._policies[policy_name] = policy.createBindingToSystem(self)

    # -- loops (base.py:58-111) -------------------------------------------
    def computeEstimatedOneSiteExpectation(self, direction=0):
        from copy import copy
        system = copy(self)
        e1 = system.computeExpectation()
        system.contractTowards(direction)
        return system.computeExpectation() - e1

    def runUntilConverged(self):
        log.info("Beginning run.")
        self.number_of_sweeps = 0
        self.number_of_iterations = 0
        self.sweepUntilConverged()
        self._updatePolicy("run convergence")
        while not self._hasConverged("run convergence"):
            self._applyPolicy("bandwidth increase")
            self.sweepUntilConverged()
            self._updatePolicy("run convergence")
        log.info("Finished run with %d total sweeps and %d total iterations.", self.number_of_sweeps,
                 self.number_of_iterations)

    def sweepUntilConverged(self):
        self.number_of_sweeps += 1
        log.info("Starting sweep #%d", self.number_of_sweeps)
        self._resetPolicy("contraction")
        self._resetPolicy("sweep convergence")
        self.iteration_number_for_sweep = 1
        self._applyPolicy("pre-optimization hook", optional=True)
        self.minimizeExpectation()
        self._applyPolicy("post-optimization hook", optional=True)
        self._updatePolicy("sweep convergence")
        while not self._hasConverged("sweep convergence"):
            self._applyPolicy("contraction")
            self._applyPolicy("state compression", optional=True)
            self._applyPolicy("operator compression", optional=True)
            self.iteration_number_for_sweep += 1
            self.number_of_iterations += 1
            try:
                self._applyPolicy("pre-optimization hook", optional=True)
                self.minimizeExpectation()
                self._applyPolicy("post-optimization hook", optional=True)
                self._updatePolicy("sweep convergence")
            except RelaxFailed:
                pass

    # -- bandwidth increase (base.py:114-160) -----------------------------
    def _increaseBandwidth(self, axis, by=None, to=None, do_as_much_as_possible=False, enlargeners=None):
        center = self.state_center_data
        O_axis = O(axis) if center.ndim == 5 else 1 - axis
        d = center.shape[-1]
        old = center.shape[axis]
        new = computeNewDimension(old, by=by, to=to)
        if new == old:
            return
        if new > d * old:
            if do_as_much_as_possible:
                new = d * old
            else:
                raise ValueError("New dimension must be less than the physical dimension times the old dimension "
                                 "({} > {}*{}).".format(new, d, old))
        neighbor_0 = center.normalizeAxis(O_axis)[0]
        neighbor_1 = center.normalizeAxis(axis)[0]
        if enlargeners is None:
            enlarge_a, enlarge_b = center.newEnlargener(old, new)
        else:
            enlarge_a, enlarge_b = enlargeners
        center = center.absorbMatrixAt(axis, enlarge_a)
        neighbor_0 = neighbor_0.absorbMatrixAt(O_axis, enlarge_b)
        neighbor_0, center = neighbor_0.normalizeAxisAndDenormalize(O_axis, axis, center)
        neighbor_1 = neighbor_1.absorbMatrixAt(axis, enlarge_a)
        center = center.absorbMatrixAt(O_axis, enlarge_b)
        neighbor_1, center = neighbor_1.normalizeAxisAndDenormalize(axis, O_axis, center)
        self.setStateCenter(center)
        self.contractUnnormalizedTowards(axis, neighbor_0)
        self.contractUnnormalizedTowards(O_axis, neighbor_1)
        self.just_increased_bandwidth = True
        return enlarge_a, enlarge_b
