"""Policies of the sweep driver (carcassonne/policies.py:11-243): bandwidth
increase, state compression, contraction pattern, convergence tests and
hooks, bound to a System by ``System.setPolicy(name, policy)``.

The classes keep the reference's names, constructor arguments and decisions;
the quantities they compare (expectations, centers, gauge residuals) are
computed by the System on the GPU and read back as scalars.  A policy object
is a template: ``createBindingToSystem`` returns a proxy holding the system,
through which the driver calls ``apply`` / ``converged`` / ``reset`` /
``update`` (policies.py:11-44), so one policy object can serve several
systems.
"""
from __future__ import annotations

import logging

import torch

from .utils import O

log = logging.getLogger(__name__)


# -- binding (policies.py:11-44) ---------------------------------------------
class Policy:
    def createBindingToSystem(self, system):
        return self.Proxy(self, system)


class Proxy:
    """Per-system view of a policy: attribute reads fall through to the
    policy, attribute writes (the policy's running state) stay on the proxy."""

    def __init__(self, forward, system):
        self.forward = forward
        self.system = system

    def __getattr__(self, name):
        return getattr(self.forward, name)


class ApplyProxy(Proxy):
    def apply(self):
        return type(self.forward).apply(self)


class ConvergedProxy(Proxy):
    def converged(self):
        return type(self.forward).converged(self)


class ResetProxy(Proxy):
    def reset(self):
        return type(self.forward).reset(self)


class UpdateProxy(Proxy):
    def update(self):
        return type(self.forward).update(self)


# -- bandwidth increase (policies.py:46-76) ----------------------------------
class BandwidthIncreasePolicy(Policy):
    Proxy = ApplyProxy


class AlternatingDirectionsIncrementBandwidthIncreasePolicy(BandwidthIncreasePolicy):
    """Grows one bandwidth axis per application, alternating between the two.
    (The reference's ``apply`` reads an ``increment`` attribute its
    constructor never sets, and steps the axis with O(), which maps 0 to 2,
    an axis increaseBandwidth rejects; here the increment is an argument with
    default 1 and the axes alternate 0, 1, 0, ...)"""

    def __init__(self, directions=(0, 1), increment=1):
        self.directions = directions
        self.direction = 0
        self.increment = increment

    def apply(self):
        self.system.increaseBandwidth(self.direction, by=self.increment, do_as_much_as_possible=True)
        self.direction = 1 - self.direction


class AllDirectionsIncrementBandwidthIncreasePolicy(BandwidthIncreasePolicy):
    def __init__(self, increment=1):
        self.increment = increment

    def apply(self):
        log.info("Increasing bandwidth in all directions by %s", self.increment)
        for direction in (0, 1):
            self.system.increaseBandwidth(direction, by=self.increment, do_as_much_as_possible=True)


class OneDirectionIncrementBandwidthIncreasePolicy(BandwidthIncreasePolicy):
    def __init__(self, direction, increment=1):
        self.direction = direction
        self.increment = increment

    def apply(self):
        log.info("Increasing bandwidth in direction %s by %s", self.direction, self.increment)
        self.system.increaseBandwidth(self.direction, by=self.increment, do_as_much_as_possible=True)


# -- state compression (policies.py:78-90) -----------------------------------
class CompressionPolicy(Policy):
    Proxy = ApplyProxy


class ConstantStateCompressionPolicy(CompressionPolicy):
    """Every corner compressed towards both of its sides to new_dimension."""

    def __init__(self, new_dimension):
        self.new_dimension = new_dimension

    def apply(self):
        log.debug("Compressing to %s", self.new_dimension)
        for corner_id in range(4):
            for direction in range(2):
                self.system.compressCornerStateTowards(corner_id, direction, self.new_dimension)


# -- contraction pattern (policies.py:92-116) --------------------------------
class ContractionPolicy(Policy):
    class Proxy(ApplyProxy, ResetProxy):
        pass


class RepeatPatternContractionPolicy(ContractionPolicy):
    """Contracts towards the given directions in turn, starting over at the
    beginning of the pattern after each reset and when it runs out."""

    def __init__(self, directions):
        self.directions = directions
        self.reset()

    def apply(self):
        try:
            direction = next(self.iteration)
        except StopIteration:
            self.iteration = iter(self.directions)
            try:
                direction = next(self.iteration)
            except StopIteration:
                raise ValueError("An empty sequence of contraction directions was provided! ({})".format(
                    self.directions)) from None
        log.debug("Contracting towards direction %s", direction)
        self.system.contractTowards(direction)

    def reset(self):
        self.iteration = iter([])


# -- convergence (policies.py:118-243) ---------------------------------------
def _relative_change(current, last):
    """|current - last| and its size relative to the mean magnitude."""
    absolute = abs(current - last)
    return absolute, absolute / abs(current + last) * 2


class ConvergencePolicy(Policy):
    class Proxy(ConvergedProxy, ResetProxy, UpdateProxy):
        pass


class PeriodicyThresholdConvergencePolicy(ConvergencePolicy):
    """Converged when, summed over the directions, the center differs by less
    than threshold from its own gauge-moved form (normalized along the
    direction, then the opposite side's denormalizer absorbed): the state
    repeats with the lattice period."""

    def __init__(self, threshold, *directions):
        self.threshold = threshold
        if not directions:
            raise ValueError("at least one direction must be specified")
        self.directions = directions

    def converged(self):
        center = self.system.state_center_data
        difference = 0.0
        for direction in self.directions:
            normalized = center.normalizeAxis(direction)[0]
            denormalizer = center.normalizeAxis(O(direction))[-1]
            difference += (center - normalized.absorbMatrixAt(direction, denormalizer)).norm()
        return difference < self.threshold

    def reset(self):
        pass

    def update(self):
        pass


class RelativeEstimatedOneSiteExpectationDifferenceThresholdConvergencePolicy(ConvergencePolicy):
    """Compares successive estimates of the one-site expectation (the energy
    gained by one more contraction, System.computeEstimatedOneSiteExpectation)."""

    def __init__(self, threshold, direction=0):
        self.direction = direction
        self.threshold = threshold
        self.last = None
        self.current = None

    def converged(self):
        last, current = self.last, self.current
        if last is not None and current is not None:
            magnitude = abs(current + last)
            if magnitude < 1e-15:
                return True
            absolute, relative = _relative_change(current, last)
            log.debug("estimated one-site expectation %s, absolute difference %s, relative difference %s, "
                      "magnitude %s", current, absolute, relative, magnitude)
            return relative < self.threshold

    def reset(self):
        self.last = None
        self.current = None

    def update(self):
        self.last = self.current
        self.current = self.system.computeEstimatedOneSiteExpectation(self.direction)


class RelativeExpectationDifferenceDifferenceThresholdConvergencePolicy(ConvergencePolicy):
    """Compares successive differences of the total expectation (the energy
    added per step): converged when that increment stops changing."""

    def __init__(self, threshold):
        self.threshold = threshold
        self.reset()

    def converged(self):
        last, current = self.last_difference, self.current_difference
        if last is not None and current is not None:
            absolute = abs(current - last)
            if absolute < 1e-15:
                return True
            return absolute / abs(current + last) * 2 < self.threshold

    def reset(self):
        self.last_value = None
        self.last_difference = None
        self.current_value = None
        self.current_difference = None

    def update(self):
        self.last_value = self.current_value
        self.last_difference = self.current_difference
        self.current_value = self.system.computeExpectation()
        if self.last_value is not None:
            self.current_difference = self.current_value - self.last_value


class RelativeOneSiteExpectationDifferenceThresholdConvergencePolicy(ConvergencePolicy):
    """Compares successive one-site expectations (System.computeOneSiteExpectation)."""

    def __init__(self, threshold):
        self.threshold = threshold
        self.last = None
        self.current = None

    def converged(self):
        last, current = self.last, self.current
        if last is not None and current is not None:
            if current - last > self.threshold:
                log.info("Current expectation (%s) is greater than last expectation (%s)!", current, last)
            absolute = abs(current - last)
            if absolute < 1e-15:
                return True
            relative = absolute / abs(current + last) * 2
            log.debug("Expectations: current = %s; last = %s; absolute difference = %s; relative difference = %s",
                      current, last, absolute, relative)
            return relative < self.threshold

    def reset(self):
        self.last = None
        self.current = None

    def update(self):
        expectation = self.system.computeOneSiteExpectation()
        self.last = self.current
        self.current = expectation


class RelativeStateDifferenceThresholdConvergencePolicy(ConvergencePolicy):
    """Compares successive state centers (2-norm of the difference over the
    mean norm), on the device."""

    def __init__(self, threshold):
        self.threshold = threshold
        self.last = None
        self.current = None

    def converged(self):
        last, current = self.last, self.current
        if last is None or current is None or last.shape != current.shape:
            return False
        magnitude = float(torch.linalg.vector_norm(current + last))
        if magnitude < 1e-15:
            return True
        relative = float(torch.linalg.vector_norm(current - last)) / magnitude * 2
        log.debug("site relative difference = %s (magnitude = %s)", relative, magnitude)
        return relative < self.threshold

    def reset(self):
        self.last = None
        self.current = None

    def update(self):
        self.last = self.current
        self.current = self.system.state_center_data._t.detach().clone()


# -- hooks (policies.py:245-252) ---------------------------------------------
class HookPolicy(Policy):
    Proxy = ApplyProxy

    def __init__(self, callback):
        self.callback = callback

    def apply(self):
        return self.callback(self.system)


__all__ = [
    "Policy",
    "Proxy",
    "ApplyProxy",
    "ConvergedProxy",
    "ResetProxy",
    "UpdateProxy",
    "BandwidthIncreasePolicy",
    "AllDirectionsIncrementBandwidthIncreasePolicy",
    "AlternatingDirectionsIncrementBandwidthIncreasePolicy",
    "OneDirectionIncrementBandwidthIncreasePolicy",
    "CompressionPolicy",
    "ConstantStateCompressionPolicy",
    "ContractionPolicy",
    "RepeatPatternContractionPolicy",
    "ConvergencePolicy",
    "PeriodicyThresholdConvergencePolicy",
    "RelativeEstimatedOneSiteExpectationDifferenceThresholdConvergencePolicy",
    "RelativeExpectationDifferenceDifferenceThresholdConvergencePolicy",
    "RelativeOneSiteExpectationDifferenceThresholdConvergencePolicy",
    "RelativeStateDifferenceThresholdConvergencePolicy",
    "HookPolicy",
]
