"""Policies of the sweep driver (carcassonne/policies.py) against a scripted
stand-in system: the contraction pattern, the binding proxies and each
convergence rule's decisions, on the CPU."""
import pytest
import torch

from carcassonne_gb300 import policies as P
from carcassonne_gb300.system.base import BaseSystem


class FakeSystem(BaseSystem):
    def __init__(self, values=()):
        super().__init__()
        self.contracted = []
        self.grown = []
        self.compressed = []
        self.values = list(values)

    def contractTowards(self, direction):
        self.contracted.append(direction)

    def increaseBandwidth(self, direction, by=None, to=None, do_as_much_as_possible=False):
        self.grown.append((direction, by, do_as_much_as_possible))

    def compressCornerStateTowards(self, corner_id, direction, new_dimension):
        self.compressed.append((corner_id, direction, new_dimension))

    def computeOneSiteExpectation(self):
        return self.values.pop(0)

    computeExpectation = computeOneSiteExpectation


def test_repeat_pattern_cycles_and_restarts_after_reset():
    s = FakeSystem()
    s.setPolicy("contraction", P.RepeatPatternContractionPolicy([0, 2, 1]))
    for _ in range(5):
        s._applyPolicy("contraction")
    assert s.contracted == [0, 2, 1, 0, 2]
    s._resetPolicy("contraction")
    s._applyPolicy("contraction")
    assert s.contracted[-1] == 0


def test_repeat_pattern_empty_raises():
    s = FakeSystem()
    s.setPolicy("contraction", P.RepeatPatternContractionPolicy([]))
    with pytest.raises(ValueError):
        s._applyPolicy("contraction")


def test_policy_registry_rules():
    s = FakeSystem()
    with pytest.raises(ValueError):
        s.setPolicy("no such policy", P.HookPolicy(lambda system: None))
    s.setPolicy("post-optimization hook", P.HookPolicy(lambda system: system.contracted.append("hook")))
    with pytest.raises(ValueError):
        s.setPolicy("post-optimization hook", P.HookPolicy(lambda system: None))
    s._applyPolicy("post-optimization hook")
    assert s.contracted == ["hook"]
    with pytest.raises(ValueError):
        s._applyPolicy("contraction")          # required and unset
    s._applyPolicy("pre-optimization hook", optional=True)  # optional and unset


def test_bandwidth_and_compression_policies():
    s = FakeSystem()
    s.setPolicy("bandwidth increase", P.AllDirectionsIncrementBandwidthIncreasePolicy(2))
    s._applyPolicy("bandwidth increase")
    assert s.grown == [(0, 2, True), (1, 2, True)]
    t = FakeSystem()
    t.setPolicy("bandwidth increase", P.AlternatingDirectionsIncrementBandwidthIncreasePolicy())
    for _ in range(3):
        t._applyPolicy("bandwidth increase")
    assert [g[0] for g in t.grown] == [0, 1, 0]
    u = FakeSystem()
    u.setPolicy("state compression", P.ConstantStateCompressionPolicy(3))
    u._applyPolicy("state compression")
    assert u.compressed == [(c, d, 3) for c in range(4) for d in range(2)]


def test_one_site_expectation_convergence_rule():
    s = FakeSystem([-1.0, -1.2, -1.2000001])
    s.setPolicy("sweep convergence", P.RelativeOneSiteExpectationDifferenceThresholdConvergencePolicy(1e-5))
    s._updatePolicy("sweep convergence")
    assert not s._hasConverged("sweep convergence")      # one value only
    s._updatePolicy("sweep convergence")
    assert not s._hasConverged("sweep convergence")      # relative change 0.18
    s._updatePolicy("sweep convergence")
    assert s._hasConverged("sweep convergence")          # relative change 8e-8
    s._resetPolicy("sweep convergence")
    assert not s._hasConverged("sweep convergence")


def test_expectation_difference_difference_rule():
    s = FakeSystem([1.0, 2.0, 3.0, 4.0 + 1e-9])
    s.setPolicy("run convergence", P.RelativeExpectationDifferenceDifferenceThresholdConvergencePolicy(1e-6))
    results = []
    for _ in range(4):
        s._updatePolicy("run convergence")
        results.append(bool(s._hasConverged("run convergence")))
    # differences 1, 1, 1+1e-9: converged once two differences exist and agree
    assert results == [False, False, True, True]


def test_state_difference_rule():
    class S(FakeSystem):
        pass
    s = S()
    from types import SimpleNamespace
    center = lambda scale: SimpleNamespace(_t=torch.ones(2, 2, 2, 2, 2, dtype=torch.complex128) * scale)  # noqa: E731
    s.setPolicy("sweep convergence", P.RelativeStateDifferenceThresholdConvergencePolicy(1e-6))
    s.state_center_data = center(1.0)
    s._updatePolicy("sweep convergence")
    assert not s._hasConverged("sweep convergence")
    s.state_center_data = center(1 + 1e-9)
    s._updatePolicy("sweep convergence")
    assert s._hasConverged("sweep convergence")
    s.state_center_data = center(2.0)
    s._updatePolicy("sweep convergence")
    assert not s._hasConverged("sweep convergence")


def test_one_policy_object_serves_two_systems():
    pol = P.RelativeOneSiteExpectationDifferenceThresholdConvergencePolicy(1e-3)
    a, b = FakeSystem([1.0, 1.0]), FakeSystem([5.0, 9.0])
    a.setPolicy("sweep convergence", pol)
    b.setPolicy("sweep convergence", pol)
    for _ in range(2):
        a._updatePolicy("sweep convergence")
        b._updatePolicy("sweep convergence")
    assert a._hasConverged("sweep convergence") and not b._hasConverged("sweep convergence")
