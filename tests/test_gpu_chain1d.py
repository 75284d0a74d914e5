"""The 1D chain on the GPU: contractions and the expectation multiplier
against the reference's outputs (tests/golden/chain1d.npz), total and one-site
expectations of transverse-Ising systems, and the known answers of the
reference's 1D system and simulator tests (a field and a weakly coupled
transverse Ising chain reached by the driver with its policies)."""
import os

import numpy as np
import pytest

from tests.test_gpu_system import env  # noqa: F401  (fixture)

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "chain1d.npz")


def _close(a, b, tol=1e-12):
    return np.abs(a - b).max() <= tol * max(1.0, np.abs(b).max())


@pytest.mark.parametrize("case", range(4))
def test_contractions_and_multiplier(env, case):
    from carcassonne_gb300.data import TorchData
    from carcassonne_gb300.tensors import _1d as t1
    z = np.load(GOLD)
    L, R, O, S, L2, R2 = (TorchData(z[f"c{case}_{k}"]) for k in ("L", "R", "O", "S", "L2", "R2"))
    Sc = S.conj()
    assert _close(t1.absorbCenterOSSIntoLeftEnvironment(L, O, S, Sc).toArray(), z[f"c{case}_ossL"])
    assert _close(t1.absorbCenterOSSIntoRightEnvironment(R, O, S, Sc).toArray(), z[f"c{case}_ossR"])
    assert _close(t1.absorbCenterSSIntoLeftEnvironment(L2, S, Sc).toArray(), z[f"c{case}_ssL"])
    assert _close(t1.absorbCenterSSIntoRightEnvironment(R2, S, Sc).toArray(), z[f"c{case}_ssR"])
    m = t1.formExpectationMultiplier(R, L, O)
    assert _close(m(S).toArray(), z[f"c{case}_y"])
    M = m.formMatrix()
    assert _close(M.toArray(), z[f"c{case}_M"])
    assert (m.cost_of_multiply, m.cost_of_formMatrix) == tuple(int(c) for c in z[f"c{case}_cost"])
    # formMatrix agrees with multiply (tests/test_tensors_1d.py)
    assert _close(M.contractWith(S.ravel(), (1,), (0,)).toArray().reshape(S.shape), m(S).toArray(), 1e-11)


@pytest.mark.parametrize("case", range(3))
def test_expectations_match_reference(env, case):
    from carcassonne_gb300.system._1d import System
    from carcassonne_gb300.utils import Pauli, buildTensor
    z = np.load(GOLD)
    h = float(z[f"e{case}_h"])
    mpo = buildTensor((3, 3, 2, 2), {(0, 0): Pauli.I, (0, 2): h * Pauli.Z, (0, 1): -0.01 * Pauli.X,
                                     (1, 2): Pauli.X, (2, 2): Pauli.I})
    system = System([1, 0, 0], [0, 0, 1], mpo, z[f"e{case}_S"], z[f"e{case}_rb"], z[f"e{case}_lb"])
    E, one = complex(z[f"e{case}_E"]), complex(z[f"e{case}_one"])
    assert abs(system.computeExpectation() - E.real) <= 1e-10 * max(1.0, abs(E))
    assert abs(system.computeOneSiteExpectation() - abs(one)) <= 1e-8 * max(1.0, abs(one))


@pytest.mark.parametrize("channels", [2, 3, 4])
def test_one_site_expectation_of_a_field_all_up(env, channels):
    """The Z field (alone, or closing a ZZ / ZZZ string) on the all-up state:
    the one-site expectation is |field strength| (tests/test_system_1d.py)."""
    from carcassonne_gb300.system._1d import System
    from carcassonne_gb300.utils import Pauli, buildTensor
    rng = np.random.default_rng(channels)
    for _ in range(3):
        phase, strength = rng.uniform(0, 2 * np.pi), rng.uniform(-3, 3)
        comps = {(0, 0): Pauli.I, (0, 1): strength * Pauli.Z, (channels - 1, channels - 1): Pauli.I}
        for c in range(1, channels - 1):
            comps[(c, c + 1)] = Pauli.Z
        boundary_r = [1] + [0] * (channels - 1)
        boundary_l = [0] * (channels - 1) + [1]
        system = System(boundary_r, boundary_l, buildTensor((channels, channels, 2, 2), comps),
                        np.array([[[np.cos(phase) + 1j * np.sin(phase), 0]]]))
        assert abs(system.computeOneSiteExpectation() - abs(strength)) < 1e-7


def test_increase_bandwidth_keeps_the_expectation(env):
    """Growing the bond (tests/test_system_1d.py:63-80): the expectation after
    increaseBandwidth equals the one after contracting the normalized center
    both ways."""
    from copy import copy
    from carcassonne_gb300.system._1d import System
    np.random.seed(7)
    for operator_dimension, state_dimension, physical_dimension in ((1, 2, 2), (3, 2, 3), (2, 3, 2)):
        new_dimension = np.random.randint(state_dimension + 1, physical_dimension * state_dimension + 1)
        system1 = System.newRandom(operator_dimension, state_dimension, physical_dimension)
        system2 = copy(system1)
        system1.increaseBandwidth(0, to=new_dimension)
        system2.contractNormalizedTowards(0)
        system2.contractNormalizedTowards(1)
        e1, e2 = system1.computeExpectation(), system2.computeExpectation()
        assert abs(e1 - e2) <= 1e-8 * max(1.0, abs(e2)), (e1, e2)


class _TooManyIterations(Exception):
    pass


def _cap(limit):
    # a post-optimization hook that ends a run that does not converge
    from carcassonne_gb300 import policies as P
    count = [0]

    def hook(system):
        count[0] += 1
        if count[0] > limit:
            raise _TooManyIterations("no convergence after %d optimizations" % limit)
    return P.HookPolicy(hook)


def _driver(system, run_policy, bandwidth):
    from carcassonne_gb300 import policies as P
    system.setPolicy("post-optimization hook", _cap(100))
    system.setPolicy("sweep convergence", P.RelativeStateDifferenceThresholdConvergencePolicy(1e-5))
    system.setPolicy("run convergence", run_policy)
    system.setPolicy("bandwidth increase", bandwidth)
    system.setPolicy("contraction", P.RepeatPatternContractionPolicy([0, 1]))
    system.runUntilConverged()
    return system


def test_simulator_transverse_ising(env):
    """tests/test_simulator_1d.py: the weakly coupled transverse Ising chain's
    one-site expectation 1.0000250001562545."""
    from carcassonne_gb300 import policies as P
    from carcassonne_gb300.system._1d import System
    from carcassonne_gb300.utils import Pauli, buildTensor
    system = System([1, 0, 0], [0, 0, 1],
                    buildTensor((3, 3, 2, 2), {(0, 0): Pauli.I, (0, 2): Pauli.Z, (0, 1): -0.01 * Pauli.X,
                                               (1, 2): Pauli.X, (2, 2): Pauli.I}),
                    np.ones((1, 1, 2)))
    _driver(system, P.RelativeOneSiteExpectationDifferenceThresholdConvergencePolicy(1e-7),
            P.OneDirectionIncrementBandwidthIncreasePolicy(0, 2))
    assert abs(system.computeOneSiteExpectation() - 1.0000250001562545) < 1e-6


def test_simulator_magnetic_field(env):
    """tests/test_simulator_1d.py: a field's estimated one-site expectation
    reaches magnitude 1."""
    from carcassonne_gb300 import policies as P
    from carcassonne_gb300.system._1d import System
    from carcassonne_gb300.utils import Pauli, buildProductTensor, buildTensor
    system = System(buildProductTensor([1, 0]), buildProductTensor([0, 1]),
                    buildTensor((2, 2, 2, 2), {(0, 0): Pauli.I, (1, 1): Pauli.I, (0, 1): -Pauli.Z}),
                    np.ones((1, 1, 2)))
    _driver(system, P.RelativeEstimatedOneSiteExpectationDifferenceThresholdConvergencePolicy(1e-2),
            P.OneDirectionIncrementBandwidthIncreasePolicy(0))
    assert abs(abs(system.computeEstimatedOneSiteExpectation(0)) - 1) < 1e-2
