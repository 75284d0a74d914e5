"""The sweep driver with the reference's policies on the GPU System: the
known answers of the reference's 2D-in-1.5D simulator tests (a uniform field,
a ferromagnetic coupling along either axis, a weakly coupled transverse
Ising model), reached by runUntilConverged with state compression,
bandwidth increases and the repeating contraction pattern."""
import pytest

from tests.test_gpu_system import env  # noqa: F401  (fixture)

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[0, 1, 2], autouse=True)
def seeded(request):
    """The runs draw their bandwidth enlargeners and compressor starts from
    numpy's and Python's global generators, as the reference's do: each test
    runs for three fixed seeds, independent of the tests before it."""
    import random
    import numpy as np
    np.random.seed(request.param)
    random.seed(request.param)
    return request.param


def _run(system, bandwidth_policy):
    from carcassonne_gb300 import policies as P
    count = [0]

    def cap(system):  # ends a run that does not converge
        count[0] += 1
        assert count[0] <= 200, "no convergence after 200 optimizations"
    system.setPolicy("post-optimization hook", P.HookPolicy(cap))
    system.setPolicy("state compression", P.ConstantStateCompressionPolicy(1))
    system.setPolicy("sweep convergence", P.RelativeOneSiteExpectationDifferenceThresholdConvergencePolicy(1e-7))
    system.setPolicy("run convergence", P.RelativeOneSiteExpectationDifferenceThresholdConvergencePolicy(1e-7))
    system.setPolicy("bandwidth increase", bandwidth_policy)
    system.setPolicy("contraction", P.RepeatPatternContractionPolicy(range(4)))
    system.runUntilConverged()
    return system.computeOneSiteExpectation()


def test_magnetic_field(env):
    from carcassonne_gb300 import policies as P
    from carcassonne_gb300.data import TorchData
    from carcassonne_gb300.system import System
    e = _run(System.newTrivialWithSimpleSparseOperator(O=TorchData.Z), P.AllDirectionsIncrementBandwidthIncreasePolicy())
    assert abs(e - (-1)) < 1e-6


@pytest.mark.parametrize("direction", [0, 1])
def test_ferromagnetic_coupling(env, direction):
    from carcassonne_gb300 import policies as P
    from carcassonne_gb300.data import TorchData
    from carcassonne_gb300.system import System
    pair = [TorchData.Z, -TorchData.Z]
    system = (System.newTrivialWithSimpleSparseOperator(OO_LR=pair) if direction == 0
              else System.newTrivialWithSimpleSparseOperator(OO_UD=pair))
    e = _run(system, P.AllDirectionsIncrementBandwidthIncreasePolicy())
    assert abs(e - (-1)) < 1e-6


@pytest.mark.parametrize("direction", [0, 1])
def test_transverse_ising(env, direction):
    from carcassonne_gb300 import policies as P
    from carcassonne_gb300.data import TorchData
    from carcassonne_gb300.system import System
    pair = [TorchData.X, -0.01 * TorchData.X]
    system = (System.newTrivialWithSimpleSparseOperator(O=-TorchData.Z, OO_LR=pair) if direction == 0
              else System.newTrivialWithSimpleSparseOperator(O=-TorchData.Z, OO_UD=pair))
    e = _run(system, P.OneDirectionIncrementBandwidthIncreasePolicy(direction))
    assert abs(e - (-1.0000250001562545)) < 1e-6
