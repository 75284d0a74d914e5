"""The growth runs' compression retry (bench._compress_retry) on the CPU with
a stand-in system: a compression whose normal equations end above the
tolerance (AssertionError, as the reference's ``assert info == 0``) is
retried from a reseeded start, at most three times, and every failed attempt
is logged; a fourth failure is raised."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


class _System:
    def __init__(self, failures):
        self.failures = failures
        self.seeds = []

    def compressCornerStateTowards(self, corner, direction, new_dimension):
        self.seeds.append(int(np.random.get_state()[1][0]))
        if len(self.seeds) <= self.failures:
            raise AssertionError("normal equations of the product compressor did not converge (round 0)")
        return "P"


@pytest.fixture(autouse=True)
def _no_device(monkeypatch):
    monkeypatch.setattr(bench, "_sync_time", lambda fn: (fn(), 0.25))


@pytest.mark.parametrize("failures", [0, 1, 3])
def test_retries_until_a_start_converges(failures):
    system, log = _System(failures), []
    t = bench._compress_retry(system, 2, 1, 8, 1000 * 5 + 21, log, step=5)
    assert t == 0.25
    assert len(system.seeds) == failures + 1
    assert len(set(system.seeds)) == failures + 1  # a new start each time
    assert [e["attempt"] for e in log] == list(range(failures))
    assert all(e["step"] == 5 and e["corner"] == 2 and e["direction"] == 1 for e in log)


def test_first_attempt_uses_the_run_seed():
    system = _System(0)
    bench._compress_retry(system, 0, 0, 8, 1234, [], step=1)
    np.random.seed(1234)
    assert system.seeds[0] == int(np.random.get_state()[1][0])


def test_a_fourth_failure_is_raised():
    system, log = _System(4), []
    with pytest.raises(AssertionError):
        bench._compress_retry(system, 1, 0, 8, 7, log, step=3)
    assert len(log) == 4 and len(system.seeds) == 4
