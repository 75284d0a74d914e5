"""Batched uneven problems: the CUDA-graph replay gives the launch loop's
results exactly, the autotuner stores a choice the matvec then uses, and the
tensor-core results stay within the split-BF16 tolerance of FP64."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batched():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import batched as B
    return B


def test_graph_replay_matches_loop_and_fp64(batched):
    specs = [(2, 16, 2.5, 11), (3, 24, 3.1, 12), (2, 40, 3.9, 13), (4, 16, 2.2, 14)]
    ops = [batched.build_operator(*s) for s in specs]
    b = batched.Batch(ops, nvec=3, seed=1)
    b.run_loop()
    loop = [y.clone() for y in b.y]
    b.capture()
    for y in b.y:
        y.zero_()
    b.replay()
    torch.cuda.synchronize()
    b.check_status()
    for op, x, y0, y1 in zip(ops, b.x, loop, b.y):
        assert torch.equal(y0, y1)
        ref = op.apply(x, None, 3)
        err = ((y1 - ref).abs().max() / ref.abs().max()).item()
        assert err < 5e-5, err


def test_autotune_choice_is_used(batched):
    from carcassonne_gb300 import _lib
    op = batched.build_operator(3, 32, 3.0, 21)
    res = batched.autotune(op, 4, candidates=(0, -1, 38, 152), reps=1)
    assert res and all(e["best"] in (0, -1, 38, 152) for e in res)
    x = torch.randn((4,) + op.in_shape, dtype=torch.complex128, device="cuda")
    ref = op.apply(x, None, 4)
    got = op.apply_tc(x, None, 4)
    op.check_status()
    assert ((got - ref).abs().max() / ref.abs().max()).item() < 5e-5
    _lib.check(_lib.load().carc_tc_autotune_clear())


def test_run_small_distribution(batched, tmp_path):
    out = batched.run(count=6, nvec=2, seed=5, mem_budget=1 << 30, reps=1, tune_file=str(tmp_path / "t.json"))
    assert out["problems"] == 6 and out["loop_gflops"] > 0 and out["graph_gflops"] > 0


def test_tuning_file_round_trip(batched, tmp_path):
    """Choices saved to the tuning file are applied by a later load, and the
    matvec stays within the split-BF16 tolerance on the loaded choice."""
    from carcassonne_gb300 import _lib
    op = batched.build_operator(2, 24, 2.7, 31)
    res = batched.autotune(op, 2, candidates=(0, 76), reps=1)
    path = str(tmp_path / "tune.json")
    batched.save_tuning(res + res, path)  # duplicates are written once
    _lib.check(_lib.load().carc_tc_autotune_clear())
    loaded = batched.load_tuning(path)
    assert [e["best"] for e in loaded] == [e["best"] for e in res]
    assert batched.load_tuning(str(tmp_path / "missing.json")) == []
    x = torch.randn((2,) + op.in_shape, dtype=torch.complex128, device="cuda")
    ref = op.apply(x, None, 2)
    got = op.apply_tc(x, None, 2)
    op.check_status()
    assert ((got - ref).abs().max() / ref.abs().max()).item() < 5e-5
    _lib.check(_lib.load().carc_tc_autotune_clear())
