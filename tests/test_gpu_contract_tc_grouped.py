"""The grouped tensor-core contraction (carc_zcontract_tc_grouped): one call
for a whole tag-pair table against the FP64 grouped contraction (within the
split-BF16 tolerance) and against the per-pair tensor-core path, with
repeated operands, outputs fed by non-consecutive entries, conjugation,
accumulation and strided operands."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
TC_TOL = 5e-5


def _rand(shape, g):
    return torch.complex(torch.randn(shape, generator=g, dtype=torch.float64),
                         torch.randn(shape, generator=g, dtype=torch.float64)).cuda()


@pytest.fixture(scope="module")
def engine():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import engine as E
    return E


CASES = [
    # spec, A shape, B shape, out shape, n_a, n_b, n_c, entries
    ("abk,kc->abc", (5, 7, 33), (33, 9), (5, 7, 9), 3, 2, 2,
     [(0, 0, 1), (1, 1, 0), (2, 0, 1), (0, 1, 0), (1, 0, 1)]),
    ("ak,bk->ab", (130, 64), (40, 64), (130, 40), 2, 3, 3, [(0, 2, 2), (1, 0, 0), (1, 1, 2), (0, 0, 1)]),
    ("xayb,ybz->xaz", (4, 6, 8, 5), (8, 5, 300), (4, 6, 300), 2, 2, 1, [(0, 0, 0), (1, 1, 0), (1, 0, 0)]),
]


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("conj_a,conj_b,accumulate", [(False, False, False), (True, False, True), (False, True, False)])
def test_grouped_tc_matches_fp64_and_per_pair(engine, case, conj_a, conj_b, accumulate):
    spec, sa, sb, sc, n_a, n_b, n_c, entries = CASES[case]
    g = torch.Generator().manual_seed(10 + case)
    A = [_rand(sa, g) for _ in range(n_a)]
    B = [_rand(sb, g) for _ in range(n_b)]
    C0 = [_rand(sc, g) for _ in range(n_c)]
    ref = [c.clone() for c in C0]
    engine.contract_grouped(spec, A, B, ref, entries, conj_a=conj_a, conj_b=conj_b, accumulate=accumulate)
    got = [c.clone() for c in C0]
    st = engine.contract_grouped_tc(spec, A, B, got, entries, conj_a=conj_a, conj_b=conj_b, accumulate=accumulate)
    assert st.numel() == 1 and int(st.abs().max()) == 0
    pair = [c.clone() for c in C0]
    st2 = engine.contract_grouped_tc(spec, A, B, pair, entries, conj_a=conj_a, conj_b=conj_b, accumulate=accumulate,
                                     grouped=False)
    assert int(st2.abs().max()) == 0
    used = {c for _, _, c in entries}
    for k in range(n_c):
        if k not in used:  # outputs no entry names are left as they were
            assert torch.equal(got[k], C0[k])
            continue
        scale = ref[k].abs().max().item()
        assert (got[k] - ref[k]).abs().max().item() <= TC_TOL * scale
        assert (pair[k] - ref[k]).abs().max().item() <= TC_TOL * scale


def test_grouped_tc_strided_operands(engine):
    """Operands that are permuted views (shared strides) of larger tensors."""
    g = torch.Generator().manual_seed(3)
    A = [_rand((9, 20, 6), g).permute(1, 0, 2) for _ in range(2)]    # (20, 9, 6) view
    B = [_rand((6, 11), g) for _ in range(2)]
    ref = [torch.zeros((20, 9, 11), dtype=torch.complex128, device="cuda") for _ in range(2)]
    got = [torch.zeros_like(r) for r in ref]
    entries = [(0, 1, 1), (1, 0, 0), (1, 1, 1)]
    engine.contract_grouped("abk,kc->abc", A, B, ref, entries)
    st = engine.contract_grouped_tc("abk,kc->abc", A, B, got, entries)
    assert int(st.abs().max()) == 0
    for r, o in zip(ref, got):
        assert (o - r).abs().max().item() <= TC_TOL * r.abs().max().item()


def test_grouped_tc_is_deterministic(engine):
    g = torch.Generator().manual_seed(4)
    A = [_rand((64, 96), g) for _ in range(4)]
    B = [_rand((96, 48), g) for _ in range(4)]
    entries = [(i, j, (i + j) % 3) for i in range(4) for j in range(4)]
    outs = []
    for _ in range(2):
        C = [torch.zeros((64, 48), dtype=torch.complex128, device="cuda") for _ in range(3)]
        engine.contract_grouped_tc("ak,kb->ab", A, B, C, entries)
        outs.append(C)
    for x, y in zip(*outs):
        assert torch.equal(x, y)


def test_absorb_matrices_tc_matches_fp64(engine):
    """The compressor's application to every tag of a boundary
    (compression.absorb_matrices): one grouped tensor-core call per shape
    class and matrix against the FP64 absorbMatrixAt chain, with tags of two
    shapes (a compressed operator axis)."""
    from carcassonne_gb300.compression import absorb_matrices, compression_precision
    from carcassonne_gb300.data import TorchData
    g = torch.Generator().manual_seed(8)
    sparse = {"a": TorchData(_rand((6, 5, 1, 12, 12, 1, 3, 3), g)), "b": TorchData(_rand((6, 5, 1, 12, 12, 1, 3, 3), g)),
              "c": TorchData(_rand((6, 5, 2, 12, 12, 1, 3, 3), g))}
    P = TorchData(_rand((4, 12), g))
    Pc = P.conj()
    ref = absorb_matrices(sparse, 3, P, 4, Pc)
    with compression_precision("tc"):
        got = absorb_matrices(sparse, 3, P, 4, Pc)
    assert list(got) == list(ref)
    for t in ref:
        r, o = ref[t]._t, got[t]._t
        assert tuple(o.shape) == tuple(r.shape) == tuple(sparse[t].shape[:3]) + (4, 4) + tuple(sparse[t].shape[5:])
        assert (o - r).abs().max().item() <= TC_TOL * r.abs().max().item()
