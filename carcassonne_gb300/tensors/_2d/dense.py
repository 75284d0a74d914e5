"""Dense contractors of the 2D center-site path (tensors/_2d/dense.py:10-242).

Each contractor is a callable with the reference's signature and a
``grouped`` form that runs all tag pairs of one sparse contraction in a single
launch of the grouped GETT kernel.  The index contract of every contractor is
the one pinned by the reference's tests (tests/test_tensors_dense.py) and is
written here as an einsum-style spec over the raw (unjoined) axes; the
reference's trailing ``join`` is folded into the output strides.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ... import _lib, engine
from ...data import TorchData
from ...data.cost_tracker import stage3_form_matrix_cost, stage3_multiply_cost
from ...engine import CDT, current_stream_handle
from ...utils import L, R, O, Multiplier, UnexpectedTensorRankError, DimensionMismatchError


def _t(x):
    return x._t if isinstance(x, TorchData) else TorchData(x)._t


def _check_rank(number, t, rank):
    if t.dim() != rank:
        raise UnexpectedTensorRankError(number, rank, t.dim())


def _check_dims(ln, li, a, rn, ri, b):
    if a.shape[li] != b.shape[ri]:
        raise DimensionMismatchError(ln, li, int(a.shape[li]), rn, ri, int(b.shape[ri]))


class _PairContractor:
    """A two-operand contractor given by a spec and an output-shape rule."""

    def __init__(self, name, spec, ranks, joins, shape_fn, doc):
        self.__name__ = name
        self.spec = engine.Spec(spec)
        self.ranks = ranks
        self.joins = joins          # [(operand, axis, operand, axis)] dimension checks
        self.shape_fn = shape_fn
        self.__doc__ = doc

    def _validate(self, a, b):
        _check_rank(0, a, self.ranks[0])
        _check_rank(1, b, self.ranks[1])
        ops = (a, b)
        for ln, li, rn, ri in self.joins:
            _check_dims(ln, li, ops[ln], rn, ri, ops[rn])

    def __call__(self, a, b):
        ta, tb = _t(a), _t(b)
        self._validate(ta, tb)
        out = torch.empty(self.shape_fn(ta.shape, tb.shape), dtype=CDT, device=ta.device)
        engine.contract_grouped(self.spec, [ta], [tb], [out], [(0, 0, 0)])
        return TorchData(out)

    def grouped(self, list_a, list_b, table, n_out):
        ta = [_t(x) for x in list_a]
        tb = [_t(x) for x in list_b]
        self._validate(ta[0], tb[0])
        shape = self.shape_fn(ta[0].shape, tb[0].shape)
        outs = [torch.empty(shape, dtype=CDT, device=ta[0].device) for _ in range(n_out)]
        for lo in range(0, len(table), _lib.MAX_ENTRIES):
            chunk = table[lo:lo + _lib.MAX_ENTRIES]
            used_a = sorted({e[0] for e in chunk})
            used_b = sorted({e[1] for e in chunk})
            used_c = sorted({e[2] for e in chunk})
            ma = {v: i for i, v in enumerate(used_a)}
            mb = {v: i for i, v in enumerate(used_b)}
            mc = {v: i for i, v in enumerate(used_c)}
            # output slots already written by an earlier chunk accumulate
            first = all(e[2] not in {x[2] for x in table[:lo]} for e in chunk)
            engine.contract_grouped(self.spec, [ta[i] for i in used_a], [tb[i] for i in used_b],
                                    [outs[i] for i in used_c], [(ma[i], mb[j], mc[k]) for i, j, k in chunk],
                                    accumulate=not first)
        return [TorchData(o) for o in outs]


absorbDenseSideIntoCornerFromLeft = _PairContractor(
    "absorbDenseSideIntoCornerFromLeft", "xyzdef,abcxyzjk->abcdjekf", (6, 8),
    [(0, 0, 1, 3), (0, 1, 1, 4), (0, 2, 1, 5)],
    lambda c, s: (s[0], s[1], s[2], c[3] * s[6], c[4] * s[7], c[5]),
    "C'[a,b,c,(d,j),(e,k),f] = sum C[x,y,z,d,e,f] T[a,b,c,x,y,z,j,k]  (tensors/_2d/dense.py:10-15)")

absorbDenseSideIntoCornerFromRight = _PairContractor(
    "absorbDenseSideIntoCornerFromRight", "abcxyz,xyzghijk->ajbkcghi", (6, 8),
    [(0, 3, 1, 0), (0, 4, 1, 1), (0, 5, 1, 2)],
    lambda c, s: (c[0] * s[6], c[1] * s[7], c[2], s[3], s[4], s[5]),
    "C'[(a,j),(b,k),c,g,h,i] = sum C[a,b,c,x,y,z] T[x,y,z,g,h,i,j,k]  (tensors/_2d/dense.py:16-21)")

formNormalizationStage1 = _PairContractor(
    "formNormalizationStage1", "abcxyz,xyzdefkl->abcdefkl", (6, 8),
    [(0, 3, 1, 0), (0, 4, 1, 1), (0, 5, 1, 2)],
    lambda c, s: (c[0] * c[1] * c[2], s[3] * s[4] * s[5], s[6], s[7]),
    "S1[(a,b,c),(d,e,f),k,l] = sum C[a,b,c,x,y,z] T[x,y,z,d,e,f,k,l]  (tensors/_2d/dense.py:95-100)")

formNormalizationStage2 = _PairContractor(
    "formNormalizationStage2", "abkl,camn->cbkmln", (4, 4),
    [(0, 0, 1, 1)],
    lambda a, b: (b[0], a[1], a[2], b[2], a[3], b[3]),
    "S2[c,b,k,m,l,n] = sum_a A[a,b,k,l] B[c,a,m,n]  (tensors/_2d/dense.py:101-113)")


# ---------------------------------------------------------------------------
# absorption of the center into a side
# ---------------------------------------------------------------------------
def _center_letters(direction, ket):
    """Letters of the state axes: the absorbed axis is k (ket) / l (bra); the
    L, R and O axes are u,v,w (ket) / x,y,z (bra); the physical axis is q."""
    letters = [None] * 5
    letters[direction] = "k" if ket else "l"
    letters[L(direction)] = "u" if ket else "x"
    letters[R(direction)] = "v" if ket else "y"
    letters[O(direction)] = "w" if ket else "z"
    letters[4] = "q"
    return "".join(letters)


def center_pair(direction, state, op=None, state_conj=None):
    """E[u,v,w,x,y,z,k,l] = sum_{p,q} S[..k..,q] O[p,q] conj(S)[..l..,p]; op None means identity.
    (the center half of absorbDenseCenterSSIntoSide / SOSIntoSide, tensors/_2d/dense.py:22-81)"""
    s = _t(state)
    _check_rank(1, s, 5)
    conj = state_conj is None
    sc = s if conj else _t(state_conj)
    ket = _center_letters(direction, True)
    bra = _center_letters(direction, False)
    if op is not None:
        o = _t(op)
        _check_rank(3, o, 2)
        if o.shape[1] != s.shape[4]:
            raise DimensionMismatchError(3, 1, int(o.shape[1]), 1, 4, int(s.shape[4]))
        so_shape = tuple(s.shape[:4]) + (o.shape[0],)
        so = engine.contract(ket + ",pq->" + ket[:4] + "p", s, o, so_shape)
        s_in, ket_in = so, ket[:4] + "p"
        bra_in = bra[:4] + "p"
    else:
        s_in, ket_in, bra_in = s, ket, bra
    ext = {c: int(s.shape[i]) for i, c in enumerate(ket[:4])}
    ext.update({c: int(sc.shape[i]) for i, c in enumerate(bra[:4])})
    shape = tuple(ext[c] for c in "uvwxyzkl")
    return engine.contract(ket_in + "," + bra_in + "->uvwxyzkl", s_in, sc, shape, conj_b=conj)


_SIDE_SPEC = engine.Spec("abcdefkl,uvwxyzkl->aubxcdveyfwz")


def _side_out_shape(side_shape, e_shape):
    a, b, c, d, e, f = side_shape[:6]
    u, v, w, x, y, z = e_shape[:6]
    return (a * u, b * x, c, d * v, e * y, f, w, z)


def _absorb_pairs(direction, sides, pairs_e, table, n_out):
    ts = [_t(x) for x in sides]
    for t in ts:
        _check_rank(0, t, 8)
    e0 = pairs_e[0]
    if ts[0].shape[6] != e0.shape[6]:
        raise DimensionMismatchError(0, 6, int(ts[0].shape[6]), 1, direction, int(e0.shape[6]))
    if ts[0].shape[7] != e0.shape[7]:
        raise DimensionMismatchError(0, 7, int(ts[0].shape[7]), 2, direction, int(e0.shape[7]))
    shape = _side_out_shape(ts[0].shape, e0.shape)
    outs = [torch.empty(shape, dtype=CDT, device=ts[0].device) for _ in range(n_out)]
    engine.contract_grouped(_SIDE_SPEC, ts, pairs_e, outs, table)
    return [TorchData(o) for o in outs]


def absorbDenseCenterSSIntoSide(direction, side, center, center_conj=None):
    """T'[(a,sL),(b,tL),c,(d,sR),(e,tR),f,sO,tO] = sum T[..,k,l] S[..k..,q] conj(S)[..l..,q]
    (tensors/_2d/dense.py:22-50)."""
    e = center_pair(direction, center, None, center_conj)
    return _absorb_pairs(direction, [side], [e], [(0, 0, 0)], 1)[0]


def absorbDenseCenterSOSIntoSide(direction, side, state_center_data, operator_center_data,
                                 state_center_data_conj=None):
    """As absorbDenseCenterSSIntoSide with the operator between ket and bra (tensors/_2d/dense.py:51-81)."""
    e = center_pair(direction, state_center_data, operator_center_data, state_center_data_conj)
    return _absorb_pairs(direction, [side], [e], [(0, 0, 0)], 1)[0]


# ---------------------------------------------------------------------------
# stage 3: the center-site operator
# ---------------------------------------------------------------------------
class Stage3Operator:
    """sum over terms of S2_0[i0] (x) S2_1[i1] (x) O[io] as one device operator.

    ``s2_0``/``s2_1`` are lists of same-shape stage-2 tensors (x0,x1,k0,k1,l0,l1)
    and (x1,x0,k2,k3,l2,l3); ``ops`` the (d,d) operator tensors; ``terms``
    (i0, i1, io) with io < 0 for the identity (formNormalizationStage3)."""

    def __init__(self, s2_0, s2_1, ops, terms, d):
        self.s2_0 = [_t(x).contiguous() for x in s2_0]
        self.s2_1 = [_t(x).contiguous() for x in s2_1]
        self.ops = [_t(x).contiguous() for x in ops]
        self.terms = [tuple(int(v) for v in t) for t in terms]
        self.d = int(d)
        if self.s2_0:
            _check_rank(0, self.s2_0[0], 6)
            _check_rank(1, self.s2_1[0], 6)
            if self.s2_0[0].shape[0] != self.s2_1[0].shape[1]:
                raise DimensionMismatchError(0, 0, int(self.s2_0[0].shape[0]), 1, 1, int(self.s2_1[0].shape[1]))
            if self.s2_0[0].shape[1] != self.s2_1[0].shape[0]:
                raise DimensionMismatchError(0, 1, int(self.s2_0[0].shape[1]), 1, 0, int(self.s2_1[0].shape[0]))
        self.s0_shape = tuple(int(x) for x in self.s2_0[0].shape)
        self.s1_shape = tuple(int(x) for x in self.s2_1[0].shape)
        k0, k1, l0, l1 = self.s0_shape[2:6]
        k2, k3, l2, l3 = self.s1_shape[2:6]
        self.in_shape = (k0, k1, k2, k3, self.d)
        self.out_shape = (l0, l1, l2, l3, self.d)
        self.device = self.s2_0[0].device
        self._pack()

    def _pack(self):
        self._p0, self._k0 = _lib.ptr_array([t.data_ptr() for t in self.s2_0])
        self._p1, self._k1 = _lib.ptr_array([t.data_ptr() for t in self.s2_1])
        self._po, self._ko = _lib.ptr_array([t.data_ptr() for t in self.ops])
        self._pt, self._kt = _lib.i32_array([v for t in self.terms for v in t])
        self._s0, self._ks0 = _lib.i64_array(self.s0_shape)
        self._s1, self._ks1 = _lib.i64_array(self.s1_shape)

    @property
    def n(self):
        return int(np.prod(self.out_shape))

    def cost_of_multiply(self):
        return sum(stage3_multiply_cost(self.s0_shape, self.s1_shape, self.d, io < 0) for _, _, io in self.terms)

    def cost_of_formMatrix(self):
        return len(self.terms) * stage3_form_matrix_cost(self.s0_shape, self.s1_shape, self.d)

    def apply(self, x, y=None, nvec=1, accumulate=False):
        """y = op . x for nvec stacked centers (torch tensors, contiguous)."""
        lib = _lib.load()
        x = x.contiguous()
        if y is None:
            y = torch.empty((nvec,) + self.out_shape if nvec > 1 else self.out_shape, dtype=CDT, device=x.device)
        ws_bytes = lib.carc_stage3_matvec_f64_workspace_size(self._s0, self._s1, self.d, len(self.terms), nvec)
        if ws_bytes < 0:
            _lib.check(_lib.CARC_BAD_SHAPE)
        ws = engine.Workspace.get(ws_bytes, x.device)
        _lib.call("carc_stage3_matvec_f64", self._s0, self._s1, self.d, self._p0, len(self.s2_0), self._p1,
                  len(self.s2_1), self._po, len(self.ops), self._pt, len(self.terms), ctypes.c_void_p(x.data_ptr()),
                  ctypes.c_void_p(y.data_ptr()), nvec, int(bool(accumulate)), ctypes.c_void_p(ws.data_ptr()),
                  ws_bytes, current_stream_handle())
        return y

    def __call__(self, v):
        t = _t(v)
        if tuple(t.shape) != self.in_shape:
            raise ValueError("center has shape %s, operator expects %s" % (tuple(t.shape), self.in_shape))
        return TorchData(self.apply(t))

    def form_matrix(self, out=None, accumulate=False):
        lib = _lib.load()
        n_r = self.n
        n_c = int(np.prod(self.in_shape))
        if out is None:
            out = torch.empty((n_r, n_c), dtype=CDT, device=self.device)
        ws_bytes = lib.carc_stage3_form_matrix_f64_workspace_size(self._s0, self._s1, self.d, len(self.terms))
        if ws_bytes < 0:
            _lib.check(_lib.CARC_BAD_SHAPE)
        ws = engine.Workspace.get(ws_bytes, self.device)
        _lib.call("carc_stage3_form_matrix_f64", self._s0, self._s1, self.d, self._p0, len(self.s2_0), self._p1,
                  len(self.s2_1), self._po, len(self.ops), self._pt, len(self.terms), ctypes.c_void_p(out.data_ptr()),
                  int(bool(accumulate)), ctypes.c_void_p(ws.data_ptr()), ws_bytes, current_stream_handle())
        return out

    def formMatrix(self):
        return TorchData(self.form_matrix())

    def multiplier(self):
        n_c = int(np.prod(self.in_shape))
        return Multiplier((self.n, n_c), self, self.cost_of_multiply(), self.formMatrix, self.cost_of_formMatrix())


def formDenseStage3_multiply_and_cost(stage2_0, stage2_1, site_operator):
    op = Stage3Operator([stage2_0], [stage2_1], [site_operator], [(0, 0, 0)], site_operator.shape[0])
    return op, op.cost_of_multiply()


def formDenseStage3_formMatrix_and_cost(stage2_0, stage2_1, site_operator):
    op = Stage3Operator([stage2_0], [stage2_1], [site_operator], [(0, 0, 0)], site_operator.shape[0])
    return op.formMatrix, op.cost_of_formMatrix()


def formDenseStage3(stage2_0, stage2_1, site_operator):
    """Multiplier of S2_0 (x) S2_1 (x) O (tensors/_2d/dense.py:145-203)."""
    return Stage3Operator([stage2_0], [stage2_1], [site_operator], [(0, 0, 0)], site_operator.shape[0]).multiplier()


def formNormalizationStage3(stage2_0, stage2_1, center_identity):
    """Multiplier of S2_0 (x) S2_1 (x) I (tensors/_2d/dense.py:114-144); the
    identity data only fixes the physical dimension, as in the reference."""
    return Stage3Operator([stage2_0], [stage2_1], [], [(0, 0, -1)], center_identity.shape[0]).multiplier()


def formNormalizationMultiplier(corners, sides, center_identity):
    """tensors/_2d/dense.py:82-94."""
    return formNormalizationStage3(
        formNormalizationStage2(formNormalizationStage1(corners[0], sides[0]),
                                formNormalizationStage1(corners[1], sides[1])),
        formNormalizationStage2(formNormalizationStage1(corners[2], sides[2]),
                                formNormalizationStage1(corners[3], sides[3])),
        center_identity)


def formNormalizationSubmatrix(corners, sides):
    """N_eff without the physical identity (tensors/_2d/dense.py:204-225)."""
    s2_0 = formNormalizationStage2(formNormalizationStage1(corners[0], sides[0]),
                                   formNormalizationStage1(corners[1], sides[1]))
    s2_1 = formNormalizationStage2(formNormalizationStage1(corners[2], sides[2]),
                                   formNormalizationStage1(corners[3], sides[3]))
    return Stage3Operator([s2_0], [s2_1], [], [(0, 0, -1)], 1).formMatrix()


__all__ = [
    "absorbDenseSideIntoCornerFromLeft", "absorbDenseSideIntoCornerFromRight", "absorbDenseCenterSSIntoSide",
    "absorbDenseCenterSOSIntoSide", "formDenseStage3", "formDenseStage3_formMatrix_and_cost",
    "formDenseStage3_multiply_and_cost", "formNormalizationMultiplier", "formNormalizationStage1",
    "formNormalizationStage2", "formNormalizationStage3", "formNormalizationSubmatrix", "Stage3Operator",
    "center_pair",
]
