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


# Precision of the absorptions (corner <- side, side <- center; contractTowards):
# "fp64" (default: the FP64 grouped GETT, the parity path) or "tc" (every
# tag pair on the tensor cores with split-BF16 operands, ~1e-5 relative to
# the absorbed tensor's scale).  The environment built by "tc" absorptions
# carries that error into every later energy; set it with
# ``absorption_precision(...)``.
_ABSORPTION = {"precision": "fp64", "status": []}


class absorption_precision:
    """Context manager selecting the absorptions' precision ("fp64" or "tc");
    on exit the tensor-core status words are checked."""

    def __init__(self, precision):
        if precision not in ("fp64", "tc"):
            raise ValueError("absorption precision must be 'fp64' or 'tc', not %r" % (precision,))
        self.precision = precision
        self.previous = None

    def __enter__(self):
        self.previous = _ABSORPTION["precision"]
        _ABSORPTION["precision"] = self.precision
        return self

    def __exit__(self, *exc):
        _ABSORPTION["precision"] = self.previous
        check_absorption_status()
        return False


def check_absorption_status():
    """Read the status words of the tensor-core absorptions run so far (one
    device synchronisation) and raise if a pipeline wait timed out."""
    st, _ABSORPTION["status"] = _ABSORPTION["status"], []
    if st:
        vals = torch.cat([t.reshape(-1) for t in st]).cpu()
        if int(vals.abs().max()) != 0:
            raise _lib.CarcNotConverged(int(vals.abs().max()), "tensor-core absorption: a pipeline wait timed out")


def _contract(spec, a_list, b_list, out_list, entries, accumulate, tc):
    if tc and _ABSORPTION["precision"] == "tc":
        _ABSORPTION["status"].append(engine.contract_grouped_tc(spec, a_list, b_list, out_list, entries,
                                                                accumulate=accumulate))
    else:
        engine.contract_grouped(spec, a_list, b_list, out_list, entries, accumulate=accumulate)


class _PairContractor:
    """A two-operand contractor given by a spec and an output-shape rule;
    ``tc``: an absorption, run on the tensor cores under absorption_precision("tc")."""

    def __init__(self, name, spec, ranks, joins, shape_fn, doc, tc=False):
        self.__name__ = name
        self.spec = engine.Spec(spec)
        self.ranks = ranks
        self.joins = joins          # [(operand, axis, operand, axis)] dimension checks
        self.shape_fn = shape_fn
        self.__doc__ = doc
        self.tc = tc

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
        _contract(self.spec, [ta], [tb], [out], [(0, 0, 0)], False, self.tc)
        return TorchData(out)

    def grouped(self, list_a, list_b, table, n_out):
        """All (i, j, slot) pairs of a sparse contraction.  Pairs are launched
        together per operand-shape class (tags of one boundary may differ in
        shape, e.g. a compressed operator axis); a slot reached by several
        launches accumulates, in table order within each launch."""
        ta = [_t(x) for x in list_a]
        tb = [_t(x) for x in list_b]
        classes = {}
        for e in table:
            key = (tuple(ta[e[0]].shape), tuple(tb[e[1]].shape))
            classes.setdefault(key, []).append(e)
        outs = [None] * n_out
        for (sa, sb), entries in classes.items():
            a0 = next(ta[e[0]] for e in entries)
            b0 = next(tb[e[1]] for e in entries)
            self._validate(a0, b0)
            shape = self.shape_fn(a0.shape, b0.shape)
            for lo in range(0, len(entries), _lib.MAX_ENTRIES):
                chunk = entries[lo:lo + _lib.MAX_ENTRIES]
                used_a = sorted({e[0] for e in chunk})
                used_b = sorted({e[1] for e in chunk})
                used_c = sorted({e[2] for e in chunk})
                written = [outs[c] is not None for c in used_c]
                for c in used_c:
                    if outs[c] is None:
                        outs[c] = TorchData.newZeros(shape)._t
                    elif tuple(outs[c].shape) != tuple(shape):
                        raise ValueError("operands could not be broadcast together with shapes %s %s"
                                         % (tuple(outs[c].shape), tuple(shape)))
                ma = {v: i for i, v in enumerate(used_a)}
                mb = {v: i for i, v in enumerate(used_b)}
                mc = {v: i for i, v in enumerate(used_c)}
                single = len(classes) == 1 and lo == 0
                _contract(self.spec, [ta[i] for i in used_a], [tb[i] for i in used_b], [outs[i] for i in used_c],
                          [(ma[i], mb[j], mc[k]) for i, j, k in chunk], not single or any(written), self.tc)
        return [TorchData(o) for o in outs]


absorbDenseSideIntoCornerFromLeft = _PairContractor(
    "absorbDenseSideIntoCornerFromLeft", "xyzdef,abcxyzjk->abcdjekf", (6, 8),
    [(0, 0, 1, 3), (0, 1, 1, 4), (0, 2, 1, 5)],
    lambda c, s: (s[0], s[1], s[2], c[3] * s[6], c[4] * s[7], c[5]),
    "C'[a,b,c,(d,j),(e,k),f] = sum C[x,y,z,d,e,f] T[a,b,c,x,y,z,j,k]  (tensors/_2d/dense.py:10-15)", tc=True)

absorbDenseSideIntoCornerFromRight = _PairContractor(
    "absorbDenseSideIntoCornerFromRight", "abcxyz,xyzghijk->ajbkcghi", (6, 8),
    [(0, 3, 1, 0), (0, 4, 1, 1), (0, 5, 1, 2)],
    lambda c, s: (c[0] * s[6], c[1] * s[7], c[2], s[3], s[4], s[5]),
    "C'[(a,j),(b,k),c,g,h,i] = sum C[a,b,c,x,y,z] T[x,y,z,g,h,i,j,k]  (tensors/_2d/dense.py:16-21)", tc=True)

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


def center_pairs(direction, state, ops, state_conj=None):
    """``[center_pair(direction, state, op, state_conj) for op in ops]`` in two
    grouped launches (every S . O, then every pair with conj(S)) instead of one
    or two per operator; operators whose shape does not keep the center's
    physical dimension take the single path."""
    s = _t(state)
    _check_rank(1, s, 5)
    conj = state_conj is None
    sc = s if conj else _t(state_conj)
    ts = [None if op is None else _t(op) for op in ops]
    for o in ts:
        if o is not None:
            _check_rank(3, o, 2)
            if o.shape[1] != s.shape[4]:
                raise DimensionMismatchError(3, 1, int(o.shape[1]), 1, 4, int(s.shape[4]))
    real = [o for o in ts if o is not None]
    if any(o.shape[0] != s.shape[4] for o in real) or len({(tuple(o.shape), o.stride()) for o in real}) > 1:
        return [center_pair(direction, state, op, state_conj) for op in ops]
    ket = _center_letters(direction, True)
    bra = _center_letters(direction, False)
    so = [torch.empty(tuple(s.shape), dtype=CDT, device=s.device) for _ in real]
    if real:
        engine.contract_grouped(ket + ",pq->" + ket[:4] + "p", [s], real, so, [(0, i, i) for i in range(len(real))])
    a_list, entries, k = [s.contiguous()] + so, [], 0  # grouped operands share strides
    for i, o in enumerate(ts):
        if o is None:
            entries.append((0, 0, i))
        else:
            k += 1
            entries.append((k, 0, i))
    ext = {c: int(s.shape[i]) for i, c in enumerate(ket[:4])}
    ext.update({c: int(sc.shape[i]) for i, c in enumerate(bra[:4])})
    shape = tuple(ext[c] for c in "uvwxyzkl")
    outs = [torch.empty(shape, dtype=CDT, device=s.device) for _ in ts]
    engine.contract_grouped(ket[:4] + "p," + bra[:4] + "p->uvwxyzkl", a_list, [sc], outs, entries, conj_b=conj)
    return outs


_SIDE_SPEC = engine.Spec("abcdefkl,uvwxyzkl->aubxcdveyfwz")


def _side_out_shape(side_shape, e_shape):
    a, b, c, d, e, f = side_shape[:6]
    u, v, w, x, y, z = e_shape[:6]
    return (a * u, b * x, c, d * v, e * y, f, w, z)


def _absorb_pairs(direction, sides, pairs_e, table, n_out):
    """Grouped side (x) center-pair contractions; launched per side-shape class
    (a compressed operator tag has its own shape), slots accumulating."""
    ts = [_t(x) for x in sides]
    for t in ts:
        _check_rank(0, t, 8)
    e0 = pairs_e[0]
    classes = {}
    for e in table:
        classes.setdefault(tuple(ts[e[0]].shape), []).append(e)
    outs = [None] * n_out
    for sshape, entries in classes.items():
        if sshape[6] != e0.shape[6]:
            raise DimensionMismatchError(0, 6, int(sshape[6]), 1, direction, int(e0.shape[6]))
        if sshape[7] != e0.shape[7]:
            raise DimensionMismatchError(0, 7, int(sshape[7]), 2, direction, int(e0.shape[7]))
        shape = _side_out_shape(sshape, e0.shape)
        used_s = sorted({e[0] for e in entries})
        used_c = sorted({e[2] for e in entries})
        written = any(outs[c] is not None for c in used_c)
        for c in used_c:
            if outs[c] is None:
                outs[c] = TorchData.newZeros(shape)._t if len(classes) > 1 else \
                    torch.empty(shape, dtype=CDT, device=ts[0].device)
        ms = {v: i for i, v in enumerate(used_s)}
        mc = {v: i for i, v in enumerate(used_c)}
        _contract(_SIDE_SPEC, [ts[i] for i in used_s], pairs_e, [outs[c] for c in used_c],
                  [(ms[i], j, mc[k]) for i, j, k in entries], len(classes) > 1 or written, True)
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
        for t in self.s2_0:
            _check_rank(0, t, 6)
        for t in self.s2_1:
            _check_rank(1, t, 6)
        for i0, i1, _ in self.terms:
            a, b = self.s2_0[i0], self.s2_1[i1]
            if a.shape[0] != b.shape[1]:
                raise DimensionMismatchError(0, 0, int(a.shape[0]), 1, 1, int(b.shape[1]))
            if a.shape[1] != b.shape[0]:
                raise DimensionMismatchError(0, 1, int(a.shape[1]), 1, 0, int(b.shape[0]))
        ref0 = self.s2_0[self.terms[0][0]] if self.terms else self.s2_0[0]
        ref1 = self.s2_1[self.terms[0][1]] if self.terms else self.s2_1[0]
        self.s0_shape = tuple(int(x) for x in ref0.shape)
        self.s1_shape = tuple(int(x) for x in ref1.shape)
        k0, k1, l0, l1 = self.s0_shape[2:6]
        k2, k3, l2, l3 = self.s1_shape[2:6]
        self.in_shape = (k0, k1, k2, k3, self.d)
        self.out_shape = (l0, l1, l2, l3, self.d)
        self.device = ref0.device
        self._pack()

    def _pack(self):
        """One library call per shape class of (S2_0, S2_1) pairs (the stage-2
        tags of a boundary differ in shape only through a compressed operator
        axis), split where a class has more tags of either half or more terms
        than one call takes; every call after the first accumulates."""
        classes = {}
        for t in self.terms:
            key = (tuple(self.s2_0[t[0]].shape), tuple(self.s2_1[t[1]].shape))
            classes.setdefault(key, []).append(t)
        if len(self.ops) > _lib.MAX_SLOTS:
            raise ValueError("stage 3: %d operator tags, more than the %d one call takes" %
                             (len(self.ops), _lib.MAX_SLOTS))
        chunks = []
        for key, terms in classes.items():
            cur, s0, s1 = [], set(), set()
            for t in terms:
                if cur and (len(s0 | {t[0]}) > _lib.MAX_SLOTS or len(s1 | {t[1]}) > _lib.MAX_SLOTS
                            or len(cur) + 1 > _lib.MAX_ENTRIES):
                    chunks.append((key, cur))
                    cur, s0, s1 = [], set(), set()
                cur.append(t)
                s0.add(t[0])
                s1.add(t[1])
            chunks.append((key, cur))
        self._groups = []
        self._po, self._ko = _lib.ptr_array([t.data_ptr() for t in self.ops])
        for (sh0, sh1), terms in chunks:
            i0s = sorted({t[0] for t in terms})
            i1s = sorted({t[1] for t in terms})
            m0 = {v: i for i, v in enumerate(i0s)}
            m1 = {v: i for i, v in enumerate(i1s)}
            g = dict(shape0=sh0, shape1=sh1, n0=len(i0s), n1=len(i1s),
                     terms=[(m0[a], m1[b], c) for a, b, c in terms])
            g["p0"], g["k0"] = _lib.ptr_array([self.s2_0[i].data_ptr() for i in i0s])
            g["p1"], g["k1"] = _lib.ptr_array([self.s2_1[i].data_ptr() for i in i1s])
            g["pt"], g["kt"] = _lib.i32_array([v for t in g["terms"] for v in t])
            g["s0"], g["ks0"] = _lib.i64_array(sh0)
            g["s1"], g["ks1"] = _lib.i64_array(sh1)
            self._groups.append(g)

    @property
    def n(self):
        return int(np.prod(self.out_shape))

    def cost_of_multiply(self):
        return sum(stage3_multiply_cost(self.s2_0[i0].shape, self.s2_1[i1].shape, self.d, io < 0)
                   for i0, i1, io in self.terms)

    def cost_of_formMatrix(self):
        return sum(stage3_form_matrix_cost(self.s2_0[i0].shape, self.s2_1[i1].shape, self.d)
                   for i0, i1, _ in self.terms)

    # -- tensor-core (split-BF16) path --------------------------------------
    def _tc_plan(self, g):
        """Packed split-BF16 copies of this class's S2 tags (built once)."""
        if "plan" not in g:
            lib = _lib.load()
            nbytes = lib.carc_stage3_tc_plan_size(g["s0"], g["s1"], g["pt"], len(g["terms"]))
            if nbytes < 0:
                _lib.check(_lib.CARC_BAD_SHAPE)
            g["plan"] = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=self.device)
            _lib.call("carc_stage3_tc_prepare", g["s0"], g["s1"], g["p0"], g["n0"], g["p1"], g["n1"], g["pt"],
                      len(g["terms"]), ctypes.c_void_p(g["plan"].data_ptr()), nbytes, current_stream_handle())
        return g["plan"]

    def _status(self):
        if not hasattr(self, "_tc_status"):
            self._tc_status = torch.zeros((), dtype=torch.int32, device=self.device)
        return self._tc_status

    def check_status(self):
        """Raise if a tensor-core pipeline wait timed out in an earlier call (syncs)."""
        if hasattr(self, "_tc_status") and int(self._tc_status.item()) != 0:
            raise _lib.CarcError(_lib.CARC_NOT_CONVERGED, "tensor-core pipeline wait timed out")

    def apply_tc(self, x, y=None, nvec=1, accumulate=False):
        """y = op . x on the tensor cores (split-BF16 operands, ~1e-5 relative)."""
        x = x.contiguous()
        if y is None:
            y = torch.empty((nvec,) + self.out_shape if nvec > 1 else self.out_shape, dtype=CDT, device=x.device)
        self.apply_tc_ptr(x.data_ptr(), y.data_ptr(), nvec, accumulate)
        return y

    def apply_tc_ptr(self, x_ptr, y_ptr, nvec=1, accumulate=False):
        """``apply_tc`` on raw device addresses of nvec contiguous centers:
        device memory, or pinned host memory mapped into the device's address
        space (``carc_host_alloc_mapped``), which the kernels then read and
        write directly over the host link."""
        lib = _lib.load()
        if not self._groups:
            if not accumulate:
                n = nvec * int(np.prod(self.out_shape))
                _lib.call("carc_zfill", n, 0.0, 0.0, ctypes.c_void_p(int(y_ptr)), current_stream_handle())
            return
        st = self._status()
        for gi, g in enumerate(self._groups):
            plan = self._tc_plan(g)
            ws_bytes = lib.carc_stage3_matvec_tc_workspace_size(g["s0"], g["s1"], self.d, g["pt"], len(g["terms"]),
                                                                nvec)
            if ws_bytes < 0:
                _lib.check(_lib.CARC_BAD_SHAPE)
            ws = engine.Workspace.get(ws_bytes, self.device)
            _lib.call("carc_stage3_matvec_tc", g["s0"], g["s1"], self.d, ctypes.c_void_p(plan.data_ptr()), g["n0"],
                      g["n1"], self._po, len(self.ops), g["pt"], len(g["terms"]), ctypes.c_void_p(int(x_ptr)),
                      ctypes.c_void_p(int(y_ptr)), nvec, int(bool(accumulate or gi > 0)),
                      ctypes.c_void_p(ws.data_ptr()), ws_bytes, ctypes.c_void_p(st.data_ptr()),
                      current_stream_handle())

    def form_matrix_tc(self, out=None, accumulate=False):
        """H on the tensor cores (split-BF16 operands, ~1e-5 relative)."""
        lib = _lib.load()
        n_r, n_c = self.n, int(np.prod(self.in_shape))
        if out is None:
            out = torch.empty((n_r, n_c), dtype=CDT, device=self.device)
        if not self._groups:
            if not accumulate:
                _lib.call("carc_zfill", out.numel(), 0.0, 0.0, ctypes.c_void_p(out.data_ptr()), current_stream_handle())
            return out
        st = self._status()
        for gi, g in enumerate(self._groups):
            ws_bytes = lib.carc_stage3_form_matrix_tc_workspace_size(g["s0"], g["s1"], self.d, len(g["terms"]))
            if ws_bytes < 0:
                _lib.check(_lib.CARC_BAD_SHAPE)
            ws = engine.Workspace.get(ws_bytes, self.device)
            _lib.call("carc_stage3_form_matrix_tc", g["s0"], g["s1"], self.d, g["p0"], g["n0"], g["p1"], g["n1"],
                      self._po, len(self.ops), g["pt"], len(g["terms"]), ctypes.c_void_p(out.data_ptr()),
                      int(bool(accumulate or gi > 0)), ctypes.c_void_p(ws.data_ptr()), ws_bytes,
                      ctypes.c_void_p(st.data_ptr()), current_stream_handle())
        return out

    def apply(self, x, y=None, nvec=1, accumulate=False):
        """y = op . x for nvec stacked centers (torch tensors, contiguous)."""
        lib = _lib.load()
        x = x.contiguous()
        if y is None:
            y = torch.empty((nvec,) + self.out_shape if nvec > 1 else self.out_shape, dtype=CDT, device=x.device)
        if not self._groups:
            if not accumulate:
                _lib.call("carc_zfill", y.numel(), 0.0, 0.0, ctypes.c_void_p(y.data_ptr()), current_stream_handle())
            return y
        for gi, g in enumerate(self._groups):
            ws_bytes = lib.carc_stage3_matvec_f64_workspace_size(g["s0"], g["s1"], self.d, len(g["terms"]), nvec)
            if ws_bytes < 0:
                _lib.check(_lib.CARC_BAD_SHAPE)
            ws = engine.Workspace.get(ws_bytes, x.device)
            _lib.call("carc_stage3_matvec_f64", g["s0"], g["s1"], self.d, g["p0"], g["n0"], g["p1"], g["n1"],
                      self._po, len(self.ops), g["pt"], len(g["terms"]), ctypes.c_void_p(x.data_ptr()),
                      ctypes.c_void_p(y.data_ptr()), nvec, int(bool(accumulate or gi > 0)),
                      ctypes.c_void_p(ws.data_ptr()), ws_bytes, current_stream_handle())
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
        if not self._groups:
            if not accumulate:
                _lib.call("carc_zfill", out.numel(), 0.0, 0.0, ctypes.c_void_p(out.data_ptr()), current_stream_handle())
            return out
        for gi, g in enumerate(self._groups):
            ws_bytes = lib.carc_stage3_form_matrix_f64_workspace_size(g["s0"], g["s1"], self.d, len(g["terms"]))
            if ws_bytes < 0:
                _lib.check(_lib.CARC_BAD_SHAPE)
            ws = engine.Workspace.get(ws_bytes, self.device)
            _lib.call("carc_stage3_form_matrix_f64", g["s0"], g["s1"], self.d, g["p0"], g["n0"], g["p1"], g["n1"],
                      self._po, len(self.ops), g["pt"], len(g["terms"]), ctypes.c_void_p(out.data_ptr()),
                      int(bool(accumulate or gi > 0)), ctypes.c_void_p(ws.data_ptr()), ws_bytes,
                      current_stream_handle())
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
    "center_pair", "center_pairs", "absorption_precision", "check_absorption_status",
]
