"""Contraction planner: einsum-style specs lowered onto the grouped GETT kernel.

A spec such as ``"xyzdef,abcxyzjk->abcdjekf"`` names every axis of the two
operands and of the result.  Letters shared by both operands and absent from
the result are contracted (K), letters of one operand that survive go to M
(first operand) or N (second operand).  The result is written in place with
arbitrary strides, so the reference's ``contractWith`` followed by ``join``
(transpose + reshape) becomes a single kernel launch with no intermediate
permutation.  Adjacent axes that are contiguous in every tensor that carries
them are merged, which keeps the descriptor within the kernel's limit of six
sub-dimensions per group.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib

CDT = torch.complex128


def current_stream_handle():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class Workspace:
    """Grow-only device scratch arena, one per device.  All users enqueue on the
    current stream, so reusing the arena between consecutive launches is safe."""

    _arenas = {}

    @classmethod
    def get(cls, nbytes, device):
        nbytes = max(int(nbytes), 256)
        key = (device.type, device.index)
        buf = cls._arenas.get(key)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(int(nbytes * 1.25) + 256, dtype=torch.uint8, device=device)
            cls._arenas[key] = buf
        return buf


def _coalesce(dims):
    """dims: list of (extent, stride_x, stride_y); merge runs that are contiguous
    in both strided tensors and drop unit extents."""
    dims = [d for d in dims if d[0] != 1]
    out = []
    for e, sx, sy in dims:
        if out:
            pe, psx, psy = out[-1]
            if psx == sx * e and psy == sy * e:
                out[-1] = (pe * e, sx, sy)
                continue
        out.append((e, sx, sy))
    return out


class Spec:
    """A parsed contraction spec with per-letter extents."""

    def __init__(self, spec):
        lhs, out = spec.split("->")
        a, b = lhs.split(",")
        self.a, self.b, self.out = a, b, out
        for s in (a, b, out):
            if len(set(s)) != len(s):
                raise ValueError("repeated letter in %r" % spec)
        sa, sb, so = set(a), set(b), set(out)
        if (sa & sb & so):
            raise ValueError("batch letters are not supported: %r" % spec)
        self.m = [c for c in out if c in sa]
        self.n = [c for c in out if c in sb]
        self.k = [c for c in a if c in sb and c not in so]
        missing = so - sa - sb
        if missing:
            raise ValueError("output letters %s appear in no operand" % missing)
        dropped = (sa - sb - so) | (sb - sa - so)
        if dropped:
            raise ValueError("letters %s would be summed over one operand only" % dropped)


def _tensor_letter_strides(letters, t):
    if len(letters) != t.dim():
        raise ValueError("spec has %d letters for a rank-%d tensor" % (len(letters), t.dim()))
    return {c: (int(t.shape[i]), int(t.stride(i))) for i, c in enumerate(letters)}


def out_letter_strides(out_letters, ext):
    """Strides of a C-contiguous tensor whose axes are ``out_letters``."""
    st = {}
    s = 1
    for c in reversed(out_letters):
        st[c] = s
        s *= ext[c]
    return st


def build_desc(spec, ext, a_str, b_str, c_str, conj_a=False, conj_b=False):
    m = _coalesce([(ext[c], a_str[c], c_str[c]) for c in spec.m])
    n = _coalesce([(ext[c], b_str[c], c_str[c]) for c in spec.n])
    k = _coalesce([(ext[c], a_str[c], b_str[c]) for c in spec.k])
    if max(len(m), len(n), len(k)) > _lib.MAX_SUBDIMS:
        return None
    d = _lib.ContractDesc()
    d.nm, d.nn, d.nk = len(m), len(n), len(k)
    d.conj_a, d.conj_b = int(bool(conj_a)), int(bool(conj_b))
    for i, (e, sa, sc) in enumerate(m):
        d.m_ext[i], d.a_m[i], d.c_m[i] = e, sa, sc
    for i, (e, sb, sc) in enumerate(n):
        d.n_ext[i], d.b_n[i], d.c_n[i] = e, sb, sc
    for i, (e, sa, sb) in enumerate(k):
        d.k_ext[i], d.a_k[i], d.b_k[i] = e, sa, sb
    return d


def _extents(spec, a_ext, b_ext, extra=None):
    ext = {}
    for src in (a_ext, b_ext):
        for c, (e, _) in src.items():
            if c in ext and ext[c] != e:
                raise ValueError("dimension mismatch on index %r: %d vs %d" % (c, ext[c], e))
            ext[c] = e
    if extra:
        ext.update(extra)
    return ext


def contract_grouped(spec, a_list, b_list, out_list, entries, out_letters_shape=None, conj_a=False,
                     conj_b=False, alpha=1.0, accumulate=False):
    """Run ``out[c] (+)= alpha * sum_{(i,j,c) in entries} A[i] . B[j]`` for a spec.

    All tensors of a list share one shape.  ``out_list`` tensors must be
    C-contiguous; their axes may merge several spec letters (C order).
    """
    sp = spec if isinstance(spec, Spec) else Spec(spec)
    a0, b0, c0 = a_list[0], b_list[0], out_list[0]
    a_ls = _tensor_letter_strides(sp.a, a0)
    b_ls = _tensor_letter_strides(sp.b, b0)
    ext = _extents(sp, a_ls, b_ls)
    if not c0.is_contiguous():
        raise ValueError("output must be contiguous")
    c_str = out_letter_strides(sp.out, ext)
    total = 1
    for c in sp.out:
        total *= ext[c]
    if total != c0.numel():
        raise ValueError("output has %d elements, spec needs %d" % (c0.numel(), total))
    for t in a_list:
        if tuple(t.shape) != tuple(a0.shape) or t.stride() != a0.stride():
            raise ValueError("grouped operands must share shape and strides")
    for t in b_list:
        if tuple(t.shape) != tuple(b0.shape) or t.stride() != b0.stride():
            raise ValueError("grouped operands must share shape and strides")
    a_str = {c: s for c, (e, s) in a_ls.items()}
    b_str = {c: s for c, (e, s) in b_ls.items()}
    desc = build_desc(sp, ext, a_str, b_str, c_str, conj_a, conj_b)
    if desc is None:
        raise ValueError("contraction %r needs more than %d sub-dimensions per group" %
                         (sp.a + "," + sp.b + "->" + sp.out, _lib.MAX_SUBDIMS))
    return _launch(desc, a_list, b_list, out_list, entries, alpha, accumulate)


def _split_table(n_c, entries, limit, max_entries):
    """Calls of at most ``limit`` distinct A, B and output slots and
    ``max_entries`` entries covering a grouped table:
    [(a_idx, b_idx, c_idx, local entries, accumulate_all)].  Every output
    keeps all its entries, in their order, in one call, unless its own
    entries need more than ``limit`` A or B slots or ``max_entries`` entries;
    then its entries go to consecutive calls of that output alone, the later
    ones accumulating onto the first.  Outputs without entries are still
    written (zeroed)."""
    by_c = {}
    for e in entries:
        by_c.setdefault(int(e[2]), []).append((int(e[0]), int(e[1])))
    calls = []  # (a set, b set, outputs, global entries, accumulate)
    cur = dict(a=set(), b=set(), c=[], e=[])

    def flush():
        if cur["c"]:
            calls.append((cur["a"], cur["b"], cur["c"], cur["e"], False))
        cur.update(a=set(), b=set(), c=[], e=[])

    for c in range(n_c):
        ab = by_c.get(c, [])
        a_new, b_new = {a for a, _ in ab}, {b for _, b in ab}
        if len(a_new) > limit or len(b_new) > limit or len(ab) > max_entries:
            flush()
            part, pa, pb, first = [], set(), set(), True
            for a, b in ab:
                if len(pa | {a}) > limit or len(pb | {b}) > limit or len(part) + 1 > max_entries:
                    calls.append((pa, pb, [c], part, not first))
                    part, pa, pb, first = [], set(), set(), False
                part.append((a, b, c))
                pa.add(a)
                pb.add(b)
            calls.append((pa, pb, [c], part, not first))
            continue
        if (len(cur["a"] | a_new) > limit or len(cur["b"] | b_new) > limit or len(cur["c"]) + 1 > limit
                or len(cur["e"]) + len(ab) > max_entries):
            flush()
        cur["a"] |= a_new
        cur["b"] |= b_new
        cur["c"].append(c)
        cur["e"].extend((a, b, c) for a, b in ab)
    flush()
    out = []
    for a_set, b_set, c_idx, ents, acc in calls:
        a_idx, b_idx = sorted(a_set), sorted(b_set)
        am = {x: i for i, x in enumerate(a_idx)}
        bm = {x: i for i, x in enumerate(b_idx)}
        cm = {x: i for i, x in enumerate(c_idx)}
        out.append((a_idx, b_idx, c_idx, [(am[a], bm[b], cm[c]) for a, b, c in ents], acc))
    return out


def _launch(desc, a_list, b_list, out_list, entries, alpha=1.0, accumulate=False):
    limit = _lib.MAX_SLOTS
    if len(a_list) > limit or len(b_list) > limit or len(out_list) > limit or len(entries) > _lib.MAX_ENTRIES:
        for a_idx, b_idx, c_idx, ents, acc in _split_table(len(out_list), entries, limit, _lib.MAX_ENTRIES):
            if not ents and not a_idx:
                # outputs with no entry: the smallest operands keep the call valid
                a_idx, b_idx, ents = [0], [0], []
            _launch(desc, [a_list[i] for i in a_idx], [b_list[j] for j in b_idx], [out_list[c] for c in c_idx],
                    ents, alpha, accumulate or acc)
        return
    lib = _lib.load()
    device = out_list[0].device
    n_c = len(out_list)
    ws_bytes = lib.carc_zcontract_workspace_size(ctypes.byref(desc), n_c)
    if ws_bytes < 0:
        _lib.check(_lib.CARC_BAD_ARG)
    ws = Workspace.get(ws_bytes, device) if ws_bytes > 0 else None
    pa, _ka = _lib.ptr_array([t.data_ptr() for t in a_list])
    pb, _kb = _lib.ptr_array([t.data_ptr() for t in b_list])
    pc, _kc = _lib.ptr_array([t.data_ptr() for t in out_list])
    flat = [int(x) for e in entries for x in e]
    pe, _ke = _lib.i32_array(flat)
    alpha = complex(alpha)
    _lib.call("carc_zcontract_grouped", ctypes.byref(desc), pa, len(a_list), pb, len(b_list), pc, n_c, pe,
              len(entries), alpha.real, alpha.imag, int(bool(accumulate)),
              ctypes.c_void_p(ws.data_ptr() if ws is not None else 0), int(ws_bytes if ws is not None else 0),
              current_stream_handle())


def contract_grouped_tc(spec, a_list, b_list, out_list, entries, conj_a=False, conj_b=False, accumulate=False,
                        grouped=True):
    """``out[c] (+)= sum_{(i,j,c) in entries} A[i] . B[j]`` with every pair on
    the tensor cores (operands split into BF16 hi + lo, FP32 accumulation,
    FP64 reduction; ~1e-5 relative to the result's scale).  Same spec and
    layout rules as ``contract_grouped``.  The whole table is one grouped call
    (``carc_zcontract_tc_grouped``: each distinct operand packed once, one
    grouped GEMM over (entry, tile, split), one grouped reduction) when it
    fits the library's table limits (and ``grouped``), else one
    ``carc_zcontract_tc`` per entry.  Returns the device int32 status words (one per call; each call
    clears its own word and sets it on a pipeline timeout); the caller checks
    them."""
    sp = spec if isinstance(spec, Spec) else Spec(spec)
    a0, b0, c0 = a_list[0], b_list[0], out_list[0]
    a_ls = _tensor_letter_strides(sp.a, a0)
    b_ls = _tensor_letter_strides(sp.b, b0)
    ext = _extents(sp, a_ls, b_ls)
    for t in out_list:
        if not t.is_contiguous() or tuple(t.shape) != tuple(c0.shape):
            raise ValueError("outputs must be contiguous and of one shape")
    for lst, t0 in ((a_list, a0), (b_list, b0)):
        for t in lst:
            if tuple(t.shape) != tuple(t0.shape) or t.stride() != t0.stride():
                raise ValueError("grouped operands must share shape and strides")
    c_str = out_letter_strides(sp.out, ext)
    desc = build_desc(sp, ext, {c: s for c, (e, s) in a_ls.items()}, {c: s for c, (e, s) in b_ls.items()}, c_str,
                      conj_a, conj_b)
    if desc is None:
        raise ValueError("contraction %r needs more than %d sub-dimensions per group" %
                         (sp.a + "," + sp.b + "->" + sp.out, _lib.MAX_SUBDIMS))
    lib = _lib.load()
    if (grouped and entries and len(a_list) <= _lib.MAX_SLOTS and len(b_list) <= _lib.MAX_SLOTS
            and len(out_list) <= _lib.MAX_SLOTS and len(entries) <= _lib.MAX_ENTRIES):
        ws_bytes = lib.carc_zcontract_tc_grouped_workspace_size(ctypes.byref(desc), len(a_list), len(b_list),
                                                                 len(entries))
        if ws_bytes < 0:
            _lib.check(_lib.CARC_BAD_ARG)
        ws = Workspace.get(ws_bytes, c0.device)
        status = torch.zeros(1, dtype=torch.int32, device=c0.device)
        pa, _ka = _lib.ptr_array([t.data_ptr() for t in a_list])
        pb, _kb = _lib.ptr_array([t.data_ptr() for t in b_list])
        pc, _kc = _lib.ptr_array([t.data_ptr() for t in out_list])
        pe, _ke = _lib.i32_array([int(x) for e in entries for x in e])
        _lib.call("carc_zcontract_tc_grouped", ctypes.byref(desc), pa, len(a_list), pb, len(b_list), pc,
                  len(out_list), pe, len(entries), 1.0, 0.0, int(bool(accumulate)), ctypes.c_void_p(ws.data_ptr()),
                  ws_bytes, ctypes.c_void_p(status.data_ptr()), current_stream_handle())
        return status
    ws_bytes = lib.carc_zcontract_tc_workspace_size(ctypes.byref(desc), 0)
    if ws_bytes < 0:
        _lib.check(_lib.CARC_BAD_ARG)
    ws = Workspace.get(ws_bytes, c0.device)
    status = torch.zeros(max(1, len(entries)), dtype=torch.int32, device=c0.device)
    seen = set()
    for k, (i, j, c) in enumerate(entries):
        acc = accumulate or c in seen
        seen.add(c)
        _lib.call("carc_zcontract_tc", ctypes.byref(desc), ctypes.c_void_p(a_list[i].data_ptr()),
                  ctypes.c_void_p(b_list[j].data_ptr()), ctypes.c_void_p(out_list[c].data_ptr()), 1.0, 0.0,
                  int(acc), 0, ctypes.c_void_p(ws.data_ptr()), ws_bytes, ctypes.c_void_p(status[k].data_ptr()),
                  current_stream_handle())
    return status


def contract(spec, a, b, out_shape, conj_a=False, conj_b=False, alpha=1.0):
    """Single contraction; returns a new C-contiguous tensor of ``out_shape``."""
    out = torch.empty(tuple(int(x) for x in out_shape), dtype=CDT, device=a.device)
    contract_grouped(spec, [a], [b], [out], [(0, 0, 0)], conj_a=conj_a, conj_b=conj_b, alpha=alpha)
    return out


def permute(t, perm, conj=False):
    """C-contiguous copy of t.permute(perm) (optionally conjugated)."""
    perm = list(perm)
    shape = [int(t.shape[p]) for p in perm]
    out = torch.empty(shape, dtype=CDT, device=t.device)
    if out.numel() == 0:
        return out
    # merge runs of output axes that stay adjacent and contiguous in the input
    dims = []
    for p in perm:
        e, s = int(t.shape[p]), int(t.stride(p))
        if e == 1:
            continue
        if dims and dims[-1][1] == s * e:
            dims[-1] = (dims[-1][0] * e, s)
        else:
            dims.append((e, s))
    if not dims:
        dims = [(1, 0)]
    pshape, _k1 = _lib.i64_array([d[0] for d in dims])
    pstr, _k2 = _lib.i64_array([d[1] for d in dims])
    _lib.call("carc_zpermute", ctypes.c_void_p(t.data_ptr()), ctypes.c_void_p(out.data_ptr()), len(dims), pshape,
              pstr, int(bool(conj)), current_stream_handle())
    return out
