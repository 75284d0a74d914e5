"""Boundary compression: computeProductCompressor (compression.py:11-46).

Finds an isometry P (old x new) such that inserting P P^H between the two
halves L (l,old,old,op) and R (old,old,op,r) of a boundary reproduces L.R,
by four rounds of: form the normal equations A^H A x = A^H b of the linear
map A(P) of the reference's five-tensor contractor, solve them, and take the
polar factor of x.  Returns P^T (new, old).

The reference forms A (l r x old new) explicitly and solves by GMRES.  Here
A is never formed: with t1 = L . conj(P) and t3 = conj(P) . P . R (the two
halves of the reference's contractor),
    G = A^H A = sum_{o,j,o',j'} (t1^H t1)[a,o,j; a',o',j'] (t3^H t3)[i,j,o; i',j',o'],
    A^H b = t1^H . (t3^H . b),
which costs l (old op new)^2 + r (new^2 op)^2 + (old new)^2 (op new)^2
complex MACs per round instead of the l r (old new)^2 of A^H A (at a
boundary of l = 1024, r = 64, old = 32, new = 8: 7e7 instead of 4.3e9).
The system (Hermitian positive semi-definite and consistent) is solved on
the GPU by conjugate gradients to a relative residual of 1e-12 in one
cooperative launch per round (``carc_zcg_hpsd_grid``, no host round trip per
iteration); the four rounds' status words (CG and the polar factors'
Jacobi SVDs) are read once at the end, and a solve that ends its budget above
the reference's GMRES tolerance (1e-5) raises AssertionError where GMRES
would report non-convergence (compression.py:43).  Systems larger than the single-block
solver takes fall back to a CG driven from the host, one launch per step.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib, engine, linalg
from .data import TorchData
from .engine import CDT, current_stream_handle

CG_MAX_N = 2048  # CARC_CG_MAX_N
# CG aims at a relative residual of 1e-12; when it stalls above that within its
# budget (singular or ill-conditioned normal equations stop near cond(G) u),
# the solve is accepted below the reference's own GMRES tolerance (scipy's
# default rtol 1e-5, compression.py:38-43), and is an error above it
ACCEPT_RESIDUAL = 1e-5


# Precision of the normal equations' contractions: "fp64" (the parity path)
# or "tc" (every contraction on the tensor cores with split-BF16 operands,
# ~1e-5 relative, the size of the reference's own GMRES tolerance); set it
# with ``compression_precision(...)``.
_PRECISION = {"precision": "fp64", "status": []}


class compression_precision:
    """Context manager selecting the compressor's contraction precision
    ("fp64" or "tc"); on exit the tensor-core status words are checked."""

    def __init__(self, precision):
        if precision not in ("fp64", "tc"):
            raise ValueError("compression precision must be 'fp64' or 'tc', not %r" % (precision,))
        self.precision = precision
        self.previous = None

    def __enter__(self):
        self.previous = _PRECISION["precision"]
        _PRECISION["precision"] = self.precision
        return self

    def __exit__(self, *exc):
        _PRECISION["precision"] = self.previous
        st, _PRECISION["status"] = _PRECISION["status"], []
        if st and int(torch.cat([t.reshape(-1) for t in st]).abs().max().item()) != 0:
            raise _lib.CarcNotConverged(_lib.CARC_NOT_CONVERGED, "tensor-core compression: a pipeline wait timed out")
        return False


def _ct(spec, a, b, out_shape, conj_a=False, conj_b=False, big=False):
    """One contraction of the normal equations; the big ones (``big``) go to
    the tensor cores in "tc" mode."""
    if big and _PRECISION["precision"] == "tc":
        out = torch.empty(tuple(int(x) for x in out_shape), dtype=CDT, device=a.device)
        _PRECISION["status"].append(engine.contract_grouped_tc(spec, [a], [b], [out], [(0, 0, 0)], conj_a=conj_a,
                                                               conj_b=conj_b))
        return out
    return engine.contract(spec, a, b, out_shape, conj_a=conj_a, conj_b=conj_b)


def absorb_matrices(sparse, ax1, M1, ax2, M2):
    """``{tag: d.absorbMatrixAt(ax1, M1).absorbMatrixAt(ax2, M2)}`` over a
    sparse boundary (the compressor's application in
    compressCornerStateTowards, system/_2d.py:191-228).  In the "tc" mode of
    ``compression_precision`` every tag of one shape takes one grouped
    tensor-core call per matrix (the tags are the B operands of M . d over
    the axis); otherwise each tag its FP64 contractions."""
    from .data import LETTERS
    if _PRECISION["precision"] != "tc":
        return {t: d.absorbMatrixAt(ax1, M1).absorbMatrixAt(ax2, M2) for t, d in sparse.items()}
    classes = {}
    for t, d in sparse.items():
        classes.setdefault((tuple(d.shape), tuple(d._t.stride())), []).append(t)
    out = {}
    for (shape, _), tags in classes.items():
        ts = [sparse[t]._t for t in tags]
        for axis, M in ((ax1, M1), (ax2, M2)):
            m = M._t if isinstance(M, TorchData) else torch.as_tensor(M)
            n = len(ts[0].shape)
            la = LETTERS[:n]
            o = list(la)
            o[axis] = "Z"
            spec = "Z" + la[axis] + "," + la + "->" + "".join(o)
            shp = list(ts[0].shape)
            if m.shape[1] != shp[axis]:
                raise ValueError("shape-mismatch for sum")
            shp[axis] = m.shape[0]
            outs = [torch.empty(shp, dtype=CDT, device=ts[0].device) for _ in ts]
            _PRECISION["status"].append(engine.contract_grouped_tc(spec, [m.contiguous()], ts, outs,
                                                                   [(0, i, i) for i in range(len(ts))]))
            ts = outs
        out.update({t: TorchData(x) for t, x in zip(tags, ts)})
    return {t: out[t] for t in sparse}


def _normal_equations(Lt, Rt, P, b2):
    """G = A^H A and c = A^H b of A[(l,r),(a,i)] = sum L[l,a,b,o] conj(P[b,j])
    conj(P[c,i]) P[e,j] R[c,e,o,r] (the reference's join list, compression.py:12-25),
    through the factors t1 and t3 of A."""
    l, old, _, op = Lt.shape
    r = Rt.shape[3]
    new = P.shape[1]
    n = old * new
    # the terms with the long boundary index l (t1, X, u, c, and b2 above)
    # carry almost all of the work; the rest stay in FP64
    t1 = _ct("labo,bj->laoj", Lt, P, (l, old, op, new), conj_b=True, big=True)
    t2 = _ct("ej,ceor->jcor", P, Rt, (new, old, op, r))
    t3 = _ct("ci,jcor->ijor", P, t2, (new, new, op, r), conj_a=True)
    X = _ct("laoj,lbpk->aojbpk", t1, t1, (old, op, new, old, op, new), conj_a=True, big=True)
    Y = _ct("ijor,xkpr->ijoxkp", t3, t3, (new, new, op, new, new, op), conj_a=True)
    G = _ct("aojbpk,ijoxkp->aibx", X, Y, (old, new, old, new)).reshape(n, n)
    if _PRECISION["precision"] == "tc":
        # the split-precision X is Hermitian only to its rounding: so is G
        G = TorchData(G)._axpby(0.5, TorchData(G), 0.5, TorchData(engine.permute(G, (1, 0), conj=True)))._t
    u = _ct("ijor,lr->lijo", t3, b2, (l, new, new, op), conj_a=True, big=True)
    c = _ct("laoj,lijo->ai", t1, u, (old, new), conj_a=True, big=True).reshape(n)
    return G, c


def _dot(x, y):
    return TorchData(x)._dot(TorchData(y))


def _cg_host(G, c, tol=1e-12, max_iter=None):
    """Conjugate gradients on G x = c from x = 0 (G Hermitian PSD, device), one
    launch per step, for systems above the single-block solver's size.  As
    the device solver: the iterate with the smallest residual is kept, the
    iteration stops once the residual is 1e8 above that best (a rounding-level
    part of c outside the range of a singular G makes the iterates grow
    without bound), and that iterate's true residual decides acceptance."""
    n = c.numel()
    max_iter = max_iter or max(4 * n, 50)
    x = torch.zeros(n, dtype=CDT, device=c.device)
    r = c.clone()
    p = r.clone()
    rr = float(_dot(r, r).real.item())
    c2 = rr
    if c2 == 0.0:
        return x
    best, xb = rr, x
    for it in range(max_iter):
        Gp = engine.contract("pq,q->p", G, p, (n,))
        pGp = float(_dot(p, Gp).real.item())
        if pGp <= 0.0:
            break
        alpha = rr / pGp
        x = TorchData(x)._axpby(1.0, TorchData(x), alpha, TorchData(p))._t
        r = TorchData(r)._axpby(1.0, TorchData(r), -alpha, TorchData(Gp))._t
        rr_new = float(_dot(r, r).real.item())
        if rr_new < best:
            best, xb = rr_new, x
        if rr_new <= tol * tol * c2 or rr_new > 1e8 * best:
            break
        p = TorchData(r)._axpby(1.0, TorchData(r), rr_new / rr, TorchData(p))._t
        rr = rr_new
    res = TorchData(c)._axpby(1.0, TorchData(c), -1.0, TorchData(engine.contract("pq,q->p", G, xb, (n,))))._t
    true_res = float(_dot(res, res).real.item()) ** 0.5 / c2 ** 0.5
    if true_res <= max(tol, ACCEPT_RESIDUAL):
        return xb
    raise AssertionError("normal equations of the product compressor did not converge "
                         "(residual %.3e after %d iterations)" % (true_res, it + 1))


def _cg_device(G, c, status, residual, tol=1e-12, max_iter=None):
    """CG on the device with no host round trip: over a cooperative grid
    (``carc_zcg_hpsd_grid``: G p spread over the SMs, a few microseconds per
    iteration) -- FP64 issues slowly on this part, and on one SM alone an
    iteration costs n^2 complex multiply-adds at a sixty-fourth of the GPU's
    FP64 rate."""
    n = c.numel()
    max_iter = max_iter or max(10 * n, 500)  # iterations are cheap: ill-conditioned systems need more
    x = torch.empty(n, dtype=CDT, device=c.device)
    ws_bytes = _lib.load().carc_zcg_hpsd_grid_workspace_size(n)
    ws = engine.Workspace.get(ws_bytes, c.device)
    _lib.call("carc_zcg_hpsd_grid", n, ctypes.c_void_p(G.data_ptr()), ctypes.c_void_p(c.data_ptr()),
              ctypes.c_void_p(x.data_ptr()), float(tol), int(max_iter), ctypes.c_void_p(status.data_ptr()),
              ctypes.c_void_p(residual.data_ptr()), ctypes.c_void_p(ws.data_ptr()), ws_bytes,
              current_stream_handle())
    return x


def computeProductCompressor(L, R, new_dimension, rounds=4, initial=None):
    if L.shape[1] != L.shape[2]:
        raise ValueError("left inward dimensions do not match (given " + str(L.shape) + ")")
    if R.shape[0] != R.shape[1]:
        raise ValueError("right inward dimensions do not match (given " + str(R.shape) + ")")
    if L.shape[1] != R.shape[1]:
        raise ValueError("left and right shapes are incompatible (given " + str(L.shape) + " and " + str(R.shape) + ")")
    old = L.shape[1]
    Lt = L._t.contiguous()
    Rt = R._t.contiguous()
    l, r = Lt.shape[0], Rt.shape[3]
    b2 = _ct("labo,abor->lr", Lt, Rt, (l, r), big=True)
    if initial is None:
        initial = TorchData.newRandom(old, new_dimension)  # numpy's global generator, as the reference
    svd_status = []
    P = linalg.unitize(initial if isinstance(initial, TorchData) else TorchData(np.asarray(initial)),
                       deferred=svd_status)
    n = old * new_dimension
    on_device = n <= CG_MAX_N
    if on_device:
        status = torch.zeros((rounds, 2), dtype=torch.int32, device=Lt.device)
        residual = torch.zeros(rounds, dtype=torch.float64, device=Lt.device)
    for k in range(rounds):
        G, c = _normal_equations(Lt, Rt, P._t, b2)
        # the split-precision normal equations are exact to ~1e-5: a residual
        # of 1e-9 (four orders below the reference's GMRES tolerance) is enough
        tol = 1e-9 if _PRECISION["precision"] == "tc" else 1e-12
        x = _cg_device(G, c, status[k], residual[k], tol=tol) if on_device else _cg_host(G, c, tol=tol)
        P = linalg.unitize(TorchData(x.reshape(old, new_dimension)), deferred=svd_status)
    linalg.check_deferred(svd_status)
    if on_device:
        st = status.cpu().numpy()
        res = residual.cpu().numpy()
        bad = (st[:, 1] == 0) & (res > ACCEPT_RESIDUAL)
        if bad.any():
            k = int(np.argmax(bad))
            raise AssertionError("normal equations of the product compressor did not converge "
                                 "(round %d: residual %.3e after %d iterations)" % (k, float(res[k]), int(st[k, 0])))
    return P.transpose()


__all__ = ["computeProductCompressor", "compression_precision", "absorb_matrices"]
