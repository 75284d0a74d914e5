"""Center-site solves in plain FP64 and in mixed precision.

plain  : H_eff and N_eff formed in FP64 on the CUDA cores, lowest generalized
         eigenpair by the Cholesky-reduced restarted Lanczos (linalg.hegv_lowest).
mixed  : H_eff and N_eff formed on the tensor cores from split-BF16 operands
         (~1e-5 relative), N factored and L inverted in complex64, the pencil
         reduced with tensor-core GEMMs and the Lanczos iteration run in
         complex64 on it; then one FP64 application of H and N gives the
         exact residual of that eigenvector, one Newton step against the
         tensor-core pencil (MINRES on its reduced form) corrects the vector,
         and the energy is the Rayleigh quotient of the corrected vector
         (exact first-order terms, tensor-core second-order terms).  Without
         the Newton step (newton=False) the energy is the Rayleigh quotient of
         the tensor-core eigenvector itself, with the exact H x and N x.

Both return the energy, the N-normalized center and a breakdown of where the
time went (CUDA events on the current stream).  Where N is too ill-conditioned
for the mixed reduction, or out of FP32's range, the mixed solve runs the
plain one; where FP64
Cholesky rejects N too, the pencil is solved on the range of N
(linalg.hegv_lowest_projected).  The result's ``fallback`` key names the path
taken ("plain" or "projected"; None when there was none).
"""
from __future__ import annotations

import numpy as np
import torch

from . import linalg
from .data import TorchData
from .engine import CDT


class _Timer:
    def __init__(self):
        self.events = []

    def mark(self, name):
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        self.events.append((name, e))

    def breakdown(self):
        torch.cuda.synchronize()
        out = {}
        for (n0, e0), (n1, e1) in zip(self.events, self.events[1:]):
            out[n1] = e0.elapsed_time(e1)
        out["total"] = self.events[0][1].elapsed_time(self.events[-1][1])
        return out


def _dot(a, b):
    """conj(a) . b on the device (carc_zdot); returns a complex Python scalar."""
    return complex(TorchData(a.reshape(-1))._dot(TorchData(b.reshape(-1))).item())


def _lin(a, x, b, y):
    return TorchData(x)._axpby(a, TorchData(x), b, TorchData(y))._t


def _apply(op, x):
    return op.apply(x.reshape(op.in_shape)).reshape(-1)


def _mv(A, v):
    """A v for a dense (n, n) device matrix (one strided contraction launch)."""
    return TorchData(A).contractWith(TorchData(v), (1,), (0,))._t


def _mhv(A, v):
    """A^H v."""
    return TorchData(A).conj().contractWith(TorchData(v), (0,), (0,))._t


def _norm(v):
    return abs(_dot(v, v)) ** 0.5


def _correct(Hop, Nop, x, Ht, Nt, factors):
    """Energy and vector from the tensor-core eigenvector x, recovered to FP64
    accuracy with one FP64 application of H and N.

    r = H x - E N x is the exact residual.  One Newton step against the
    tensor-core pencil (H~ - E N~) delta = -r, taken in the reduced
    coordinates (C~ - E) z = -L^-1 r with z orthogonal to u (the Lanczos
    eigenvector of C~, which x maps to) and solved by MINRES on the device
    (linalg.minres_projected), moves the
    eigenvector error from eps/gap to (eps/gap)^2, eps ~ 1e-5 the pencil's
    error.  The new Rayleigh quotient uses the exact H x, N x and the
    tensor-core matrices only for the second-order terms delta^H H~ delta,
    delta^H N~ delta (error eps |delta|^2): no second FP64 application."""
    n = Ht.shape[0]
    C = factors[: n * n].reshape(n, n)
    Li = factors[n * n: 2 * n * n].reshape(n, n)
    u = factors[2 * n * n:]
    xf = x.reshape(-1)
    hx, nx = _apply(Hop, xf), _apply(Nop, xf)
    nn = _dot(xf, nx).real
    xhx = _dot(xf, hx).real
    e = xhx / nn
    r = _lin(1.0, hx, -e, nx)
    uu = _lin(1.0 / _norm(u), u, 0.0, u)
    b = _lin(-1.0, _mv(Li, r), 0.0, r)
    z, _ = linalg.minres_projected(C, uu, e, b, maxit=60, rtol=1e-3)
    d = _mhv(Li, z)
    hd, nd = _mv(Ht, d), _mv(Nt, d)
    num = xhx + 2.0 * _dot(d, hx).real + _dot(d, hd).real
    den = nn + 2.0 * _dot(d, nx).real + _dot(d, nd).real
    x2 = _lin(1.0, xf, 1.0, d)
    return num / den, _lin(1.0 / abs(den) ** 0.5, x2, 0.0, x2), e


def _rayleigh(Hop, Nop, x):
    """Rayleigh quotient of x with one FP64 application of H and N, and x
    N-normalized."""
    xf = x.reshape(-1)
    hx, nx = _apply(Hop, xf), _apply(Nop, xf)
    nn = _dot(xf, nx).real
    return _dot(xf, hx).real / nn, _lin(1.0 / abs(nn) ** 0.5, xf, 0.0, xf)


def solve_center(H, N, x0=None, precision="plain", tol=None, newton=True):
    """Lowest eigenpair of (H_eff, N_eff) given the two stage-3 Multipliers.

    mixed: the eigenvector of the tensor-core pencil is accurate to about the
    operands' 1e-5 over the gap; one Newton correction against the same
    pencil with the exact FP64 residual (``_correct``) recovers FP64-level
    energies.  The pencil is reduced and iterated in complex64
    (linalg.hegv_lowest single=True).  newton=False skips the correction:
    the energy is then the Rayleigh quotient of the tensor-core eigenvector
    with the exact H x and N x, whose error is second order in the
    eigenvector's error and so grows as the spectral gap shrinks (6.5e-10
    relative on the benchmark pencil, 3.7e-8 on a small-gap golden case),
    and the center is that eigenvector.  ``tol`` is the Lanczos residual tolerance
    (default 1e-13 plain; 1e-7 mixed, clamped to 2e-6 by the complex64
    iteration: the tensor-core pencil's own error dominates the
    eigenvector's below that)."""
    Hop, Nop = getattr(H, "operator", None), N.operator
    timer = _Timer()
    timer.mark("start")
    if Hop is None:
        # H_eff = 0: every vector is an eigenvector with eigenvalue 0
        xt = (x0._t if isinstance(x0, TorchData) else torch.ones(Nop.in_shape, dtype=CDT, device="cuda"))
        xt = xt.reshape(Nop.in_shape)
        nrm = abs(_dot(xt.reshape(-1), Nop.apply(xt).reshape(-1))) ** 0.5
        timer.mark("eigensolve")
        return dict(energy=0.0, center=TorchData(_lin(1.0 / nrm, xt, 0.0, xt)), iterations=0,
                    timing_ms=timer.breakdown(), lanczos_eigenvalue=0.0, rayleigh_before_correction=None,
                    fallback=None)
    if precision == "plain":
        Hm = Hop.form_matrix()
        Nm = Nop.form_matrix()
    elif precision == "mixed":
        Hm = Hop.form_matrix_tc()
        Nm = Nop.form_matrix_tc()
    else:
        raise ValueError("precision must be 'plain' or 'mixed'")
    timer.mark("form")
    if tol is None:
        tol = 1e-7 if precision == "mixed" else 1e-13
    factors = None
    if precision == "mixed":
        n = Hm.shape[0]
        factors = torch.empty(2 * n * n + n, dtype=CDT, device=Hm.device)
    try:
        lam, x, iters = linalg.hegv_lowest(TorchData(Hm), TorchData(Nm), x0=x0, tol=tol,
                                           tensor_core=(precision == "mixed"), factors=factors,
                                           single=(precision == "mixed"))
    except np.linalg.LinAlgError:
        if precision == "mixed":
            # the tensor-core N (about 1e-5 relative) factored in complex64
            # is not positive definite: N's condition number is beyond what
            # the mixed reduction resolves, or its entries lie outside FP32's
            # range, so this step is solved in FP64
            out = solve_center(H, N, x0=x0, precision="plain")
            out["fallback"] = "plain" if out.get("fallback") is None else out["fallback"]
            return out
        # FP64 Cholesky rejects N (nearly singular, rounding-level negative
        # eigenvalues): the pencil on the range of N
        lam, x, kept = linalg.hegv_lowest_projected(TorchData(Hm), TorchData(Nm))
        timer.mark("eigensolve")
        return dict(energy=float(lam), center=TorchData(x._t.reshape(Hop.in_shape)), iterations=0,
                    timing_ms=timer.breakdown(), lanczos_eigenvalue=float(lam), rayleigh_before_correction=None,
                    fallback="projected", kept=kept)
    timer.mark("eigensolve")
    xt = x._t
    energy = lam
    rq0 = None
    if precision == "mixed":
        Hop.check_status()
        Nop.check_status()
        if newton:
            energy, xt, rq0 = _correct(Hop, Nop, xt, Hm, Nm, factors)
        else:
            energy, xt = _rayleigh(Hop, Nop, xt)
            rq0 = energy
        energy = float(energy)
        timer.mark("refine")
    out = TorchData(xt.reshape(Hop.in_shape))
    return dict(energy=float(energy), center=out, iterations=iters, timing_ms=timer.breakdown(),
                lanczos_eigenvalue=float(lam), rayleigh_before_correction=rq0 if precision == "mixed" else None,
                fallback=None)


__all__ = ["solve_center"]
