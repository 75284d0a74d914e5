"""Center-site solves in plain FP64 and in mixed precision.

plain  : H_eff and N_eff formed in FP64 on the CUDA cores, lowest generalized
         eigenpair by the Cholesky-reduced restarted Lanczos (linalg.hegv_lowest).
mixed  : H_eff and N_eff formed on the tensor cores from split-BF16 operands
         (~1e-5 relative), the same eigensolver on them; the energy is the FP64
         Rayleigh quotient of that eigenvector with the exact operators (one
         FP64 application of each), whose error is quadratic in the
         eigenvector's; optional Rayleigh-Ritz steps on span{x, t}, t the FP64
         residual H x - E N x, also refine the vector.

Both return the energy, the N-normalized center and a breakdown of where the
time went (CUDA events on the current stream).
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


def _refine(Hop, Nop, x):
    """One Rayleigh-Ritz step with the FP64 operators on span{x, r},
    r = H x - E N x the FP64 residual; the 2x2 pencil is solved by the GPU
    generalized eigensolver."""
    shp = Hop.in_shape
    xx = x.reshape(-1)
    Hx = Hop.apply(x.reshape(shp)).reshape(-1)
    Nx = Nop.apply(x.reshape(shp)).reshape(-1)
    e = (_dot(xx, Hx) / _dot(xx, Nx)).real
    r = _lin(1.0, Hx, -e, Nx)
    rn = abs(_dot(r, r)) ** 0.5
    if rn == 0.0:
        return e, x
    tt = _lin(1.0 / rn, r, 0.0, r)
    Ht = Hop.apply(tt.reshape(shp)).reshape(-1)
    Nt = Nop.apply(tt.reshape(shp)).reshape(-1)
    hxt, nxt = _dot(xx, Ht), _dot(xx, Nt)
    Hs = np.array([[_dot(xx, Hx).real, hxt], [np.conj(hxt), _dot(tt, Ht).real]], np.complex128)
    Ns = np.array([[_dot(xx, Nx).real, nxt], [np.conj(nxt), _dot(tt, Nt).real]], np.complex128)
    try:
        lam2, c, _ = linalg.hegv_lowest(TorchData(Hs), TorchData(Ns), max_krylov=2)
    except (np.linalg.LinAlgError, RuntimeError):
        return e, x
    cc = c.toArray()
    y = _lin(complex(cc[0]), xx, complex(cc[1]), tt)
    Ny = _lin(complex(cc[0]), Nx, complex(cc[1]), Nt)
    Hy = _lin(complex(cc[0]), Hx, complex(cc[1]), Ht)
    e2 = (_dot(y, Hy) / _dot(y, Ny)).real
    if not (e2 <= e):
        return e, x
    nrm = abs(_dot(y, Ny)) ** 0.5
    return e2, _lin(1.0 / nrm, y, 0.0, y)


def _rayleigh(Hop, Nop, x):
    """FP64 Rayleigh quotient of x and x N-normalized with the FP64 operators."""
    shp = Hop.in_shape
    xf = x.reshape(-1)
    hx = Hop.apply(x.reshape(shp)).reshape(-1)
    nx = Nop.apply(x.reshape(shp)).reshape(-1)
    nn = _dot(xf, nx).real
    e = _dot(xf, hx).real / nn
    return e, _lin(1.0 / abs(nn) ** 0.5, xf, 0.0, xf)


def solve_center(H, N, x0=None, precision="plain", refine_steps=0, tol=1e-13):
    """Lowest eigenpair of (H_eff, N_eff) given the two stage-3 Multipliers.

    mixed: the eigenvector of the tensor-core pencil is accurate to about the
    operands' 1e-5, so the FP64 Rayleigh quotient of it is accurate to about
    1e-10 (quadratic); ``refine_steps`` > 0 adds Rayleigh-Ritz steps with the
    FP64 residual that also improve the vector."""
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
                    timing_ms=timer.breakdown(), lanczos_eigenvalue=0.0)
    if precision == "plain":
        Hm = Hop.form_matrix()
        Nm = Nop.form_matrix()
    elif precision == "mixed":
        Hm = Hop.form_matrix_tc()
        Nm = Nop.form_matrix_tc()
    else:
        raise ValueError("precision must be 'plain' or 'mixed'")
    timer.mark("form")
    lam, x, iters = linalg.hegv_lowest(TorchData(Hm), TorchData(Nm), x0=x0, tol=tol)
    timer.mark("eigensolve")
    xt = x._t
    energy = lam
    if precision == "mixed":
        Hop.check_status()
        Nop.check_status()
        for _ in range(refine_steps):
            e, xt = _refine(Hop, Nop, xt)
        # FP64 Rayleigh quotient and N-normalization with the exact operators
        energy, xt = _rayleigh(Hop, Nop, xt)
        energy = float(energy)
        timer.mark("refine")
    out = TorchData(xt.reshape(Hop.in_shape))
    return dict(energy=float(energy), center=out, iterations=iters, timing_ms=timer.breakdown(),
                lanczos_eigenvalue=float(lam))


__all__ = ["solve_center"]
