"""TorchData: the reference's duck-typed ``Data`` protocol over CUDA tensors.

Mirrors ``NDArrayData`` (carcassonne/data/__init__.py:30-364) method for
method: value semantics (every method returns a new object) except the
in-place ``+=``, ``*=`` and ``[]=``.  All arithmetic runs in libcarcgb300
kernels on the current CUDA stream; the tensor is complex128 (or real float64
for a few constructors, promoted on first use) and lives on a CUDA device.
"""
from __future__ import annotations

import ctypes
import math
from functools import reduce

import numpy as np
import torch

from .. import _lib
from .. import engine
from ..engine import CDT, current_stream_handle

LETTERS = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"


def default_device():
    return torch.device("cuda", torch.cuda.current_device())


def _as_cdt(t):
    if t.dtype != CDT:
        t = t.to(CDT)
    return t


class ARPACKError(Exception):
    """Declared by the reference's data module (data/__init__.py:12) for
    ARPACK failures; kept so that code importing or catching it still works.
    The device eigensolvers report non-convergence through the library's
    status words instead."""


class Data:
    """Base of the Data protocol (data/__init__.py:17-26)."""

    def size(self):
        return int(np.prod(self.shape, dtype=np.int64))


class TorchData(Data):

    # -- construction ---------------------------------------------------------
    def __init__(self, t):
        if isinstance(t, TorchData):
            t = t._t
        if isinstance(t, np.ndarray) or np.isscalar(t):
            t = torch.as_tensor(np.asarray(t, dtype=np.complex128)).to(default_device())
        elif not isinstance(t, torch.Tensor):
            raise TypeError("TorchData wraps a torch tensor or numpy array, not %r" % type(t))
        if t.device.type != "cuda":
            t = t.to(default_device())
        self._t = _as_cdt(t)

    @classmethod
    def fromArray(cls, arr):
        return cls(np.asarray(arr, dtype=np.complex128))

    @classmethod
    def newCollected(cls, datas):
        datas = list(datas)
        return cls(torch.stack([d._t for d in datas]))

    @classmethod
    def newDiagonal(cls, data):
        return cls(torch.diag(data._t if isinstance(data, TorchData) else torch.as_tensor(np.asarray(data))))

    @classmethod
    def newFilled(cls, shape, value, dtype=None):
        out = torch.empty(tuple(shape), dtype=CDT, device=default_device())
        v = complex(value)
        _lib.call("carc_zfill", out.numel(), v.real, v.imag, ctypes.c_void_p(out.data_ptr()), current_stream_handle())
        return cls(out)

    @classmethod
    def newIdentity(cls, N, dtype=None):
        return cls(np.identity(N, dtype=np.complex128))

    @classmethod
    def newRandom(cls, *shape):
        # same distribution as utils.randomComplexSample (utils.py:795-796),
        # drawn from numpy's global generator like the reference
        s = tuple(shape)
        arr = np.random.random_sample(s) * 2 - 1 + np.random.random_sample(s) * 2j - 1j
        return cls(arr)

    @classmethod
    def newRandomHermitian(cls, *shape):
        d = cls.newRandom(*shape)
        d += d.transpose().conj()
        return d

    @classmethod
    def newNormalizedRandom(cls, *shape):
        return cls.newRandom(*shape).normalized()

    @classmethod
    def newTrivial(cls, shape, dtype=None):
        return cls.newFilled(shape, 1.0)

    @classmethod
    def newZeros(cls, shape, dtype=None):
        return cls.newFilled(shape, 0.0)

    @classmethod
    def newOuterProduct(cls, *factors):
        fs = [f if isinstance(f, TorchData) else TorchData(f) for f in factors]
        return reduce(lambda a, b: a.contractWith(b, (), ()), fs)

    @classmethod
    def newEnlargener(cls, old_dimension, new_dimension, dtype=None):
        if new_dimension == old_dimension:
            return (cls.newIdentity(new_dimension),) * 2
        from ..linalg import qr_economic
        m = qr_economic(cls.newRandom(new_dimension, old_dimension))
        return m, m.conj()

    # -- properties ---------------------------------------------------------
    dtype = property(lambda self: np.dtype(np.complex128))
    ndim = property(lambda self: self._t.dim())
    shape = property(lambda self: tuple(int(x) for x in self._t.shape))

    def tensor(self):
        return self._t

    def toArray(self):
        return self._t.detach().cpu().numpy()

    def toNDArrayData(self):
        return self.toArray()

    # -- elementwise --------------------------------------------------------
    def _axpby(self, a, x, b, y):
        out = torch.empty(self._t.shape, dtype=CDT, device=self._t.device)
        a, b = complex(a), complex(b)
        xt = x._t.contiguous() if x is not None else None
        yt = y._t.contiguous() if y is not None else None
        if xt is not None and xt.shape != out.shape or yt is not None and yt.shape != out.shape:
            raise ValueError("operands could not be broadcast together with shapes %s %s" %
                             (tuple(xt.shape) if xt is not None else None, tuple(yt.shape) if yt is not None else None))
        _lib.call("carc_zaxpby", out.numel(), a.real, a.imag,
                  ctypes.c_void_p(xt.data_ptr() if xt is not None else 0), b.real, b.imag,
                  ctypes.c_void_p(yt.data_ptr() if yt is not None else 0), ctypes.c_void_p(out.data_ptr()),
                  current_stream_handle())
        return TorchData(out)

    def __add__(self, other):
        return self._axpby(1, self, 1, other)

    def __sub__(self, other):
        return self._axpby(1, self, -1, other)

    def __neg__(self):
        return self._axpby(-1, self, 0, None)

    def __iadd__(self, other):
        # in place, like numpy's += (data/__init__.py:99-101)
        t = self._t
        if not t.is_contiguous():
            self._t = self._axpby(1, self, 1, other)._t
            return self
        y = other._t.contiguous()
        if y.shape != t.shape:
            raise ValueError("operands could not be broadcast together")
        _lib.call("carc_zaxpby", t.numel(), 1.0, 0.0, ctypes.c_void_p(t.data_ptr()), 1.0, 0.0,
                  ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(t.data_ptr()), current_stream_handle())
        return self

    def __mul__(self, other):
        if isinstance(other, TorchData):
            if other.shape != self.shape:
                a, b = torch.broadcast_tensors(self._t, other._t)
                return TorchData(a.contiguous())._mul(TorchData(b.contiguous()))
            return self._mul(other)
        return self._axpby(complex(other), self, 0, None)

    __rmul__ = __mul__

    def _mul(self, other):
        x, y = self._t.contiguous(), other._t.contiguous()
        out = torch.empty(x.shape, dtype=CDT, device=x.device)
        _lib.call("carc_zmul", out.numel(), ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                  ctypes.c_void_p(out.data_ptr()), current_stream_handle())
        return TorchData(out)

    def __imul__(self, other):
        r = self * other
        self._t = r._t
        return self

    def __truediv__(self, other):
        if isinstance(other, TorchData):
            return TorchData(self._t / other._t)
        return self._axpby(1.0 / complex(other), self, 0, None)

    def __getitem__(self, index):
        return TorchData(self._t[index].contiguous())

    def __setitem__(self, index, value):
        self._t[index] = value._t if isinstance(value, TorchData) else torch.as_tensor(value)

    def __copy__(self):
        return TorchData(self._t.clone())

    copy = __copy__

    def __repr__(self):
        return "TorchData(%r)" % (self.toArray(),)

    # -- shape manipulation ---------------------------------------------------
    def join(self, *groups):
        groups = [[g] if isinstance(g, (int, np.integer)) else list(g) for g in groups]
        perm = [int(i) for g in groups for i in g]
        if sorted(perm) != list(range(self.ndim)):
            raise ValueError("join groups %s do not cover the %d axes exactly" % (groups, self.ndim))
        shp = self.shape
        new_shape = [int(np.prod([shp[i] for i in g], dtype=np.int64)) for g in groups]
        if perm == list(range(self.ndim)):
            return TorchData(self._t.contiguous().reshape(new_shape))
        t = engine.permute(self._t, perm)
        return TorchData(t.reshape(new_shape))

    def transpose(self, *args):
        if len(args) == 1 and not isinstance(args[0], (int, np.integer)):
            args = tuple(args[0])
        perm = list(args) if args else list(range(self.ndim))[::-1]
        return TorchData(engine.permute(self._t, perm))

    def split(self, *splits):
        return TorchData(self._t.contiguous().reshape([int(s) for s in splits]))

    def splitAt(self, index, *split):
        shp = list(self.shape)
        if int(np.prod(split)) != shp[index]:
            raise AssertionError("split %s does not match dimension %d" % (split, shp[index]))
        return self.split(*(shp[:index] + list(split) + shp[index + 1:]))

    def ravel(self):
        return TorchData(self._t.contiguous().reshape(-1))

    def fold(self, axis):
        others = [i for i in range(self.ndim) if i != axis]
        return self.join(axis, others)

    def dropUnitAxis(self, axis):
        if self.shape[axis] != 1:
            raise ValueError("Axis {} has non-unit dimension {}.".format(axis, self.shape[axis]))
        shp = list(self.shape)
        del shp[axis]
        return TorchData(self._t.contiguous().reshape(shp))

    def conj(self):
        return TorchData(engine.permute(self._t, list(range(self.ndim)), conj=True))

    def adjoint(self):
        if self.ndim != 2:
            raise ValueError("Adjoint may only be computed for rank 2 tensors.")
        return TorchData(engine.permute(self._t, [1, 0], conj=True))

    # -- contractions -------------------------------------------------------
    def contractWith(self, other, self_axes, other_axes):
        """tensordot (data/__init__.py:157-159) as one strided GETT launch."""
        sa = [int(i) % max(self.ndim, 1) for i in self_axes]
        ob = [int(i) % max(other.ndim, 1) for i in other_axes]
        if len(sa) != len(ob):
            raise ValueError("shape-mismatch for sum")
        for i, j in zip(sa, ob):
            if self.shape[i] != other.shape[j]:
                raise ValueError("shape-mismatch for sum")
        la = list(LETTERS[:self.ndim])
        lb = list(LETTERS[self.ndim:self.ndim + other.ndim])
        for i, j in zip(sa, ob):
            lb[j] = la[i]
        out_letters = [la[i] for i in range(self.ndim) if i not in sa] + \
                      [lb[j] for j in range(other.ndim) if j not in ob]
        out_shape = [self.shape[i] for i in range(self.ndim) if i not in sa] + \
                    [other.shape[j] for j in range(other.ndim) if j not in ob]
        spec = "".join(la) + "," + "".join(lb) + "->" + "".join(out_letters)
        return TorchData(engine.contract(spec, self._t, other._t, out_shape))

    def contractWithAlongAll(self, other):
        assert self.ndim == other.ndim
        return self.contractWith(other, range(self.ndim), range(self.ndim))

    def absorbMatrixAt(self, axis, matrix):
        """matrix.contractWith(self,(1,),axis) moved back into place (data/__init__.py:148-150)."""
        if not isinstance(matrix, TorchData):
            matrix = TorchData(matrix)
        n = self.ndim
        la = list(LETTERS[:n])
        ma = "Z" + la[axis]
        out = list(la)
        out[axis] = "Z"
        shp = list(self.shape)
        if matrix.shape[1] != shp[axis]:
            raise ValueError("shape-mismatch for sum")
        shp[axis] = matrix.shape[0]
        spec = ma + "," + "".join(la) + "->" + "".join(out)
        return TorchData(engine.contract(spec, matrix._t, self._t, shp))

    def matvecWith(self, v):
        return v.absorbMatrixAt(0, self)

    def extractScalar(self):
        if self.ndim != 0:
            raise ValueError("tensor is not a scalar")
        return np.complex128(self._t.item())

    # -- reductions ---------------------------------------------------------
    def _dot(self, other, conj_x=True):
        x = self._t.contiguous()
        y = other._t.contiguous()
        n = x.numel()
        ws_bytes = _lib.load().carc_zdot_workspace_size(n)
        ws = engine.Workspace.get(ws_bytes, x.device)
        out = torch.empty((), dtype=CDT, device=x.device)
        _lib.call("carc_zdot", n, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), int(conj_x),
                  ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(ws.data_ptr()), ws_bytes, current_stream_handle())
        return out

    def norm(self):
        return math.sqrt(max(0.0, float(self._dot(self).real.item())))

    def normalized(self):
        return self * (1.0 / self.norm())

    def hasNaN(self):
        flag = torch.empty((), dtype=torch.int32, device=self._t.device)
        x = self._t.contiguous()
        _lib.call("carc_zhasnan", x.numel(), ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(flag.data_ptr()),
                  current_stream_handle())
        return bool(flag.item())

    def allcloseTo(self, other, rtol=1e-05, atol=1e-08):
        if self.shape != other.shape:
            return False
        d = (self - other).toArray()
        return bool(np.all(np.abs(d) <= atol + rtol * np.abs(other.toArray())))

    def isCloseTo(self, other, rtol=1e-7, atol=1e-7):
        nd = (self - other).norm()
        return nd <= atol or nd / (self.norm() + other.norm()) / 2 <= rtol

    def sqrt(self):
        return TorchData(torch.sqrt(self._t))

    # -- linear algebra (implemented in linalg.py) --------------------------
    def svd(self, full_matrices=True):
        from ..linalg import svd
        return svd(self, full_matrices)

    def qr(self, mode="full"):
        from ..linalg import qr
        return qr(self, mode)

    def unitize(self):
        from ..linalg import unitize
        return unitize(self)

    def normalizeAxis(self, axis, sqrt_svals=False, dont_recip_under=1e-14):
        from ..linalg import normalize_axis
        return normalize_axis(self, axis, sqrt_svals, dont_recip_under)

    def normalizeAxisAndDenormalize(self, axis_to_norm, axis_to_denorm, data_to_denormalize=None,
                                    sqrt_svals=False, dont_recip_under=1e-14):
        if data_to_denormalize is None:
            data_to_denormalize = self
        if self.shape[axis_to_norm] != data_to_denormalize.shape[axis_to_denorm]:
            raise ValueError("Normalized axis and denormalized axis have different sizes ({} != {}).".format(
                self.shape[axis_to_norm], data_to_denormalize.shape[axis_to_denorm]))
        normalized, _, denormalizer = self.normalizeAxis(axis_to_norm, sqrt_svals, dont_recip_under)
        return normalized, data_to_denormalize.absorbMatrixAt(axis_to_denorm, denormalizer)


def _pauli(m):
    return np.array(m, dtype=np.complex128)


PAULI = {
    "I": _pauli([[1, 0], [0, 1]]),
    "X": _pauli([[0, 1], [1, 0]]),
    "Y": _pauli([[0, -1j], [1j, 0]]),
    "Z": _pauli([[1, 0], [0, -1]]),
}


def pauli(name):
    return TorchData(PAULI[name])


class _LazyPauli:
    """Class attribute TorchData.X etc.: a device copy made on first access
    (NDArrayData.I/X/Y/Z, data/__init__.py:360-363)."""

    def __init__(self, name):
        self.name = name

    def __get__(self, obj, cls):
        return pauli(self.name)


for _n in "IXYZ":
    setattr(TorchData, _n, _LazyPauli(_n))


__all__ = ["ARPACKError", "Data", "TorchData", "pauli", "PAULI"]
