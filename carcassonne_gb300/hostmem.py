"""Pinned host memory mapped into the device's address space.

``MappedHostBuffer`` holds a block of page-locked host memory allocated by the
library (``carc_host_alloc_mapped``): ``host`` is a numpy view for the host,
``device_ptr`` the address kernels use.  Handing ``device_ptr`` to a matvec
(``Stage3Operator.apply_tc_ptr``) lets the kernels read the input block and
write the result over the host link themselves (NVLink-C2C on Grace parts),
in place of a host-to-device copy before the call and a device-to-host copy
after it.  The numpy view must not outlive the buffer.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


class MappedHostBuffer:
    def __init__(self, shape, dtype=np.complex128):
        self.shape = tuple(int(s) for s in shape)
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        h, d = ctypes.c_void_p(), ctypes.c_void_p()
        _lib.call("carc_host_alloc_mapped", self.nbytes, ctypes.byref(h), ctypes.byref(d))
        self._host_ptr, self.device_ptr = h.value, d.value
        buf = (ctypes.c_char * self.nbytes).from_address(self._host_ptr)
        self.host = np.frombuffer(buf, dtype=self.dtype).reshape(self.shape)

    def close(self):
        if self._host_ptr:
            self.host = None
            _lib.call("carc_host_free", ctypes.c_void_p(self._host_ptr))
            self._host_ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["MappedHostBuffer"]
