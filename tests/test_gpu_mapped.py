"""Matvecs on pinned host memory mapped into the device's address space
(hostmem.MappedHostBuffer, carc_host_alloc_mapped): the kernels read the
block and write the result on the host directly, and the result equals the
same matvec on device memory bitwise, on a shape of the compact-operand fused
kernel (D=4, chi=32) and one of the two-kernel path (D=5, chi=40)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("D,ck,cb,seed", [(4, 8, 4, 1), (5, 8, 5, 3)])
def test_mapped_host_matvec_equals_device(D, ck, cb, seed):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from carcassonne_gb300 import workloads
    from carcassonne_gb300.hostmem import MappedHostBuffer
    from carcassonne_gb300.tensors._2d import sparse as tsp
    c, s, o = workloads.to_device(*workloads.matvec_problem_arrays(D=D, c_ket=ck, c_bra=cb, seed=seed))
    H, _ = tsp.formExpectationAndNormalizationMultipliers(c, s, o)
    op = H.operator
    nvec = 8
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((nvec,) + op.in_shape) + 1j * rng.standard_normal((nvec,) + op.in_shape)
    y_dev = op.apply_tc(torch.as_tensor(x).cuda(), None, nvec).cpu().numpy()
    xm = MappedHostBuffer((nvec,) + op.in_shape)
    ym = MappedHostBuffer((nvec,) + op.out_shape)
    try:
        xm.host[...] = x
        ym.host[...] = np.nan
        op.apply_tc_ptr(xm.device_ptr, ym.device_ptr, nvec)
        torch.cuda.synchronize()
        op.check_status()
        assert np.array_equal(ym.host, y_dev)
    finally:
        xm.close()
        ym.close()
