"""Seeded synthetic center-site problems with the shapes of the benchmark configs.

The tag structure of a grown boundary is obtained by running the product's
own schedules on tags alone (no data), e.g. one absorption round 0,1,2,3 of
the transverse-field Ising operator gives corners with 4 tags and sides with
5 tags, i.e. 9 stage-3 terms.  Tensor entries are i.i.d. N(0,1) from
``numpy.random.default_rng(seed)``, each tensor scaled to unit Frobenius norm.
"""
from __future__ import annotations

import numpy as np

from .sparse import (Identity, OneSiteOperator, TwoSiteOperator, compileSparseSchedule)
from .utils import L, R

X = np.array([[0, 1], [1, 0]], np.complex128)
Y = np.array([[0, -1j], [1j, 0]], np.complex128)
Z = np.array([[1, 0], [0, -1]], np.complex128)


def ti_operator_arrays(h=3.0, J=1.0):
    """Transverse-field Ising center: O=-h Z, OO_UD=OO_LR=(X, -J X)
    (the convention of makeSimpleSparseOperator, sparse.py:288-294)."""
    return [
        (OneSiteOperator(None), -h * Z),
        (TwoSiteOperator(0, 3, 0), X.copy()),
        (TwoSiteOperator(0, 1, 0), -J * X),
        (TwoSiteOperator(0, 0, 0), X.copy()),
        (TwoSiteOperator(0, 2, 0), -J * X),
        (Identity(), np.eye(2, dtype=np.complex128)),
    ]


def heisenberg_operator_arrays(J=1.0):
    """XXX antiferromagnet with spin-1/2 factor 1/4: makeSparseOperator(OO_UDs=[(X,X),(Y,Y),(Z,Z)]*J/4, same LR)."""
    out = []
    pairs = [(X, X), (Y, Y), (Z, Z)]
    for i, (a, b) in enumerate(pairs):
        out.append((TwoSiteOperator(i, 3, 0), a.copy()))
        out.append((TwoSiteOperator(i, 1, 0), 0.25 * J * b))
    for i, (a, b) in enumerate(pairs):
        out.append((TwoSiteOperator(i, 0, 0), a.copy()))
        out.append((TwoSiteOperator(i, 2, 0), 0.25 * J * b))
    out.append((Identity(), np.eye(2, dtype=np.complex128)))
    return out


def simulate_tags(op_tags, directions):
    """Tag lists of corners and sides after absorbing towards each direction."""
    from .tensors._2d import sparse as tsp
    corners = [[Identity()] for _ in range(4)]
    sides = [[Identity()] for _ in range(4)]
    for d in directions:
        corners[d] = compileSparseSchedule(tsp.RULES["absL"](), corners[d], sides[L(d)]).result_tags
        sides[d] = compileSparseSchedule(tsp._center_rules(d), sides[d], list(op_tags)).result_tags
        corners[R(d)] = compileSparseSchedule(tsp.RULES["absR"](), corners[R(d)], sides[R(d)]).result_tags
    return corners, sides


def random_unit(rng, shape, complex_=False):
    a = rng.standard_normal(shape)
    if complex_:
        a = a + 1j * rng.standard_normal(shape)
    a = a.astype(np.complex128)
    return a / np.linalg.norm(a)


def matvec_problem_arrays(D=4, c_ket=8, c_bra=4, seed=1, op_arrays=None, rounds=1, complex_=False):
    """Host arrays of the stage-3 microbenchmark: corners (c,c',1,c,c',1) and
    sides (c,c',1,c,c',1,D,D) per tag, chi = c*c' merged boundary dimension;
    real entries, or complex ones (re and im i.i.d. N(0,1)) with ``complex_``."""
    rng = np.random.default_rng(seed)
    op_arrays = ti_operator_arrays() if op_arrays is None else op_arrays
    op_tags = [t for t, _ in op_arrays]
    corners_t, sides_t = simulate_tags(op_tags, list(range(4)) * rounds)
    cshape = (c_ket, c_bra, 1, c_ket, c_bra, 1)
    sshape = cshape + (D, D)
    corners = [[(t, random_unit(rng, cshape, complex_)) for t in ct] for ct in corners_t]
    sides = [[(t, random_unit(rng, sshape, complex_)) for t in st] for st in sides_t]
    return corners, sides, op_arrays


def _ket_bra(rng, ket_shape, rank):
    """sum_r A_r (x) conj(A_r) with the ket and bra axes interleaved as the
    boundaries store them: (k_l, b_l, 1, k_r, b_r, 1[, D_k, D_b])."""
    a = rng.standard_normal((rank,) + ket_shape) + 1j * rng.standard_normal((rank,) + ket_shape)
    if len(ket_shape) == 2:
        t = np.einsum("rij,rkl->ikjl", a, a.conj())
        t = t.reshape(ket_shape[0], ket_shape[0], 1, ket_shape[1], ket_shape[1], 1)
    else:
        t = np.einsum("rijp,rklq->ikjlpq", a, a.conj())
        c0, c1, dd = ket_shape
        t = t.reshape(c0, c0, 1, c1, c1, 1, dd, dd)
    return t / np.linalg.norm(t)


def hermitian_problem_arrays(D=4, c=8, seed=2, op_arrays=None, rounds=1, rank=None):
    """A center-site problem whose pencil (H_eff, N_eff) is Hermitian with N_eff
    positive definite: every boundary tag is a sum of ket (x) conj(ket)
    products (c_ket = c_bra = c, chi = c^2), so every term is a tensor product
    of Hermitian factors with a Hermitian site operator.  The tag structure is
    the operator's after ``rounds`` absorption rounds (Heisenberg by default)."""
    rng = np.random.default_rng(seed)
    op_arrays = heisenberg_operator_arrays() if op_arrays is None else op_arrays
    rank = max(2, c) if rank is None else rank
    op_tags = [t for t, _ in op_arrays]
    corners_t, sides_t = simulate_tags(op_tags, list(range(4)) * rounds)
    corners = [[(t, _ket_bra(rng, (c, c), rank)) for t in ct] for ct in corners_t]
    sides = [[(t, _ket_bra(rng, (c, c, D), rank * D)) for t in st] for st in sides_t]
    return corners, sides, op_arrays


def bond_start_arrays(D, d, seed):
    """Start of a growth run: unit corners (1,1,1,1,1,1), each side a random
    Hermitian positive-definite bond matrix a a^H + I/2 (a with re and im
    i.i.d. N(0,1)) stored as (1,1,1,1,1,1,D,D), and a random real N(0,1)
    center (D,D,D,D,d) of unit norm, all from ``default_rng(seed)`` in that
    order."""
    rng = np.random.default_rng(seed)
    corners = [np.ones((1,) * 6, np.complex128) for _ in range(4)]
    sides = []
    for _ in range(4):
        a = rng.standard_normal((D, D)) + 1j * rng.standard_normal((D, D))
        bond = a @ a.conj().T + 0.5 * np.eye(D)
        sides.append(bond.reshape((1,) * 6 + (D, D)).astype(np.complex128))
    st = rng.standard_normal((D,) * 4 + (d,)).astype(np.complex128)
    return corners, sides, st / np.linalg.norm(st)


def growth_operator(kind):
    """Operator centers of the growth runs, as the reference's constructors
    build them: transverse Ising makeSimpleSparseOperator(O=-3 Z,
    OO_UD=(X,-X), OO_LR=(X,-X)); Heisenberg XXX (J=1 in Pauli units)
    makeSparseOperator(OO_UDs=[(X,X),(Y,Y),(Z,Z)], OO_LRs=same)."""
    from .data import TorchData
    from .sparse import makeSimpleSparseOperator, makeSparseOperator
    Xd, Yd, Zd = TorchData.X, TorchData.Y, TorchData.Z
    if kind == "ti":
        return makeSimpleSparseOperator(O=-3.0 * Zd, OO_UD=(Xd, -1.0 * Xd), OO_LR=(Xd, -1.0 * Xd))
    if kind == "heis":
        return makeSparseOperator(OO_UDs=[(Xd, Xd), (Yd, Yd), (Zd, Zd)], OO_LRs=[(Xd, Xd), (Yd, Yd), (Zd, Zd)])
    raise ValueError(kind)


# seed of the first absorbed center of each growth run (step k uses base + k)
GROWTH_CENTER_SEED = {"ti": 500, "heis": 900}


def growth_center(shape, seed):
    """The unit center absorbed at one step of a growth run: re and im i.i.d.
    N(0,1) from ``default_rng(seed)`` (re drawn first), scaled to unit norm.
    Absorbing the minimized center instead degenerates from the bond start:
    the transverse-Ising minimizer is the all-up product state at every step,
    and the Heisenberg center's first effective Hamiltonian is zero."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    return a / np.linalg.norm(a)


def bond_start_system(kind, D, seed):
    """The growth run's System on the device (bond_start_arrays, growth_operator)."""
    from .data import TorchData
    from .sparse import Identity
    from .system import System
    op = growth_operator(kind)
    d = next(iter(op.values())).shape[0]
    c, s, st = bond_start_arrays(D, d, seed)
    return System(tuple({Identity(): TorchData(a)} for a in c), tuple({Identity(): TorchData(a)} for a in s),
                  TorchData(st), op)


def to_device(corners, sides, op_arrays):
    from .data import TorchData
    c = [{t: TorchData(a) for t, a in lst} for lst in corners]
    s = [{t: TorchData(a) for t, a in lst} for lst in sides]
    o = {t: TorchData(a) for t, a in op_arrays}
    return c, s, o


def absorb_main(argv=None):
    """Grow a system by absorbing seeded random unit centers (the growth runs'
    absorption schedule, without the center solves): at every step
    contractTowards(step % 4) (system/_2d.py:435-454) with the tag pairs in
    FP64 or on the tensor cores, then compressCornerStateTowards for every
    corner axis above ``--new-dim``.  Prints one JSON line per step with the
    absorption's and the compressions' wall times (device synchronised on
    both sides); the last
    step's absorption runs inside an NVTX range named "absorb" and its
    compressions inside one named "compress", so a profiler can select their
    kernels (``ncu --nvtx --nvtx-include absorb/``)."""
    import argparse
    import json
    import time
    import torch
    from .data import TorchData
    from .sparse import Identity
    from .tensors._2d import dense
    p = argparse.ArgumentParser(prog="python -m carcassonne_gb300.workloads")
    p.add_argument("--kind", default="heis", choices=["ti", "heis"])
    p.add_argument("--D", type=int, default=4)
    p.add_argument("--seed", type=int, default=2)
    p.add_argument("--steps", type=int, default=8)
    p.add_argument("--new-dim", type=int, default=8, help="kept dimension of each corner axis (chi = new_dim^2)")
    p.add_argument("--precision", default="tc", choices=["tc", "fp64"], help="absorption precision")
    p.add_argument("--compress-precision", default="fp64", choices=["tc", "fp64"],
                   help="precision of the compressor's large contractions")
    p.add_argument("--build", type=int, default=0,
                   help="after the last step, build the center's expectation and normalization multipliers "
                        "(stages 1-3) this many times, the last inside an NVTX range named \"build\", and print "
                        "their wall times")
    a = p.parse_args(argv)
    from .compression import compression_precision
    system = bond_start_system(a.kind, a.D, a.seed)
    for step in range(a.steps):
        x0 = system.state_center_data
        system.setStateCenter(TorchData(growth_center(tuple(x0.shape), GROWTH_CENTER_SEED[a.kind] + step)))
        last = step == a.steps - 1
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if last:
            torch.cuda.nvtx.range_push("absorb")
        with dense.absorption_precision(a.precision):
            system.contractTowards(step % 4)
            torch.cuda.synchronize()
            seconds = time.perf_counter() - t0
            if last:
                torch.cuda.nvtx.range_pop()
        side = system.sides[step % 4][Identity()]
        t0 = time.perf_counter()
        if last:
            torch.cuda.nvtx.range_push("compress")
        with compression_precision(a.compress_precision):
            for corner in range(4):
                for cdir, axis in ((0, 0), (1, 3)):
                    if system.corners[corner][Identity()].shape[axis] > a.new_dim:
                        np.random.seed(1000 * step + 10 * corner + cdir)
                        system.compressCornerStateTowards(corner, cdir, a.new_dim)
        torch.cuda.synchronize()
        compress_s = time.perf_counter() - t0
        if last:
            torch.cuda.nvtx.range_pop()
        print(json.dumps(dict(step=step, precision=a.precision, compress_precision=a.compress_precision,
                              absorb_s=round(seconds, 6),
                              compress_s=round(compress_s, 6), side_shape=list(side.shape),
                              side_tags=len(system.sides[step % 4]))), flush=True)
    times = []
    for rep in range(a.build):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if rep == a.build - 1:
            torch.cuda.nvtx.range_push("build")
        system.formExpectationAndNormalizationMultipliers()
        torch.cuda.synchronize()
        times.append(round(time.perf_counter() - t0, 6))
        if rep == a.build - 1:
            torch.cuda.nvtx.range_pop()
    if times:
        print(json.dumps(dict(build_s=times, side_tags=[len(sd) for sd in system.sides],
                              corner_tags=[len(c) for c in system.corners])), flush=True)


if __name__ == "__main__":
    import sys
    if len(sys.argv) > 1 and sys.argv[1] == "absorb":
        absorb_main(sys.argv[2:])
    else:
        raise SystemExit("usage: python -m carcassonne_gb300.workloads absorb [--kind heis|ti] [--D 4] [--steps 8] "
                         "[--new-dim 8] [--precision tc|fp64]")
