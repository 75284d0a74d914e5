"""Lowest eigenpairs of many independent center-site problems in one batched
block eigensolver.

The reference solves one center problem at a time (minimizeExpectation,
system/_2d.py:489-497, with relaxOver, utils.py:805-878, or ARPACK).  Here a
batch of problems of uneven shape advances together through LOBPCG with a
block of ``m`` vectors per problem (orthonormalising form: R and P are made
N-orthonormal and N-orthogonal to X before H and N are applied to the new R,
so the Rayleigh-Ritz basis stays well conditioned under the split-BF16
matvec's rounding; every few iterations X's images are recomputed and P
restarts, which bounds their drift).  Per iteration, over the whole batch:

* per active problem, the tensor-core matvecs N R, then H R' and N R' on the
  orthonormalised residual block (Stage3Operator.apply_tc, block of m);
* for the whole batch at once, a fixed number of launches (independent of the
  batch size): ragged block inner products, two batched Jacobi eigensolves
  (n = m for the orthonormalisation, n = 3m twice for the Rayleigh-Ritz step),
  the coefficient kernels, and the block update with the residual norms
  (csrc/lobpcg.cu);
* one device-to-host read of the residuals and Ritz values, after which
  converged problems leave the active set (their kernels skip them and their
  matvecs are no longer launched).

The per-problem solve is the same algorithm on a batch of one problem.  Every
problem's arithmetic is independent of the rest of the batch (fixed-order
reductions per problem), so a batched solve and the per-problem loop give the
same iterates.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import torch

from . import _lib
from .data import TorchData
from .engine import CDT, current_stream_handle

ITEM = 256     # CARC_LOBPCG_ITEM
MAX_M = 8      # CARC_LOBPCG_MAX_M


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


class BlockEigensolver:
    """LOBPCG over a batch of Hermitian-definite pencils (H, N) given as
    tensor-core stage-3 operators with equal input and output shapes."""

    def __init__(self, problems, m=8):
        if m not in (1, 2, 4, 8):
            raise ValueError("block size must be 1, 2, 4 or 8")
        self.H = [h for h, _ in problems]
        self.N = [nn for _, nn in problems]
        for h, nn in problems:
            if not (tuple(h.in_shape) == tuple(h.out_shape) == tuple(nn.in_shape) == tuple(nn.out_shape)):
                raise ValueError("H and N must map the center space to itself")
        if not problems:
            raise ValueError("no problems")
        self.device = self.H[0].device
        self.m, self.k, self.B = m, 3 * m, len(problems)
        self.n = [int(np.prod(h.in_shape)) for h in self.H]
        self.off, total = [], 0
        for nb in self.n:
            self.off.append(total)
            total += -(-self.k * nb // 16) * 16
        ip, st, first = [], [], [0]
        for b, nb in enumerate(self.n):
            for e0 in range(0, nb, ITEM):
                ip.append(b)
                st.append(e0)
            first.append(len(ip))
        self.items = len(ip)
        dev = self.device
        i32 = lambda v: torch.tensor(v, dtype=torch.int32, device=dev)
        self._ip, self._is, self._first = i32(ip), i32(st), i32(first)
        self._off = torch.tensor(self.off, dtype=torch.int64, device=dev)
        self._n = i32(self.n)
        self.active = torch.ones(self.B, dtype=torch.int32, device=dev)
        z = lambda *s: torch.zeros(s, dtype=CDT, device=dev)
        f = lambda *s: torch.zeros(s, dtype=torch.float64, device=dev)
        self.S = [z(total), z(total)]
        self.HS = [z(total), z(total)]
        self.NS = [z(total), z(total)]
        B, k = self.B, self.k
        self.GH, self.GN, self.GNs, self.T, self.G, self.V1, self.V2 = (z(B, k, k) for _ in range(7))
        self.W1, self.W2, self.dk = f(B, k), f(B, k), f(B, k)
        self.C = z(B, k, m)
        self.rank = torch.zeros(B, dtype=torch.int32, device=dev)
        self.Q = z(B, 3 * m, 2 * m)
        self.Ms, self.Vo = z(B, 2, m, m), z(B, 2, m, m)
        self.dsc, self.Wo = f(B, 2, m), f(B, 2, m)
        self.M4 = z(B, 4, m, m)
        self.res = f(B, m)
        lib = _lib.load()
        self.ws_bytes = int(lib.carc_lobpcg_workspace_size(self.items, m))
        self.ws = torch.empty(max(self.ws_bytes, 256), dtype=torch.uint8, device=dev)
        self.jws_bytes = int(max(lib.carc_zheev_jacobi_workspace_size(k, B),
                                 lib.carc_zheev_jacobi_workspace_size(m, 2 * B)))
        self.jws = torch.empty(max(self.jws_bytes, 256), dtype=torch.uint8, device=dev)
        self.jstatus = torch.zeros((), dtype=torch.int32, device=dev)
        self.matvec_flops = 0.0

    # -- layout ----------------------------------------------------------------
    def rows(self, pool, b, r0, r1):
        """Rows r0..r1-1 of problem b's block in a pool, as (r1-r0,) + center shape."""
        nb, o = self.n[b], self.off[b]
        return pool[o + r0 * nb: o + r1 * nb].view((r1 - r0,) + tuple(self.H[b].in_shape))

    def _ragged(self):
        return (self.B, self.items, self.m, _vp(self._ip), _vp(self._is), _vp(self._first), _vp(self._off),
                _vp(self._n), _vp(self.active))

    def _matvec(self, ops, src, dst, buf, b, r0, r1):
        op = ops[b]
        op.apply_tc(self.rows(src[buf], b, r0, r1), self.rows(dst[buf], b, r0, r1), nvec=r1 - r0)
        self.matvec_flops += 8.0 * op.cost_of_multiply() * (r1 - r0)

    def _jacobi(self, n, batch, A, W, V):
        _lib.call("carc_zheev_jacobi", n, batch, _vp(A), _vp(W), _vp(V), _vp(self.jstatus), _vp(self.jws),
                  self.jws_bytes, current_stream_handle())

    # -- one iteration's batched steps -------------------------------------------
    def _orthonormalise(self, cur, act, refresh):
        m = self.m
        if refresh:  # fresh images of X; P restarts from zero
            for b in act:
                self._matvec(self.H, self.S, self.HS, cur, b, 0, m)
                self._matvec(self.N, self.S, self.NS, cur, b, 0, m)
        for b in act:
            self._matvec(self.N, self.S, self.NS, cur, b, m, 2 * m)
        s = current_stream_handle()
        _lib.call("carc_lobpcg_inner", *self._ragged(), _vp(self.S[cur]), 0, 3 * m, _vp(self.NS[cur]), None, m,
                  2 * m, _vp(self.Q), None, _vp(self.ws), self.ws_bytes, s)
        _lib.call("carc_lobpcg_orth_prepare", self.B, m, _vp(self.active), _vp(self.Q), self.floor, _vp(self.Ms),
                  _vp(self.dsc), s)
        self._jacobi(m, 2 * self.B, self.Ms, self.Wo, self.Vo)
        _lib.call("carc_lobpcg_orth_finish", self.B, m, _vp(self.active), _vp(self.Q), _vp(self.dsc), _vp(self.Wo),
                  _vp(self.Vo), self.drop, int(bool(refresh)), _vp(self.M4), s)
        _lib.call("carc_lobpcg_orth_apply", *self._ragged(), _vp(self.M4), _vp(self.S[cur]), _vp(self.HS[cur]),
                  _vp(self.NS[cur]), s)
        for b in act:
            self._matvec(self.H, self.S, self.HS, cur, b, m, 2 * m)
            self._matvec(self.N, self.S, self.NS, cur, b, m, 2 * m)

    def _rayleigh_ritz(self, cur):
        m, k, s = self.m, self.k, current_stream_handle()
        _lib.call("carc_lobpcg_inner", *self._ragged(), _vp(self.S[cur]), 0, k, _vp(self.HS[cur]),
                  _vp(self.NS[cur]), 0, k, _vp(self.GH), _vp(self.GN), _vp(self.ws), self.ws_bytes, s)
        _lib.call("carc_lobpcg_rr_scale", self.B, m, _vp(self.active), _vp(self.GN), _vp(self.GNs), _vp(self.dk), s)
        self._jacobi(k, self.B, self.GNs, self.W1, self.V1)
        _lib.call("carc_lobpcg_rr_reduce", self.B, m, _vp(self.active), _vp(self.GH), _vp(self.dk), _vp(self.W1),
                  _vp(self.V1), self.drop, _vp(self.T), _vp(self.G), _vp(self.rank), s)
        self._jacobi(k, self.B, self.G, self.W2, self.V2)
        _lib.call("carc_lobpcg_rr_combine", self.B, m, _vp(self.active), _vp(self.T), _vp(self.V2), _vp(self.C), s)
        nxt = 1 - cur
        _lib.call("carc_lobpcg_update", *self._ragged(), _vp(self.C), _vp(self.W2), _vp(self.S[cur]),
                  _vp(self.HS[cur]), _vp(self.NS[cur]), _vp(self.S[nxt]), _vp(self.HS[nxt]), _vp(self.NS[nxt]),
                  _vp(self.res), _vp(self.ws), self.ws_bytes, s)
        return nxt

    # -- the solve ---------------------------------------------------------------
    def start(self, seeds):
        """Random N(0,1) complex start blocks, one seeded generator per problem."""
        for pool in self.S + self.HS + self.NS:
            pool.zero_()
        for b, seed in enumerate(seeds):
            g = torch.Generator().manual_seed(int(seed))
            shape = (self.m, self.n[b])
            x = torch.complex(torch.randn(shape, generator=g, dtype=torch.float64),
                              torch.randn(shape, generator=g, dtype=torch.float64))
            self.rows(self.S[0], b, 0, self.m).copy_(x.view((self.m,) + tuple(self.H[b].in_shape)))

    def solve(self, seeds, tol=1e-4, max_iter=150, drop=1e-8, floor=1e-10, refresh=20):
        """Run to |R_0| / (|H x_0| + |theta_0| |N x_0|) <= tol for every
        problem (or max_iter Rayleigh-Ritz steps).  Every ``refresh``
        iterations H X and N X are recomputed and P restarts from zero: the
        implicitly updated images otherwise drift under the split-precision
        rounding until the Rayleigh-Ritz step follows the drift below the
        true eigenvalue.  Returns per-problem energies (the lowest Ritz
        value), iteration counts and residuals."""
        self.drop, self.floor = float(drop), float(floor)
        self.matvec_flops = 0.0
        B, m = self.B, self.m
        self.start(seeds)
        self.active.fill_(1)
        act_h = np.ones(B, bool)
        iters = np.zeros(B, np.int64)
        energy = np.full(B, np.nan)
        resid = np.full(B, np.nan)
        self.final = np.zeros(B, np.int64)
        cur = 0
        t0 = time.perf_counter()
        for b in range(B):
            self._matvec(self.H, self.S, self.HS, cur, b, 0, m)
            self._matvec(self.N, self.S, self.NS, cur, b, 0, m)
        for it in range(max_iter):
            act = np.flatnonzero(act_h).tolist()
            if it > 0:
                self._orthonormalise(cur, act, refresh and it % refresh == 0)
            cur = self._rayleigh_ritz(cur)
            host = torch.cat([self.res[:, 0], self.W2[:, 0]]).cpu().numpy()
            changed = False
            for b in act:
                iters[b] = it + 1
                energy[b], resid[b] = host[B + b], host[b]
                self.final[b] = cur
                if host[b] <= tol:
                    act_h[b] = False
                    changed = True
            if not act_h.any():
                break
            if changed:
                self.active.copy_(torch.from_numpy(act_h.astype(np.int32)))
        torch.cuda.synchronize()
        seconds = time.perf_counter() - t0
        if int(self.jstatus.item()) != 0:
            raise _lib.CarcError(_lib.CARC_NOT_CONVERGED, "batched Jacobi eigensolver did not converge")
        for h in self.H + self.N:
            h.check_status()
        self.active.fill_(1)
        return dict(energy=energy, iterations=iters, residual=resid, converged=~act_h, seconds=seconds,
                    matvec_flops=self.matvec_flops)

    def vector(self, b):
        """Problem b's lowest Ritz vector (center shape), from the buffer of its last update."""
        return self.rows(self.S[int(self.final[b])], b, 0, 1)[0]

    def verify(self):
        """Fresh tensor-core products of each problem's returned vector: its
        Rayleigh quotient and relative residual (not the iteration's recurrences)."""
        out = []
        for b in range(self.B):
            x = self.vector(b).contiguous()
            hx = self.H[b].apply_tc(x)
            nx = self.N[b].apply_tc(x)
            X, Hx, Nx = TorchData(x), TorchData(hx), TorchData(nx)
            e = complex(X._dot(Hx).item()).real / complex(X._dot(Nx).item()).real
            r = Hx._axpby(1.0, Hx, -e, Nx)
            nr = abs(complex(r._dot(r).item())) ** 0.5
            nh = abs(complex(Hx._dot(Hx).item())) ** 0.5
            nn = abs(complex(Nx._dot(Nx).item())) ** 0.5
            out.append((e, nr / (nh + abs(e) * nn)))
        return out


def solve_batch(problems, seeds, m=8, **kw):
    """All problems in one batched solve."""
    return BlockEigensolver(problems, m).solve(seeds, **kw)


def solve_each(problems, seeds, m=8, **kw):
    """The per-problem loop: the same solver on one problem at a time."""
    out = dict(energy=[], iterations=[], residual=[], converged=[], seconds=0.0, matvec_flops=0.0)
    for p, s in zip(problems, seeds):
        r = BlockEigensolver([p], m).solve([s], **kw)
        for key in ("energy", "iterations", "residual", "converged"):
            out[key].append(r[key][0])
        out["seconds"] += r["seconds"]
        out["matvec_flops"] += r["matvec_flops"]
    for key in ("energy", "iterations", "residual", "converged"):
        out[key] = np.asarray(out[key])
    return out


__all__ = ["BlockEigensolver", "solve_batch", "solve_each", "ITEM", "MAX_M"]
