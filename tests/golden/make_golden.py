"""Generate golden vectors by running the reference implementation itself.

Run where the reference is checked out, naming its root with
``CARC_REFERENCE`` (or ``--reference PATH`` as the first arguments):
``CARC_REFERENCE=/path/to/Carcassonne python tests/golden/make_golden.py [sections]``.  It writes
``dense.npz``, ``tables.json``, ``trajectory.npz`` and ``numerics.npz`` next to
this file.  The reference's randomness comes from numpy's global generator, so
every case seeds it (``numpy.random.seed``) before calling into it.
The GPU tests never run this script; they only read its outputs.
"""
import json
import os
import sys

import numpy as np

if len(sys.argv) > 2 and sys.argv[1] == "--reference":
    REF = sys.argv[2]
    del sys.argv[1:3]
else:
    REF = os.environ.get("CARC_REFERENCE")
if not REF:
    sys.exit("make_golden.py: set CARC_REFERENCE (or pass --reference PATH) to the reference's checkout")
sys.path.insert(0, REF)
sys.dont_write_bytecode = True

from carcassonne.data import NDArrayData  # noqa: E402
from carcassonne import sparse as rsparse  # noqa: E402
from carcassonne.tensors._2d import dense as rdense  # noqa: E402
from carcassonne.tensors._2d import sparse as rsp2  # noqa: E402
from carcassonne.system import System  # noqa: E402
from carcassonne.utils import relaxOver, computeCompressor, Multiplier, unitize  # noqa: E402
from carcassonne.compression import computeProductCompressor  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def cn(rng, *shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex128)


def D(a):
    return NDArrayData(np.ascontiguousarray(a))


def dense_cases():
    rng = np.random.default_rng(1234)
    out = {}
    n = 0
    for case in range(4):
        dims = rng.integers(1, 4, size=12)
        a, b, c, d, e, f, g, h, i, j, k, l = [int(x) for x in dims]
        # stage 1: corner (a,b,c,d,e,f), side (d,e,f,g,h,i,j,k)
        C = cn(rng, a, b, c, d, e, f)
        S = cn(rng, d, e, f, g, h, i, j, k)
        out[f"stage1_{case}_C"], out[f"stage1_{case}_S"] = C, S
        out[f"stage1_{case}_out"] = rdense.formNormalizationStage1(D(C), D(S)).toArray().copy()
        # absorb side into corner from the left: corner (a,b,c,d,e,f), side (g,h,i,a,b,c,j,k)
        S2 = cn(rng, g, h, i, a, b, c, j, k)
        out[f"absL_{case}_C"], out[f"absL_{case}_S"] = C, S2
        out[f"absL_{case}_out"] = rdense.absorbDenseSideIntoCornerFromLeft(D(C), D(S2)).toArray().copy()
        out[f"absR_{case}_C"], out[f"absR_{case}_S"] = C, S
        out[f"absR_{case}_out"] = rdense.absorbDenseSideIntoCornerFromRight(D(C), D(S)).toArray().copy()
        # stage 2: A (a,b,c,d), B (e,a,f,g)
        A2 = cn(rng, a, b, c, d)
        B2 = cn(rng, e, a, f, g)
        out[f"stage2_{case}_A"], out[f"stage2_{case}_B"] = A2, B2
        out[f"stage2_{case}_out"] = rdense.formNormalizationStage2(D(A2), D(B2)).toArray().copy()
        # stage 3: s2_0 (x0,x1,k0,k1,l0,l1), s2_1 (x1,x0,k2,k3,l2,l3)
        x0, x1 = a, b
        k0, k1, k2, k3 = c, d, e, f
        p = int(rng.integers(1, 4))
        s20 = cn(rng, x0, x1, k0, k1, k0, k1)
        s21 = cn(rng, x1, x0, k2, k3, k2, k3)
        op = cn(rng, p, p)
        v = cn(rng, k0, k1, k2, k3, p)
        out[f"stage3_{case}_s20"], out[f"stage3_{case}_s21"] = s20, s21
        out[f"stage3_{case}_op"], out[f"stage3_{case}_v"] = op, v
        m = rdense.formDenseStage3(D(s20), D(s21), D(op))
        out[f"stage3_{case}_Hv"] = m(D(v)).toArray().copy()
        out[f"stage3_{case}_H"] = m.formMatrix().toArray().copy()
        out[f"stage3_{case}_cost"] = np.array([m.cost_of_multiply, m.cost_of_formMatrix])
        nm = rdense.formNormalizationStage3(D(s20), D(s21), NDArrayData.newIdentity(p))
        out[f"stage3_{case}_Nv"] = nm(D(v)).toArray().copy()
        out[f"stage3_{case}_N"] = nm.formMatrix().toArray().copy()
        out[f"stage3_{case}_ncost"] = np.array([nm.cost_of_multiply, nm.cost_of_formMatrix])
        # center into side, every direction
        for direction in range(4):
            g2 = int(rng.integers(1, 3))
            side = cn(rng, a, b, c, d, e, f, g2, g2)
            shp = [int(x) for x in rng.integers(1, 3, size=5)]
            shp[direction] = g2
            st = cn(rng, *shp)
            o = cn(rng, shp[4], shp[4])
            key = f"center_{case}_{direction}"
            out[key + "_side"], out[key + "_S"], out[key + "_O"] = side, st, o
            out[key + "_SS"] = rdense.absorbDenseCenterSSIntoSide(direction, D(side), D(st)).toArray().copy()
            out[key + "_SOS"] = rdense.absorbDenseCenterSOSIntoSide(direction, D(side), D(st), D(o)).toArray().copy()
        n += 1
    np.savez_compressed(os.path.join(HERE, "dense.npz"), **out)


# --- recording of the tag-pair schedule --------------------------------------
_orig_contract = rsparse.contractSparseTensors
_log = []


def _recording_contract(dense_contractors, t1, t2):
    keys1, keys2 = list(t1), list(t2)
    rec = []
    wrapped = {}
    for key, handler in dense_contractors.items():
        def wh(x, y, handler=handler):
            r = handler(x, y)
            if r is None or r[0] is None:
                return r
            tag, fn = r

            def fn2(p, q, x=x, y=y, tag=tag, fn=fn):
                rec.append([keys1.index(x), keys2.index(y), repr(tag)])
                return fn(p, q)
            return tag, fn2
        wrapped[key] = wh
    result = _orig_contract(wrapped, t1, t2)
    _log.append(dict(tags1=[repr(k) for k in keys1], tags2=[repr(k) for k in keys2],
                     entries=rec, result=[repr(k) for k in result]))
    return result


def _install_recorder():
    rsp2.contractSparseTensors = _recording_contract


def _stage3_terms(system):
    """Term list of formExpectationStage3 recorded through the dense builders."""
    s1 = [rsp2.formExpectationStage1(system.corners[i], system.sides[i]) for i in range(4)]
    s2a = rsp2.formExpectationStage2(s1[0], s1[1])
    s2b = rsp2.formExpectationStage2(s1[2], s1[3])
    op = system.operator_center_tensor
    rec = []
    ids = {}
    for which, t in ((0, s2a), (1, s2b), (2, op)):
        for i, (k, v) in enumerate(t.items()):
            ids[(which, id(v))] = i
    orig_d, orig_n = rsp2.formDenseStage3, rsp2.formNormalizationStage3

    def rd(a, b, c):
        rec.append([ids[(0, id(a))], ids[(1, id(b))], ids[(2, id(c))], 0])
        return orig_d(a, b, c)

    def rn(a, b, c):
        if (2, id(c)) in ids:
            rec.append([ids[(0, id(a))], ids[(1, id(b))], ids[(2, id(c))], 1])
        return orig_n(a, b, c)
    rsp2.formDenseStage3, rsp2.formNormalizationStage3 = rd, rn
    try:
        H, N = rsp2.formExpectationStage3(s2a, s2b, op)
    finally:
        rsp2.formDenseStage3, rsp2.formNormalizationStage3 = orig_d, orig_n
    return dict(s2_0=[repr(k) for k in s2a], s2_1=[repr(k) for k in s2b], op=[repr(k) for k in op],
                terms=rec, cost_multiply=int(H.cost_of_multiply), cost_formMatrix=int(H.cost_of_formMatrix))


def operators():
    X, Y, Z = NDArrayData.X, NDArrayData.Y, NDArrayData.Z
    return {
        "ti": lambda: rsparse.makeSimpleSparseOperator(O=-3.0 * Z, OO_UD=(X, -1.0 * X), OO_LR=(X, -1.0 * X)),
        "heis": lambda: rsparse.makeSparseOperator(OO_UDs=[(X, X), (Y, Y), (Z, Z)], OO_LRs=[(X, X), (Y, Y), (Z, Z)]),
        "ising_ud": lambda: rsparse.makeSimpleSparseOperator(O=-1.0 * Z, OO_UD=(X, -0.5 * X)),
    }


def bond_system(op, D_, seed):
    """Unit corners and random Hermitian positive-definite bond boundaries of
    bond dimension D_ around a random center (a generic, non-degenerate start)."""
    rng = np.random.default_rng(seed)
    d = next(iter(op.values())).shape[0]
    corners = tuple({rsparse.Identity(): NDArrayData.newTrivial((1,) * 6, dtype=np.complex128)} for _ in range(4))
    sides = []
    for _ in range(4):
        a = rng.standard_normal((D_, D_)) + 1j * rng.standard_normal((D_, D_))
        bond = a @ a.conj().T + 0.5 * np.eye(D_)  # Hermitian positive definite, generic
        sides.append({rsparse.Identity(): NDArrayData(bond.reshape((1,) * 6 + (D_, D_)).astype(np.complex128))})
    sides = tuple(sides)
    st = rng.standard_normal((D_,) * 4 + (d,)).astype(np.complex128)
    st /= np.linalg.norm(st)
    return System(corners, sides, NDArrayData(st), op)


def tables_and_trajectories():
    _install_recorder()
    tables = {}
    traj = {}
    schedules = {
        "ti": (2, [0, 1, 2, 3, 0, 1], 7),
        "heis": (2, [0, 2, 1, 3, 0], 11),
        "ising_ud": (1, [0, 2, 1, 3, 1, 3, 0, 2], 5),
    }
    for name, mk in operators().items():
        D_, steps, seed = schedules[name]
        # distinct data objects per tag: the stage-3 recorder identifies data by id()
        op = {k: NDArrayData(v.toArray().copy()) for k, v in mk().items()}
        system = bond_system(op, D_, seed)
        st = system.state_center_data.toArray().copy()
        traj[f"{name}_state0"] = st
        traj[f"{name}_op_tags"] = np.array([repr(k) for k in op])
        for ki, (k, v) in enumerate(op.items()):
            traj[f"{name}_op_{ki}"] = v.toArray().astype(np.complex128)
        records = []
        for step, direction in enumerate(steps):
            _log.clear()
            Hm, Nm = system.formExpectationAndNormalizationMultipliers()
            stage_log = list(_log)
            terms = _stage3_terms(system)
            Hd = Hm.formMatrix().toArray().copy()
            Nd = Nm.formMatrix().toArray().copy()
            import scipy.linalg as sla
            w, v = sla.eigh(Hd, Nd)
            e, nrm = system.computeExpectationAndNormalization()
            traj[f"{name}_{step}_H"] = Hd
            traj[f"{name}_{step}_N"] = Nd
            traj[f"{name}_{step}_E"] = np.array([w[0], e, nrm])
            for i in range(4):
                for kj, (k, v_) in enumerate(system.corners[i].items()):
                    traj[f"{name}_{step}_corner{i}_{kj}"] = v_.toArray().copy().copy()
                for kj, (k, v_) in enumerate(system.sides[i].items()):
                    traj[f"{name}_{step}_side{i}_{kj}"] = v_.toArray().copy().copy()
            traj[f"{name}_{step}_state"] = system.state_center_data.toArray().copy()
            rec = dict(direction=direction,
                       corners=[[repr(k) for k in c] for c in system.corners],
                       sides=[[repr(k) for k in s] for s in system.sides],
                       stage_calls=stage_log, stage3=terms)
            # relaxOver from the current center
            np.random.seed(100 + step)
            x = relaxOver(system.state_center_data, Hm, Nm, maximum_number_of_multiplications=100)
            xr = x.toArray().ravel()
            rq = np.vdot(xr, Hd @ xr) / np.vdot(xr, Nd @ xr)
            traj[f"{name}_{step}_relax"] = np.array([rq])
            # minimize with the dense solver, then absorb towards direction
            system.minimizeExpectationUsingFullEigensolver()
            traj[f"{name}_{step}_minstate"] = system.state_center_data.toArray().copy()
            _log.clear()
            system.contractTowards(direction)
            rec["absorb_calls"] = list(_log)
            traj[f"{name}_{step}_after_state"] = system.state_center_data.toArray().copy()
            records.append(rec)
        tables[name] = dict(D=D_, steps=steps, seed=seed, records=records)
    rsp2.contractSparseTensors = _orig_contract
    with open(os.path.join(HERE, "tables.json"), "w") as f:
        json.dump(tables, f, indent=0, separators=(",", ":"))
    np.savez_compressed(os.path.join(HERE, "trajectory.npz"), **traj)


def numerics():
    rng = np.random.default_rng(77)
    out = {}
    # normalizeAxis
    for case, shape in enumerate([(2, 3, 2, 3, 2), (3, 3, 3, 3, 2), (4, 2, 5), (6, 1, 2)]):
        t = cn(rng, *shape)
        for axis in range(len(shape)):
            if np.prod(shape) // shape[axis] < shape[axis]:
                continue
            iso, nz, dz = NDArrayData(t).normalizeAxis(axis)
            key = f"nax_{case}_{axis}"
            out[key + "_in"] = t
            out[key + "_iso"] = iso.toArray().copy()
            out[key + "_norm"] = nz.toArray().copy()
            out[key + "_denorm"] = dz.toArray().copy()
            a, b = NDArrayData(t).normalizeAxis(axis, True)
            out[key + "_sq_a"] = a.toArray().copy()
            out[key + "_sq_b"] = b.toArray().copy()
    # unitize
    for case in range(3):
        m = cn(rng, 7, 3 + case)
        out[f"unitize_{case}_in"] = m
        out[f"unitize_{case}_out"] = unitize(m)
    # computeCompressor (eigh branch)
    for case, (old, new) in enumerate([(6, 3), (5, 5), (8, 4)]):
        a = cn(rng, 9, old)
        g = a.conj().T @ a
        c, ic = computeCompressor(old, new, Multiplier((old, old), lambda v: g @ v, 0, lambda: g, 0), np.complex128)
        out[f"cc_{case}_in"] = g
        out[f"cc_{case}_c"] = c
        out[f"cc_{case}_meta"] = np.array([old, new])
        c2, ic2 = computeCompressor(old, new, Multiplier((old, old), lambda v: g @ v, 0, lambda: g, 0), np.complex128, True)
        out[f"cc_{case}_cn"] = c2
        out[f"cc_{case}_icn"] = ic2
    # computeProductCompressor on an exactly compressible pair (tests/test_compression.py:11-30)
    for case, (new, extra, l, r, opd) in enumerate([(2, 2, 3, 4, 2), (3, 1, 2, 2, 1)]):
        old = new + extra
        Lc = cn(rng, l, new, new, opd)
        Lc = Lc + Lc.transpose(0, 2, 1, 3).conj()
        Lf = np.zeros((l, old, old, opd), np.complex128)
        Lf[:, :new, :new, :] = Lc
        Rc = cn(rng, new, new, opd, r)
        Rc = Rc + Rc.transpose(1, 0, 2, 3).conj()
        Rf = np.zeros((old, old, opd, r), np.complex128)
        Rf[:new, :new] = Rc
        np.random.seed(5 + case)
        P = computeProductCompressor(NDArrayData(Lf), NDArrayData(Rf), new).toArray().copy()
        out[f"pc_{case}_L"], out[f"pc_{case}_R"], out[f"pc_{case}_P"] = Lf, Rf, P
        out[f"pc_{case}_exact"] = np.tensordot(Lc, Rc, ((1, 2, 3), (0, 1, 2)))
    # relaxOver on small Hermitian pencils (tests/test_utils.py:857-878)
    for case, n in enumerate([4, 7, 10]):
        h = cn(rng, n, n)
        h = h + h.conj().T
        a = cn(rng, n, n)
        nm = a.conj().T @ a + n * np.eye(n)
        v0 = cn(rng, n)
        x = relaxOver(NDArrayData(v0.copy()), Multiplier.fromMatrix(NDArrayData(h)), Multiplier.fromMatrix(NDArrayData(nm)))
        out[f"relax_{case}_H"], out[f"relax_{case}_N"], out[f"relax_{case}_v0"] = h, nm, v0
        out[f"relax_{case}_x"] = x.toArray().copy()
    np.savez_compressed(os.path.join(HERE, "numerics.npz"), **out)


def chain1d():
    """The 1D chain (tensors/_1d.py, system/_1d.py): the four environment
    absorptions, the expectation multiplier and its matrix on random tensors,
    and one-site / total expectations of transverse-Ising and field systems."""
    if not hasattr(np, "product"):
        np.product = np.prod  # the reference's numpy 1 spelling
    from carcassonne.tensors import _1d as r1
    from carcassonne.system._1d import System as System1D
    from carcassonne.utils import buildTensor, Pauli
    rng = np.random.default_rng(20260104)
    out = {}
    for case, (o, sd, p) in enumerate([(1, 1, 2), (2, 3, 2), (3, 4, 3), (4, 2, 5)]):
        L, R = cn(rng, o, sd, sd), cn(rng, o, sd, sd)
        O, S = cn(rng, o, o, p, p), cn(rng, sd, sd, p)
        L2, R2 = cn(rng, sd, sd), cn(rng, sd, sd)
        Sc = S.conj()
        out[f"c{case}_L"], out[f"c{case}_R"], out[f"c{case}_O"], out[f"c{case}_S"] = L, R, O, S
        out[f"c{case}_L2"], out[f"c{case}_R2"] = L2, R2
        out[f"c{case}_ossL"] = r1.absorbCenterOSSIntoLeftEnvironment(D(L), D(O), D(S), D(Sc)).toArray().copy()
        out[f"c{case}_ossR"] = r1.absorbCenterOSSIntoRightEnvironment(D(R), D(O), D(S), D(Sc)).toArray().copy()
        out[f"c{case}_ssL"] = r1.absorbCenterSSIntoLeftEnvironment(D(L2), D(S), D(Sc)).toArray().copy()
        out[f"c{case}_ssR"] = r1.absorbCenterSSIntoRightEnvironment(D(R2), D(S), D(Sc)).toArray().copy()
        # the multiplier acts on states of shape (R.shape[1], L.shape[1], O.shape[2])
        m = r1.formExpectationMultiplier(D(R), D(L), D(O))
        out[f"c{case}_y"] = m(D(S)).toArray().copy()
        out[f"c{case}_M"] = m.formMatrix().toArray().copy()
        out[f"c{case}_cost"] = np.array([m.cost_of_multiply, m.cost_of_formMatrix])
    mpo_ti = lambda h: buildTensor((3, 3, 2, 2), {(0, 0): Pauli.I, (0, 2): h * Pauli.Z, (0, 1): -0.01 * Pauli.X,  # noqa: E731
                                                   (1, 2): Pauli.X, (2, 2): Pauli.I})
    for case, (h, sd) in enumerate([(1.0, 2), (0.5, 3), (2.0, 4)]):
        S, rb, lb = cn(rng, sd, sd, 2), cn(rng, sd), cn(rng, sd)
        system = System1D([1, 0, 0], [0, 0, 1], mpo_ti(h), S.copy(), rb.copy(), lb.copy())
        out[f"e{case}_h"], out[f"e{case}_S"], out[f"e{case}_rb"], out[f"e{case}_lb"] = np.array(h), S, rb, lb
        out[f"e{case}_E"] = np.array(complex(system.computeExpectation()))
        out[f"e{case}_one"] = np.array(complex(system.computeOneSiteExpectation()))
    np.savez_compressed(os.path.join(HERE, "chain1d.npz"), **out)


# operator-term compression followed by absorptions in every direction: the
# compressed tags (non-unit operator axes) go through the corner, side and
# stage rules; (corner, direction, contractions before, new dimension)
OPCOMP_CASES = [(0, 0, 3, 2), (1, 1, 2, 1), (2, 1, 4, 2), (3, 0, 2, 1), (0, 0, 3, 3), (2, 0, 2, 2)]


def opcomp():
    from carcassonne.system._2d import sideFromCorner
    from carcassonne.utils import L, R, O
    rng = np.random.default_rng(77)
    out = {}
    for case, (corner_id, direction, terms, new_dim) in enumerate(OPCOMP_CASES):
        side_id = sideFromCorner(corner_id, direction)
        a, b = cn(rng, 2, 2), cn(rng, 2, 2)
        ops = np.stack([(a + a.conj().T) / 2, (b + b.conj().T) / 2])
        kw = "OO_LR" if side_id in (1, 3) else "OO_UD"
        system = System.newTrivialWithSimpleSparseOperator(**{kw: [D(ops[0]), D(ops[1])]})
        system.contractTowards(R(side_id) if direction == 0 else L(side_id))
        for _ in range(terms):
            system.contractTowards(side_id)
        e0, n0 = system.computeExpectationAndNormalization()
        system.compressCornerTwoSiteOperatorTowards(corner_id, direction, new_dim)
        e1, n1 = system.computeExpectationAndNormalization()
        seq = [(complex(e0), complex(n0)), (complex(e1), complex(n1))]
        dirs = [side_id, (side_id + 1) % 4, O(side_id), (side_id + 3) % 4, side_id]
        for d in dirs:
            system.contractTowards(d)
            e, n = system.computeExpectationAndNormalization()
            seq.append((complex(e), complex(n)))
        out[f"c{case}_ops"] = ops
        out[f"c{case}_spec"] = np.array([corner_id, direction, terms, new_dim])
        out[f"c{case}_dirs"] = np.array(dirs)
        out[f"c{case}_EN"] = np.array(seq)
    np.savez_compressed(os.path.join(HERE, "opcomp.npz"), **out)


# --- config-sized cases --------------------------------------------------------
# The benchmark's shapes: the matvec microbenchmark (transverse Ising after one
# absorption round, 9 terms, D=4, chi=32 = 8x4, seed 1), the same shapes with
# the Heisenberg operator and complex boundaries, the Hermitian solve pencil
# (Heisenberg after one round, 20 terms, D=4, chi=64 = 8x8, seed 2), and two
# growth runs: transverse Ising h=3 (D=2, per-layer boundary dimension
# compressed to 8, i.e. chi=64, 20 absorptions, seed 0) and Heisenberg (D=4,
# compressed to 8, first 8 absorptions, seed 2).  Inputs come from the
# package's own seeded generators (carcassonne_gb300.workloads) and are handed
# to the reference with the same tags; every output is the reference's.

def _ref_tag(t):
    from tagrepr import parse_tag  # tests/tagrepr.py
    k = parse_tag(repr(t))
    if k[0] == "I":
        return rsparse.Identity()
    if k[0] == "C":
        return rsparse.Complete()
    if k[0] == "O":
        return rsparse.OneSiteOperator(None)
    if k[0] == "T":
        return rsparse.TwoSiteOperator(k[1], k[2], k[3])
    return rsparse.TwoSiteOperatorCompressed(k[1])


def _multiplier_cases(out, key, corners, sides, op, nx, seed):
    rc = [{_ref_tag(t): D(a) for t, a in lst} for lst in corners]
    rs = [{_ref_tag(t): D(a) for t, a in lst} for lst in sides]
    ro = {_ref_tag(t): D(a) for t, a in op}
    Hm, Nm = rsp2.formExpectationAndNormalizationMultipliers(rc, rs, ro)
    rng = np.random.default_rng(seed)
    H = Hm.formMatrix().toArray().copy()
    N = Nm.formMatrix().toArray().copy()
    vshape = tuple(int(lst[0][1].shape[6]) for lst in sides) + (int(op[0][1].shape[0]),)
    x = cn(rng, nx, *vshape)
    out[key + "_x"] = x
    out[key + "_Hx"] = np.stack([Hm(D(x[i].copy())).toArray().copy() for i in range(nx)])
    out[key + "_Nx"] = np.stack([Nm(D(x[i].copy())).toArray().copy() for i in range(nx)])
    out[key + "_H_cols"], out[key + "_N_cols"] = H[:, :8].copy(), N[:, :8].copy()
    out[key + "_H_diag"], out[key + "_N_diag"] = np.diag(H).copy(), np.diag(N).copy()
    out[key + "_H_fro"] = np.array([np.linalg.norm(H), np.linalg.norm(N)])
    out[key + "_cost"] = np.array([Hm.cost_of_multiply, Hm.cost_of_formMatrix, Nm.cost_of_multiply])
    return H, N


def _grow(name, system, steps, new_dimension, out, seed_base):
    """Per step: the lowest generalized eigenvalue of the step's (H_eff, N_eff)
    (dense eigh, as minimizeExpectationUsingFullEigensolver), ARPACK's eigsh
    and relaxOver from the current center; then a seeded random unit center
    (re and im N(0,1), default_rng(seed_base + step)) is absorbed by
    contractTowards(step % 4), and compressCornerStateTowards(corner,
    direction, new_dimension) runs for every corner axis above new_dimension.
    Absorbing the minimized center instead degenerates from this start: the
    transverse-Ising minimizer is the all-up product state at every step (the
    environment's X halves average to zero), whose rank-one boundaries make
    the compressor's normal equations singular (GMRES's assert,
    compression.py:43, failed on every retry), and the Heisenberg center's
    first effective Hamiltonian is zero.  The compressor matrices the
    reference computes are recorded in order, with the numpy seed of the
    attempt that succeeded; a failed attempt is retried with the next seed and
    logged."""
    import scipy.linalg as sla
    from scipy.sparse.linalg import LinearOperator, eigsh
    import carcassonne.system._2d as rsys
    orig = rsys.computeProductCompressor
    recorded = []

    def recording(Ld, Rd, nd):
        P = orig(Ld, Rd, nd)
        recorded.append(P.toArray().copy())
        return P
    rsys.computeProductCompressor = recording
    energies, comps, retries = [], [], []
    try:
        for step in range(steps):
            direction = step % 4
            Hm, Nm = system.formExpectationAndNormalizationMultipliers()
            H = Hm.formMatrix().toArray()
            N = Nm.formMatrix().toArray()
            w, v = sla.eigh(H, N)
            shape = system.state_center_data.shape
            n = H.shape[0]
            ar = np.nan
            if n > 2 and np.abs(H).max() > 0:  # ARPACK rejects the zero operator (a Heisenberg center's first step)
                op = LinearOperator((n, n), matvec=lambda u: Hm(D(u.reshape(shape).copy())).toArray().ravel(),
                                    dtype=np.complex128)
                ar = float(eigsh(op, k=1, M=N, which="SA", tol=1e-10)[0][0])
            np.random.seed(seed_base + 7919 * step)
            relax = np.nan
            if np.abs(H).max() > 0:
                x = relaxOver(D(system.state_center_data.toArray().copy()), Hm, Nm,
                              maximum_number_of_multiplications=100)
                xr = x.toArray().ravel()
                relax = float((np.vdot(xr, H @ xr) / np.vdot(xr, N @ xr)).real)
            rs = np.random.default_rng(seed_base + step)
            absorbed = cn(rs, *shape)
            absorbed /= np.linalg.norm(absorbed)
            system.setStateCenter(NDArrayData(absorbed.copy()))
            out[f"{name}_{step}_absorbed"] = absorbed
            system.contractTowards(direction)
            e, nrm = system.computeExpectationAndNormalization()
            energies.append([w[0], ar, relax, complex(e).real, complex(nrm).real, n,
                             sum(len(s) for s in system.sides), len(system.corners[0])])
            for corner_id in range(4):
                for cdir, axis in ((0, 0), (1, 3)):
                    if system.corners[corner_id][rsparse.Identity()].shape[axis] <= new_dimension:
                        continue
                    for attempt in range(8):
                        seed = seed_base + 1000 * step + 10 * corner_id + cdir + 100000 * attempt
                        np.random.seed(seed)
                        try:
                            system.compressCornerStateTowards(corner_id, cdir, new_dimension)
                        except AssertionError as exc:
                            retries.append([step, corner_id, cdir, attempt])
                            print("  %s step %d corner %d dir %d: attempt %d failed (%r), retrying"
                                  % (name, step, corner_id, cdir, attempt, exc))
                            recorded.clear()
                            continue
                        P = recorded.pop()
                        recorded.clear()
                        out[f"{name}_P{len(comps)}"] = P
                        comps.append([step, corner_id, cdir, seed])
                        break
                    else:
                        raise RuntimeError("%s: compression failed 8 times at step %d" % (name, step))
            print("  %s step %d: E=%.12f (eigsh %.12f, relaxOver %.12f), n=%d, side tags %d, compressions %d"
                  % (name, step, w[0], ar, relax, n, energies[-1][6], len(comps)))
    finally:
        rsys.computeProductCompressor = orig
    out[f"{name}_E"] = np.array(energies, dtype=np.float64)
    out[f"{name}_comps"] = np.array(comps, dtype=np.int64).reshape(-1, 4)
    out[f"{name}_retries"] = np.array(retries, dtype=np.int64).reshape(-1, 4)


def configs():
    import time
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    sys.path.insert(0, os.path.dirname(HERE))
    from carcassonne_gb300 import workloads
    out = {}
    t0 = time.time()
    c, s, o = workloads.matvec_problem_arrays(D=4, c_ket=8, c_bra=4, seed=1)
    _multiplier_cases(out, "mv", c, s, o, nx=8, seed=101)
    print("matvec operator: %.1f s" % (time.time() - t0))
    c, s, o = workloads.matvec_problem_arrays(D=4, c_ket=8, c_bra=4, seed=4,
                                              op_arrays=workloads.heisenberg_operator_arrays(), complex_=True)
    _multiplier_cases(out, "mvz", c, s, o, nx=4, seed=102)
    print("complex matvec operator: %.1f s" % (time.time() - t0))
    import scipy.linalg as sla
    c, s, o = workloads.hermitian_problem_arrays(D=4, c=8, seed=2)
    H, N = _multiplier_cases(out, "pencil", c, s, o, nx=2, seed=103)
    w, v = sla.eigh(H, N)
    out["pencil_E"] = np.array(w[:4])
    out["pencil_v"] = v[:, 0].copy()
    print("solve pencil: %.1f s" % (time.time() - t0))
    ops = operators()
    op = {k: NDArrayData(v.toArray().copy()) for k, v in ops["ti"]().items()}
    _grow("ti20", bond_system(op, 2, 0), 20, 8, out, seed_base=workloads.GROWTH_CENTER_SEED["ti"])
    print("TI growth: %.1f s" % (time.time() - t0))
    op = {k: NDArrayData(v.toArray().copy()) for k, v in ops["heis"]().items()}
    _grow("heis8", bond_system(op, 4, 2), 8, 8, out, seed_base=workloads.GROWTH_CENTER_SEED["heis"])
    print("Heisenberg growth: %.1f s" % (time.time() - t0))
    np.savez_compressed(os.path.join(HERE, "configs.npz"), **out)


if __name__ == "__main__":
    sections = dict(dense=dense_cases, tables=tables_and_trajectories, numerics=numerics, chain1d=chain1d,
                    opcomp=opcomp, configs=configs)
    chosen = sys.argv[1:] or list(sections)
    for name in chosen:
        sections[name]()
    for fn in ("dense.npz", "tables.json", "trajectory.npz", "numerics.npz", "chain1d.npz", "opcomp.npz",
               "configs.npz"):
        if os.path.exists(os.path.join(HERE, fn)):
            print(fn, os.path.getsize(os.path.join(HERE, fn)))
