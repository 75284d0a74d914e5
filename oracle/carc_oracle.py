"""CPU oracle for the center-site optimisation path (test infrastructure only).

This module is the checker, never the product: only the tests, the smoke
check and the CPU-baseline leg of the benchmark import it.  It restates, in
plain numpy, the algorithm of gcross/Carcassonne's center-site path so that
the CUDA implementation can be compared with it on machines where the
reference itself is not installed.

Parity pin: every function here is checked against golden vectors produced by
running the reference itself (``tests/golden/make_golden.py`` imports the
reference and writes ``tests/golden/*.npz`` / ``*.json``;
``tests/test_oracle_golden.py`` compares this module with them).

Data model (same as the reference): a boundary is an insertion-ordered dict
``{tag: ndarray}``; tags are small tuples here:
    ("I",)                 Identity           (sparse.py:25-29)
    ("C",)                 Complete           (sparse.py:30-34)
    ("O", None)            OneSiteOperator    (sparse.py:35-55; its id is always None)
    ("T", id, dir, pos)    TwoSiteOperator    (sparse.py:56-166)
    ("TC", dir)            TwoSiteOperatorCompressed (sparse.py:167-208)
Directions LEFT=0, RIGHT=1, CENTER=2 (sparse.py:211-215).
"""
from __future__ import annotations

import itertools
import numpy as np
import scipy.linalg as sla

LEFT, RIGHT, CENTER = 0, 1, 2
I_TAG = ("I",)
C_TAG = ("C",)


# --------------------------------------------------------------------------
# index helpers                                           (utils.py:886-892)
# --------------------------------------------------------------------------
def O(i): return (i + 2) % 4
def L(i): return (i + 1) % 4
def R(i): return (i - 1) % 4
def A(d, i): return i - 1 if i > d else i
def OA(i): return A(i, O(i))
def LA(i): return A(i, L(i))
def RA(i): return A(i, R(i))


def side_from_corner(corner_id, direction):          # system/_2d.py:573-574
    return (corner_id + 1 - direction) % 4


# --------------------------------------------------------------------------
# tags and their matching rules                           (sparse.py:56-208)
# --------------------------------------------------------------------------
def ttype(tag):
    return tag[0]


def T(id_, d, p=None):
    return ("T", id_, d, p)


def t_matches(l, r):                                   # sparse.py:84-91 / :181-184
    if l[0] == "T":
        if l[1] == r[1] and l[2] == RIGHT and r[2] == LEFT and l[3] == r[3]:
            return C_TAG
        return None
    if l[1] == RIGHT and r[1] == LEFT:
        return C_TAG
    return None


def t_matches_center(s, side_direction, c):            # sparse.py:92-99
    if s[1] == c[1] and s[2] == CENTER and side_direction == c[2]:
        return C_TAG
    return None


def t_matches_center_identity(s):                      # sparse.py:100-103
    if s[2] != CENTER:
        return T(s[1], s[2], s[3] + 1)
    return None


def t_matches_center_for_stage3(s, direction, other):  # sparse.py:104-110
    return s[1] == other[1] and s[2] == CENTER and s[3] + 2 * direction == other[2]


def t_matches_corner_identity_on_left(s):              # sparse.py:111-116
    if s[2] == RIGHT:
        return s
    if s[2] == CENTER:
        return T(s[1], LEFT, 0)
    return None


def t_matches_corner_identity_on_left_for_stage1(s):   # sparse.py:117-120, :185-188
    if s[0] == "T":
        return s if s[2] in (RIGHT, CENTER) else None
    return s if s[1] == RIGHT else None


def t_matches_corner_identity_on_right(s):             # sparse.py:121-126
    if s[2] == LEFT:
        return s
    if s[2] == CENTER:
        return T(s[1], RIGHT, 0)
    return None


def t_matches_side_identity_on_left(s):                # sparse.py:127-130
    return T(s[1], s[2], s[3] + 1) if s[2] == RIGHT else None


def t_matches_side_identity_on_right(s):               # sparse.py:131-134
    return T(s[1], s[2], s[3] + 1) if s[2] == LEFT else None


def t_matches_side_identity_on_right_for_stage1(s):    # sparse.py:135-138, :189-192
    d = s[2] if s[0] == "T" else s[1]
    return s if d == LEFT else None


def t_matches_side_identity_outward(s, direction):     # sparse.py:139-146
    if s[2] == L(direction):
        return T(s[1], LEFT, 0)
    if s[2] == R(direction):
        return T(s[1], RIGHT, 0)
    if s[2] == O(direction):
        return T(s[1], CENTER, None)
    return None


def t_matches_stage1_identity_on_left(s):              # sparse.py:147-152, :193-196
    if s[0] == "TC":
        return s if s[1] == RIGHT else None
    if s[2] == RIGHT:
        return s
    if s[2] == CENTER:
        return T(s[1], CENTER, LEFT)
    return None


def t_matches_stage1_identity_on_right(s):             # sparse.py:153-158, :197-200
    if s[0] == "TC":
        return s if s[1] == LEFT else None
    if s[2] == LEFT:
        return s
    if s[2] == CENTER:
        return T(s[1], CENTER, RIGHT)
    return None


def t_matches_for_stage3(x, y):                        # sparse.py:159-165, :201-203
    if x[0] == "TC":
        return (x[1], y[1]) in ((LEFT, RIGHT), (RIGHT, LEFT))
    return x[1] == y[1] and (x[2], y[2]) in ((LEFT, RIGHT), (RIGHT, LEFT)) and x[3] == y[3]


# --------------------------------------------------------------------------
# sparse contraction driver                               (sparse.py:218-240)
# --------------------------------------------------------------------------
def standard_terms():                                  # sparse.py:218-222
    return {
        ("I", "I"): lambda a, b: I_TAG,
        ("C", "I"): lambda a, b: C_TAG,
        ("I", "C"): lambda a, b: C_TAG,
    }


def sparse_table(rules, tags_1, tags_2):
    """The tag-pair schedule of ``contractSparseTensors`` (sparse.py:223-240).

    Returns (result_tags, entries) where entries lists (i1, i2, i_out) in the
    reference's iteration order (outer loop over tensor_1, inner over
    tensor_2) and result tags appear in first-insertion order.
    """
    result_tags = []
    entries = []
    for i1, t1 in enumerate(tags_1):
        for i2, t2 in enumerate(tags_2):
            rule = rules.get((t1[0], t2[0]))
            if rule is None:
                continue
            out = rule(t1, t2)
            if out is None:
                continue
            if out not in result_tags:
                result_tags.append(out)
            entries.append((i1, i2, result_tags.index(out)))
    return result_tags, entries


def contract_sparse(rules, dense, t1, t2):
    k1, k2 = list(t1), list(t2)
    out_tags, entries = sparse_table(rules, k1, k2)
    out = {}
    for i1, i2, io in entries:
        v = dense(t1[k1[i1]], t2[k2[i2]])
        tag = out_tags[io]
        out[tag] = out[tag] + v if tag in out else v
    return out


def rules_absorb_corner_left():                        # tensors/_2d/sparse.py:12-23
    r = standard_terms()
    r[("T", "I")] = lambda c, s: t_matches_side_identity_on_left(c)
    r[("I", "T")] = lambda c, s: t_matches_corner_identity_on_right(s)
    r[("T", "T")] = lambda c, s: t_matches(s, c)
    r[("TC", "TC")] = lambda c, s: t_matches(s, c)
    return r


def rules_absorb_corner_right():                       # tensors/_2d/sparse.py:24-35
    r = standard_terms()
    r[("T", "I")] = lambda c, s: t_matches_side_identity_on_right(c)
    r[("I", "T")] = lambda c, s: t_matches_corner_identity_on_left(s)
    r[("T", "T")] = lambda c, s: t_matches(c, s)
    r[("TC", "TC")] = lambda c, s: t_matches(s, c)
    return r


def rules_absorb_center(direction):
    """(side tag, operator tag) -> (result tag, uses operator?)   (tensors/_2d/sparse.py:36-58)"""
    return {
        ("I", "I"): lambda s, c: (I_TAG, False),
        ("C", "I"): lambda s, c: (C_TAG, False),
        ("I", "O"): lambda s, c: (C_TAG, True),
        ("T", "I"): lambda s, c: (t_matches_center_identity(s), False),
        ("I", "T"): lambda s, c: (t_matches_side_identity_outward(c, direction), True),
        ("T", "T"): lambda s, c: (t_matches_center(s, direction, c), True),
        ("TC", "I"): lambda s, c: (s, False),
    }


def rules_stage1():                                    # tensors/_2d/sparse.py:72-85
    r = standard_terms()
    r[("T", "I")] = lambda c, s: t_matches_side_identity_on_right_for_stage1(c)
    r[("I", "T")] = lambda c, s: t_matches_corner_identity_on_left_for_stage1(s)
    r[("T", "T")] = lambda c, s: t_matches(c, s)
    r[("TC", "I")] = lambda c, s: t_matches_side_identity_on_right_for_stage1(c)
    r[("I", "TC")] = lambda c, s: t_matches_corner_identity_on_left_for_stage1(s)
    r[("TC", "TC")] = lambda c, s: t_matches(c, s)
    return r


def rules_stage2():                                    # tensors/_2d/sparse.py:86-99
    r = standard_terms()
    r[("T", "I")] = lambda a, b: t_matches_stage1_identity_on_left(a)
    r[("I", "T")] = lambda a, b: t_matches_stage1_identity_on_right(b)
    r[("T", "T")] = lambda a, b: t_matches(b, a)
    r[("TC", "I")] = lambda a, b: t_matches_stage1_identity_on_left(a)
    r[("I", "TC")] = lambda a, b: t_matches_stage1_identity_on_right(b)
    r[("TC", "TC")] = lambda a, b: t_matches(b, a)
    return r


def stage3_terms(tags_0, tags_1, tags_op):
    """Term list of formExpectationStage3 (tensors/_2d/sparse.py:100-127):
    (i0, i1, iop, is_identity_op) in itertools.product order."""
    rules = {
        ("C", "I", "I"): lambda x, y, z: True,
        ("I", "C", "I"): lambda x, y, z: True,
        ("I", "I", "O"): lambda x, y, z: True,
        ("T", "I", "T"): lambda x, y, z: t_matches_center_for_stage3(x, 0, z),
        ("I", "T", "T"): lambda x, y, z: t_matches_center_for_stage3(y, 1, z),
        ("T", "T", "I"): lambda x, y, z: t_matches_for_stage3(x, y),
        ("TC", "TC", "I"): lambda x, y, z: t_matches_for_stage3(x, y),
    }
    terms = []
    for (i0, x), (i1, y), (i2, z) in itertools.product(enumerate(tags_0), enumerate(tags_1), enumerate(tags_op)):
        rule = rules.get((x[0], y[0], z[0]))
        if rule is None or not rule(x, y, z):
            continue
        terms.append((i0, i1, i2, z == I_TAG))
    return terms


# --------------------------------------------------------------------------
# dense contractors                                 (tensors/_2d/dense.py)
# index contracts restated from tests/test_tensors_dense.py
# --------------------------------------------------------------------------
def absorb_side_into_corner_from_left(corner, side):   # dense.py:10-15, test :27-29
    a, b, c = side.shape[0:3]
    d, e, f = corner.shape[3:6]
    j, k = side.shape[6:8]
    t = np.einsum("xyzdef,abcxyzjk->abcdjekf", corner, side)
    return t.reshape(a, b, c, d * j, e * k, f)


def absorb_side_into_corner_from_right(corner, side):  # dense.py:16-21, test :47-49
    a, b, c = corner.shape[0:3]
    g, h, i = side.shape[3:6]
    j, k = side.shape[6:8]
    t = np.einsum("abcxyz,xyzghijk->ajbkcghi", corner, side)
    return t.reshape(a * j, b * k, c, g, h, i)


def _center_pair(direction, state, state_conj, op):
    """E[s_L,s_R,s_O, t_L,t_R,t_O, k, l] = sum_{p,q} S[..k@dir..,q] O[p,q] conj(S)[..l@dir..,p]
    (dense.py:22-81, test :74-87 / :110-124)."""
    perm = [L(direction), R(direction), O(direction), direction]
    s = np.transpose(state, perm + [4])
    sc = np.transpose(state_conj, perm + [4])
    if op is None:
        return np.einsum("abckq,deflq->abcdefkl", s, sc)
    return np.einsum("abckq,pq,deflp->abcdefkl", s, op, sc)


def absorb_center_into_side(direction, side, state, op=None, state_conj=None):
    """absorbDenseCenterSSIntoSide / absorbDenseCenterSOSIntoSide (dense.py:22-81)."""
    if state_conj is None:
        state_conj = state.conj()
    e = _center_pair(direction, state, state_conj, op)
    a, b, c, d, ee, f = side.shape[:6]
    sL, sR, sO = state.shape[L(direction)], state.shape[R(direction)], state.shape[O(direction)]
    tL, tR, tO = state_conj.shape[L(direction)], state_conj.shape[R(direction)], state_conj.shape[O(direction)]
    out = np.einsum("abcdefkl,uvwxyzkl->aubxcdveyfwz", side, e)
    return out.reshape(a * sL, b * tL, c, d * sR, ee * tR, f, sO, tO)


def stage1(corner, side):                              # dense.py:95-100, test :150-152
    a = corner.shape[0] * corner.shape[1] * corner.shape[2]
    x = corner.shape[3] * corner.shape[4] * corner.shape[5]
    b = side.shape[3] * side.shape[4] * side.shape[5]
    return (corner.reshape(a, x) @ side.reshape(x, -1)).reshape(a, b, side.shape[6], side.shape[7])


def stage2(s1_0, s1_1):                                # dense.py:101-113, test :166-168
    return np.einsum("abkl,camn->cbkmln", s1_0, s1_1)


def stage3_matvec(s2_0, s2_1, op, v):
    """formDenseStage3 multiply (dense.py:145-174); op None -> formNormalizationStage3 (:114-144).
    y[l0,l1,l2,l3,p] = sum S2_0[x,y,k0,k1,l0,l1] S2_1[y,x,k2,k3,l2,l3] O[p,q] v[k0,k1,k2,k3,q]."""
    w = v if op is None else np.einsum("pq,abcdq->abcdp", op, v)
    return np.einsum("xyabef,yxcdgh,abcdp->efghp", s2_0, s2_1, w, optimize=True)


def stage3_matrix(s2_0, s2_1, op):
    """formDenseStage3_formMatrix (dense.py:175-195): H[(l,p),(k,q)]."""
    h = np.einsum("xyabef,yxcdgh->efghabcd", s2_0, s2_1, optimize=True)
    n = h.shape[0] * h.shape[1] * h.shape[2] * h.shape[3]
    h = h.reshape(n, n)
    return np.kron(h, op)


def normalization_submatrix(s2_0, s2_1):               # dense.py:204-225
    h = np.einsum("xyabef,yxcdgh->efghabcd", s2_0, s2_1, optimize=True)
    n = h.shape[0] * h.shape[1] * h.shape[2] * h.shape[3]
    return h.reshape(n, n)


# --------------------------------------------------------------------------
# sparse (tag-level) operations            (tensors/_2d/sparse.py:12-161)
# --------------------------------------------------------------------------
def absorb_sparse_side_into_corner_from_left(corner, side):
    return contract_sparse(rules_absorb_corner_left(), absorb_side_into_corner_from_left, corner, side)


def absorb_sparse_side_into_corner_from_right(corner, side):
    return contract_sparse(rules_absorb_corner_right(), absorb_side_into_corner_from_right, corner, side)


def absorb_sparse_center_into_side(direction, side, state, op_center, state_conj=None):
    if state_conj is None:
        state_conj = state.conj()
    rules = rules_absorb_center(direction)
    ks, ko = list(side), list(op_center)
    out = {}
    for s in ks:
        for c in ko:
            rule = rules.get((s[0], c[0]))
            if rule is None:
                continue
            tag, with_op = rule(s, c)
            if tag is None:
                continue
            v = absorb_center_into_side(direction, side[s], state, op_center[c] if with_op else None, state_conj)
            out[tag] = out[tag] + v if tag in out else v
    return out


def expectation_stage1(corner, side):
    return contract_sparse(rules_stage1(), stage1, corner, side)


def expectation_stage2(s1_0, s1_1):
    return contract_sparse(rules_stage2(), stage2, s1_0, s1_1)


class Multiplier:
    """Restatement of utils.Multiplier (utils.py:180-207) over numpy arrays."""

    def __init__(self, shape, multiply, cost_of_multiply, form_matrix, cost_of_form_matrix):
        self.shape = shape
        self.multiply = multiply
        self.cost_of_multiply = cost_of_multiply
        self.formMatrix = form_matrix
        self.cost_of_formMatrix = cost_of_form_matrix

    def __call__(self, v):
        return self.multiply(v)

    def isCheaperToFormMatrix(self, n):                # utils.py:203-206
        return n * self.cost_of_multiply > self.cost_of_formMatrix + n * self.shape[0] * self.shape[1]


def stage3_costs(s2_0, s2_1, d, identity_op):
    """CostTracker counts (data/cost_tracker.py:17-22) of the stage-3 contractors."""
    x = s2_0.shape[0] * s2_0.shape[1]
    k0, k1, l0, l1 = s2_0.shape[2:6]
    k2, k3, l2, l3 = s2_1.shape[2:6]
    mult = x * l0 * l1 * k0 * k1 * k2 * k3 * d + x * l0 * l1 * l2 * l3 * k2 * k3 * d
    if not identity_op:
        mult += k0 * k1 * k2 * k3 * d * d
    form = l0 * l1 * k0 * k1 * l2 * l3 * k2 * k3 * x + (l0 * l1 * k0 * k1 * l2 * l3 * k2 * k3) * d * d
    return mult, form


def expectation_and_normalization_multipliers(corners, sides, op_center):
    """formExpectationAndNormalizationMultipliers (tensors/_2d/sparse.py:59-71, :100-161)."""
    s1 = [expectation_stage1(corners[i], sides[i]) for i in range(4)]
    s2_0 = expectation_stage2(s1[0], s1[1])
    s2_1 = expectation_stage2(s1[2], s1[3])
    k0, k1, ko = list(s2_0), list(s2_1), list(op_center)
    terms = stage3_terms(k0, k1, ko)
    d = next(iter(op_center.values())).shape[0]
    ident = np.eye(d, dtype=np.complex128)

    def multiply(v):
        y = np.zeros_like(v)
        for i0, i1, io, is_id in terms:
            y = y + stage3_matvec(s2_0[k0[i0]], s2_1[k1[i1]], None if is_id else op_center[ko[io]], v)
        return y

    ni = s2_0[I_TAG]
    n = ni.shape[2] * ni.shape[3] * s2_1[I_TAG].shape[2] * s2_1[I_TAG].shape[3] * d

    def form():
        m = np.zeros((n, n), np.complex128)
        for i0, i1, io, is_id in terms:
            m = m + stage3_matrix(s2_0[k0[i0]], s2_1[k1[i1]], ident if is_id else op_center[ko[io]])
        return m

    cm = cf = 0
    for i0, i1, io, is_id in terms:
        a, b = stage3_costs(s2_0[k0[i0]], s2_1[k1[i1]], d, is_id)
        cm += a
        cf += b
    H = Multiplier((n, n), multiply, cm, form, cf)
    a, b = stage3_costs(s2_0[I_TAG], s2_1[I_TAG], d, True)
    Nm = Multiplier((n, n), lambda v: stage3_matvec(s2_0[I_TAG], s2_1[I_TAG], None, v), a,
                    lambda: stage3_matrix(s2_0[I_TAG], s2_1[I_TAG], ident), b)
    return H, Nm, dict(s1=s1, s2_0=s2_0, s2_1=s2_1, terms=terms)


# --------------------------------------------------------------------------
# numerics                                   (utils.py, data/__init__.py)
# --------------------------------------------------------------------------
def relax_over(initial, H, N=None, maximum_number_of_multiplications=None, tolerance=1e-7,
               dimension_of_krylov_space=None):
    """Restarted Krylov / Rayleigh-Ritz eigensolver of utils.relaxOver (utils.py:805-878).
    H and N are dense matrices here (the reference forms them whenever that is
    cheaper, which holds at every size these tests use)."""
    shape = initial.shape
    v0 = initial.ravel().astype(np.complex128)
    v0 = v0 / np.linalg.norm(v0)
    n = v0.size
    k = 3 if dimension_of_krylov_space is None else dimension_of_krylov_space
    if N is None:
        apply_inv_n = lambda x: x
    else:
        lu = sla.lu_factor(N)
        apply_inv_n = lambda x: sla.lu_solve(lu, x)
    mult = lambda x: apply_inv_n(H @ x)
    initial_value = np.vdot(v0, mult(v0))
    count = 0
    last = None
    complete = k == n
    while True:
        basis = np.zeros((k, n), np.complex128)
        mbasis = np.zeros((k, n), np.complex128)
        basis[0] = v0
        for i in range(k):
            mbasis[i] = mult(basis[i])
            if i < k - 1:
                nxt = mbasis[i] - (basis[:i + 1].conj() @ mbasis[i]) @ basis[:i + 1]
                nrm = np.linalg.norm(nxt)
                if nrm <= 1e-14:
                    complete = True
                    basis = basis[:i + 1]
                    mbasis = mbasis[:i + 1]
                    break
                basis[i + 1] = nxt / nrm
        count += k
        small = basis.conj() @ mbasis.T
        ev, evec = sla.eig(small)
        j = int(np.argmin(ev.real))
        lam = ev[j]
        u = evec[:, j]
        if complete or (last is not None and abs(last - lam) <= tolerance) or \
                (maximum_number_of_multiplications is not None and count >= maximum_number_of_multiplications):
            final = u @ basis
            final = final / np.linalg.norm(final)
            fv = np.vdot(final, mult(final))
            if (fv - initial_value) / (abs(fv) + abs(initial_value)) > 1 + 1e-7:
                raise RuntimeError("RelaxFailed")
            return final.reshape(shape), lam, count
        v0 = u @ basis
        v0 = v0 / np.linalg.norm(v0)
        last = lam


def lowest_generalized(Hm, Nm):
    """Dense generalized eigh, lowest pair (system/_2d.py:498-502)."""
    w, v = sla.eigh(Hm, Nm)
    return w[0], v[:, 0]


def normalize_axis(t, axis, sqrt_svals=False, dont_recip_under=1e-14):
    """NDArrayData.normalizeAxis (data/__init__.py:263-301)."""
    if t.shape[axis] == 1:
        n = np.linalg.norm(t)
        if sqrt_svals:
            n = np.sqrt(n)
            return np.array([[1 / n]]), np.array([[n]])
        return t / n, np.array([[1 / n]]), np.array([[n]])
    others = [i for i in range(t.ndim) if i != axis]
    m = np.transpose(t, others + [axis]).reshape(-1, t.shape[axis])
    if m.shape[0] < m.shape[1]:
        raise ValueError("not enough degrees of freedom to normalize axis")
    u, s, vh = sla.svd(m, full_matrices=False)
    uv = u @ vh
    si = s.copy()
    if dont_recip_under:
        nz = np.abs(si) > dont_recip_under
        si[nz] = 1.0 / si[nz]
    else:
        si = 1.0 / si
    S = s.reshape(-1, 1)
    SI = si.reshape(-1, 1)
    if sqrt_svals:
        return (vh * np.sqrt(SI)).conj(), vh * np.sqrt(S)
    split = [t.shape[i] for i in others] + [uv.shape[1]]
    inv = list(range(t.ndim - 1))
    inv.insert(axis, t.ndim - 1)
    iso = uv.reshape(split).transpose(inv)
    return iso, vh.T @ (vh * SI).conj(), vh.T.conj() @ (vh * S)


def absorb_matrix_at(t, axis, m):                      # data/__init__.py:148-150
    r = np.tensordot(m, t, (1, axis))
    perm = list(range(1, axis + 1)) + [0] + list(range(axis + 1, t.ndim))
    return np.transpose(r, perm)


def unitize(m):                                        # utils.py:879-882
    u, _, vh = sla.svd(m, full_matrices=False)
    return u @ vh


def product_compressor_matrix(Lt, Rt, P):
    """The A matrix of computeProductCompressor (compression.py:11-25).

    Tensors of the reference's join list: 0=L (l,a,b,o), 1=conj(P), 2=conj(P)^T,
    3=P^T, 4=R (c,e,o,r); rows (L.0, R.3), columns (L.1, MRU.0):
    A[(l,r),(a,i)] = sum L[l,a,b,o] conj(P[b,j]) conj(P[c,i]) P[e,j] R[c,e,o,r].
    """
    out = np.einsum("labo,bj,ci,ej,ceor->lrai", Lt, P.conj(), P.conj(), P, Rt, optimize=True)
    l, r, a, i = out.shape
    return out.reshape(l * r, a * i)


def product_compressor(Lt, Rt, new_dimension, initial, rounds=4):
    """computeProductCompressor (compression.py:26-46) with an explicit initial
    compressor (the reference draws it from numpy's global RNG) and a direct
    least-squares solve of the normal equations in place of GMRES."""
    old = Lt.shape[1]
    b = np.tensordot(Lt, Rt, ((1, 2, 3), (0, 1, 2))).ravel()
    P = unitize(initial)
    for _ in range(rounds):
        Am = product_compressor_matrix(Lt, Rt, P)
        x = sla.lstsq(Am, b)[0]
        P = unitize(x.reshape(old, new_dimension))
    return P.T


def compute_compressor(old_dimension, new_dimension, matrix, normalize=False):
    """computeCompressor (utils.py:268-302), eigh branch."""
    if new_dimension < 0 or new_dimension > old_dimension:
        raise ValueError("bad new dimension")
    if new_dimension == 0:
        z = np.zeros((0, old_dimension), np.complex128)
        return z, z
    w, v = sla.eigh(matrix)
    w = w[-new_dimension:]
    v = v[:, -new_dimension:].T
    while new_dimension > 0 and abs(w[new_dimension - 1]) < 1e-15:
        new_dimension -= 1
    if new_dimension == 0:
        raise ValueError("Input is filled with near-zero elements.")
    if normalize:
        s = np.sqrt(w).reshape(new_dimension, 1)
        return v * s, v / s
    return v, v


# --------------------------------------------------------------------------
# operator construction                                 (sparse.py:288-338)
# --------------------------------------------------------------------------
def make_sparse_operator(Os=(), OO_UDs=(), OO_LRs=()):
    op = {}
    ident = None
    for O_ in Os:
        op[("O", None)] = np.asarray(O_, np.complex128)
        ident = np.eye(O_.shape[0])
    for i, (u, d) in enumerate(OO_UDs):
        op[T(i, 3, 0)] = np.asarray(u, np.complex128)
        op[T(i, 1, 0)] = np.asarray(d, np.complex128)
        if ident is None:
            ident = np.eye(u.shape[0])
    for i, (l, r) in enumerate(OO_LRs):
        op[T(i, 0, 0)] = np.asarray(l, np.complex128)
        op[T(i, 2, 0)] = np.asarray(r, np.complex128)
        if ident is None:
            ident = np.eye(l.shape[0])
    if ident is None:
        raise ValueError("No terms have been specified.")
    op[I_TAG] = ident.astype(np.complex128)
    return op


PAULI_X = np.array([[0, 1], [1, 0]], np.complex128)
PAULI_Y = np.array([[0, -1j], [1j, 0]], np.complex128)
PAULI_Z = np.array([[1, 0], [0, -1]], np.complex128)


# --------------------------------------------------------------------------
# system                                              (system/_2d.py)
# --------------------------------------------------------------------------
class OracleSystem:
    """Restatement of the System operations on the path (system/_2d.py:97-557)."""

    def __init__(self, corners, sides, state, op_center):
        self.corners = [dict(c) for c in corners]
        self.sides = [dict(s) for s in sides]
        self.state = state
        self.op = op_center

    @classmethod
    def trivial(cls, op_center):                        # system/_2d.py:72-86
        d = next(iter(op_center.values())).shape[0]
        return cls([{I_TAG: np.ones((1,) * 6, np.complex128)} for _ in range(4)],
                   [{I_TAG: np.ones((1,) * 8, np.complex128)} for _ in range(4)],
                   np.full((1, 1, 1, 1, d), 1.0 / np.sqrt(d), np.complex128), op_center)

    def multipliers(self, op=None):
        return expectation_and_normalization_multipliers(self.corners, self.sides, self.op if op is None else op)

    def expectation_and_normalization(self):           # system/_2d.py:373-377, :429-430
        H, N, _ = self.multipliers()
        s = self.state
        e = np.vdot(s.ravel(), H(s).ravel())
        n = np.vdot(s.ravel(), N(s).ravel())
        return e / n, n

    def contract_unnormalized_towards(self, direction, state=None):   # system/_2d.py:443-454
        if state is None:
            state = self.state
        self.corners[direction] = absorb_sparse_side_into_corner_from_left(self.corners[direction], self.sides[L(direction)])
        self.sides[direction] = absorb_sparse_center_into_side(direction, self.sides[direction], state, self.op)
        self.corners[R(direction)] = absorb_sparse_side_into_corner_from_right(self.corners[R(direction)], self.sides[R(direction)])

    def contract_towards(self, direction):             # system/_2d.py:435-439
        iso, _, m = normalize_axis(self.state, O(direction))
        self.contract_unnormalized_towards(direction, iso)
        self.state = absorb_matrix_at(normalize_axis(self.state, direction)[0], direction, m)

    def minimize_full(self):                           # system/_2d.py:498-502
        H, N, _ = self.multipliers()
        w, v = lowest_generalized(H.formMatrix(), N.formMatrix())
        self.state = v.reshape(self.state.shape)
        return w

    def compress_corner_state_towards(self, corner_id, direction, new_dimension, initial, P=None):
        """compressCornerStateTowardsLeft/Right (system/_2d.py:191-228); a given
        compressor P (new, old) is applied instead of being computed."""
        mo = lambda f, s: {k: f(v) for k, v in s.items()}
        if direction == 0:
            sd = self.sides[L(corner_id)][I_TAG]
            side_j = np.transpose(sd, (0, 1, 2, 6, 7, 3, 4, 5)).reshape(-1, sd.shape[3], sd.shape[4], sd.shape[5])
            cd = self.corners[corner_id][I_TAG]
            corner_j = cd.reshape(cd.shape[0], cd.shape[1], cd.shape[2], -1)
            if P is None:
                P = product_compressor(side_j, corner_j, new_dimension, initial)
            self.sides[L(corner_id)] = mo(lambda x: absorb_matrix_at(absorb_matrix_at(x, 3, P), 4, P.conj()), self.sides[L(corner_id)])
            self.corners[corner_id] = mo(lambda x: absorb_matrix_at(absorb_matrix_at(x, 0, P.conj()), 1, P), self.corners[corner_id])
        else:
            cd = self.corners[corner_id][I_TAG]
            corner_j = cd.reshape(-1, cd.shape[3], cd.shape[4], cd.shape[5])
            sd = self.sides[corner_id][I_TAG]
            side_j = sd.reshape(sd.shape[0], sd.shape[1], sd.shape[2], -1)
            if P is None:
                P = product_compressor(corner_j, side_j, new_dimension, initial)
            self.corners[corner_id] = mo(lambda x: absorb_matrix_at(absorb_matrix_at(x, 3, P), 4, P.conj()), self.corners[corner_id])
            self.sides[corner_id] = mo(lambda x: absorb_matrix_at(absorb_matrix_at(x, 0, P.conj()), 1, P), self.sides[corner_id])
        return P


# ---------------------------------------------------------------------------
# 1D chain (tensors/_1d.py:12-93); index letters as in the GPU contractors:
# environments [o, s, t] (operator, ket, bra bonds), O[o_l, o_r, p, q],
# S[s_l, s_r, q], Sc = conj(S)
# ---------------------------------------------------------------------------
def chain_absorb_oss_left(L, O, S, Sc):                 # tensors/_1d.py:12-25
    return np.einsum("xyz,oxpq,syq,tzp->ost", L, O, S, Sc)


def chain_absorb_oss_right(R, O, S, Sc):                # tensors/_1d.py:26-39
    return np.einsum("xyz,xopq,ysq,ztp->ost", R, O, S, Sc)


def chain_absorb_ss_left(L, S, Sc):                     # tensors/_1d.py:40-49
    return np.einsum("yz,syp,tzp->st", L, S, Sc)


def chain_absorb_ss_right(R, S, Sc):                    # tensors/_1d.py:50-59
    return np.einsum("yz,ysp,ztp->st", R, S, Sc)


def chain_multiply(R, L, O, S):                         # tensors/_1d.py:61-93 (multiply)
    return np.einsum("xar,ubl,xuoq,abq->rlo", R, L, O, S)


def chain_form_matrix(R, L, O):                         # tensors/_1d.py:61-93 (formMatrix)
    m = np.einsum("xar,ubl,xuoq->rloabq", R, L, O)
    n = R.shape[2] * L.shape[2] * O.shape[2]
    return m.reshape(n, -1)
