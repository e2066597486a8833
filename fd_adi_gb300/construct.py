"""Host-side construction of operators from PDE coefficient/boundary dicts.

For engines configured the reference way -- dicts of coefficient functions
and boundary conditions (FiniteDifference/FiniteDifferenceEngine.pyx:72-152)
-- this builds the per-dimension operators once on the host with numpy
following make_discrete_operators and scale_and_combine_operators
(FiniteDifferenceEngine.pyx:423-592) and hands them to the GPU as
BandedOperator objects. Only centred schemes are supported, as on the
reference GPU path (FiniteDifferenceEngineGPU.pyx:634-635).

Row-aligned storage: ``rows[k, r]`` holds A[r, r + 2 - k] (offsets 2, 1, 0,
-1, -2) in the operator's block-major order.
"""
import itertools

import numpy as np

from .banded_operator import BandedOperator, CAN_FOLD, CANNOT_FOLD, _dev, centre_rows


class HostOp(object):
    def __init__(self, blocks, L, axis):
        self.blocks, self.L, self.axis = blocks, L, axis
        self.rows = np.zeros((5, blocks * L))
        self.R = np.zeros(blocks * L)
        self.low = None
        self.high = None
        self.top_status = CANNOT_FOLD
        self.bot_status = CANNOT_FOLD
        self.mixed = None      # (coeff, w0, w1, n0, n1) for the mixed operator
        self.derivative = 1

    def dirichlet_rows(self):
        m = np.zeros(self.blocks * self.L, dtype=bool)
        if self.low is not None:
            m[::self.L] = True
        if self.high is not None:
            m[self.L - 1::self.L] = True
        return m

    def vectorized_scale(self, vec):
        """BandedOperator.pyx:749-792 (Dirichlet rows unscaled)."""
        vec = np.array(vec, dtype=float)
        if self.mixed is not None:
            coeff = self.mixed[0] * vec
            self.mixed = (coeff,) + self.mixed[1:]
            self.R = self.R * vec
            return
        if vec.size == self.L and self.blocks > 1:
            vec = np.tile(vec, self.blocks)
        vec[self.dirichlet_rows()] = 1
        self.rows = self.rows * vec[None, :]
        self.R = self.R * vec

    def add_scalar_f32(self, val):
        """add_scalar with its C float argument (BandedOperator.pxd:32)."""
        v = float(np.float32(val))
        keep = ~self.dirichlet_rows()
        self.rows[2, keep] += v

    def add(self, other):
        """add_operator (BandedOperator.pyx:618-710)."""
        for k in (0, 1, 3, 4):
            self.rows[k] += other.rows[k]
        keep = ~self.dirichlet_rows()
        self.rows[2, keep] += other.rows[2, keep]
        self.R = self.R + other.R
        if other.top_status == CAN_FOLD:
            self.top_status = CAN_FOLD
        if other.bot_status == CAN_FOLD:
            self.bot_status = CAN_FOLD

    def to_gpu(self):
        B = BandedOperator()
        B.axis, B.blocks, B.derivative, B.order = self.axis, self.blocks, self.derivative, 2
        if self.mixed is not None:
            coeff, w0, w1, n0, n1 = self.mixed
            B.is_mixed_derivative = True
            B.n0, B.n1 = n0, n1
            B.coeff, B.w0, B.w1 = _dev(coeff), _dev(w0), _dev(w1)
            B.R = _dev(self.R)
            B.has_residual = True
            return B
        B.diags = _dev(self.rows[1:4])
        B.R = _dev(self.R)
        B.has_residual = True
        B._has_low, B._has_high = self.low is not None, self.high is not None
        B.low_dirichlet = _dev(self.low if self.low is not None else np.zeros(self.blocks))
        B.high_dirichlet = _dev(self.high if self.high is not None else np.zeros(self.blocks))
        B.top_factors = _dev(self.rows[0, ::self.L])
        B.bottom_factors = _dev(self.rows[4, self.L - 1::self.L])
        B.top_fold_status, B.bottom_fold_status = self.top_status, self.bot_status
        return B


def _line(x, derivative, lower, upper):
    """One line: centred rows plus applyboundary (BandedOperator.pyx:398-524).
    lower/upper: (type, value) with type None (free), 0 (Dirichlet), 1 (Neumann)."""
    x = np.asarray(x, dtype=float)
    n = x.size
    rows = np.zeros((5, n))
    R = np.zeros(n)
    sub, mid, sup = centre_rows(x, derivative)
    rows[1], rows[2], rows[3] = sup, mid, sub
    d1, d2 = x[1] - x[0], x[2] - x[1]
    dm1, dm2 = x[-1] - x[-2], x[-2] - x[-3]
    lt, lv = lower
    ut, uv = upper
    low = high = None
    if lt == 0:
        rows[2, 0] = 1
        low = lv
    elif lt == 1:
        R[0] = lv
    elif derivative == 1:
        rows[1, 0] = 1 / d1
        rows[2, 0] = -1 / d1
    elif lv is not None:
        xx = d1 * d1
        rows[1, 0] = 2 / xx
        rows[2, 0] = -2 / xx
        R[0] = -lv * 2 / d1
    else:
        rd = 1.0 / (0.5 * (d2 + d1) * d2 * d1)
        rows[0, 0] = d1 * rd
        rows[1, 0] = -(d2 + d1) * rd
        rows[2, 0] = d2 * rd
    if ut == 0:
        rows[2, -1] = 1
        high = uv
    elif ut == 1:
        R[-1] = uv
    elif derivative == 1:
        rows[2, -1] = 1.0 / dm1
        rows[3, -1] = -1.0 / dm1
    elif uv is not None:
        xx = dm1 * dm1
        rows[2, -1] = -2 / xx
        rows[3, -1] = 2 / xx
        R[-1] = (uv * 2) / dm1
    else:
        rd = 1.0 / (0.5 * (dm2 + dm1) * dm2 * dm1)
        rows[4, -1] = dm1 * rd
        rows[3, -1] = -(dm2 + dm1) * rd
        rows[2, -1] = dm2 * rd
    return rows, R, low, high


def coefficient_vector(mesh, f, t, dim):
    """f evaluated on the mesh product with ``dim`` varying fastest
    (FiniteDifferenceEngine.pyx:389-418)."""
    mesh = list(mesh)
    m = mesh.pop(dim)
    mesh.append(m)
    prod = np.array(list(itertools.product(*mesh)), dtype=float)
    args = [prod[:, k] for k in range(prod.shape[1])]
    last = args.pop()
    args.insert(dim, last)
    ret = f(t, *args)
    if np.isscalar(ret):
        ret = np.repeat(float(ret), prod.shape[0])
    return np.asarray(ret, dtype=float)


def make_operators(mesh, coefficients, boundaries, t=0.0):
    """Per-dimension combined operators and the mixed operator, as host ops.

    Returns {dim: HostOp, (0, 1): HostOp} following make_discrete_operators and
    scale_and_combine_operators (FiniteDifferenceEngine.pyx:423-592)."""
    mesh = [np.asarray(m, dtype=float) for m in mesh]
    ndim = len(mesh)
    shape = tuple(m.size for m in mesh)
    size = int(np.prod(shape))
    simple = {}
    for d in coefficients:
        if d == ():
            continue
        d = tuple(d)
        if len(set(d)) > 1:
            continue
        dim = d[0]
        derivative = len(d)
        if d not in boundaries:
            raise ValueError("%s has no boundary specified." % (d,))
        b = boundaries[d]
        x = mesh[dim]
        blocks = size // shape[dim]
        op = HostOp(blocks, shape[dim], dim)
        op.derivative = derivative
        other = [mesh[k] for k in range(ndim) if k != dim]
        lows, highs = [], []
        for bi, a in enumerate(itertools.product(*other)):
            args_lo = list(a)
            args_lo.insert(dim, x[0])
            args_hi = list(a)
            args_hi.insert(dim, x[-1])
            lower = (b[0][0], b[0][1](t, *args_lo))
            upper = (b[1][0], b[1][1](t, *args_hi))
            rows, R, lo, hi = _line(x, derivative, lower, upper)
            sl = slice(bi * x.size, (bi + 1) * x.size)
            op.rows[:, sl] = rows
            op.R[sl] = R
            if b[0][0] == 0:
                lows.append(lo)
            if b[1][0] == 0:
                highs.append(hi)
        if lows:
            op.low = np.array(lows, dtype=float)
        if highs:
            op.high = np.array(highs, dtype=float)
        # offsets chosen by _min_possible_bandwidth (FiniteDifference.pyx:295-351)
        if b[0][0] is None and derivative == 2 and b[0][1](0, 0) is None:
            op.top_status = CAN_FOLD
        if b[1][0] is None and derivative == 2 and b[1][1](0, 0) is None:
            op.bot_status = CAN_FOLD
        simple[d] = op
    mixed = [tuple(d) for d in coefficients if d != () and len(set(tuple(d))) > 1]
    for d in mixed:
        n0, n1 = shape[d[0]], shape[d[1]]
        op = HostOp(n0, n1, 1)
        w0 = np.vstack(centre_rows(mesh[d[0]], 1))
        w1 = np.vstack(centre_rows(mesh[d[1]], 1))
        op.mixed = (np.ones(n0 * n1), w0, w1, n0, n1)
        simple[d] = op
    ops = {}
    for d in sorted(simple):
        op = simple[d]
        dim = op.axis if op.mixed is None else 1
        if d in coefficients:
            op.vectorized_scale(coefficient_vector(mesh, coefficients[d], t, dim))
        if len(set(d)) > 1:
            ops[d] = op
        elif dim not in ops:
            ops[dim] = op
            if () in coefficients:
                op.add_scalar_f32(coefficients[()](t) / float(ndim))
        else:
            ops[dim].add(op)
    return ops
