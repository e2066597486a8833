"""GPU banded operators: a drop-in for FiniteDifference.BandedOperatorGPU.

``BandedOperator`` keeps the reference GPU operator's interface
(FiniteDifference/BandedOperatorGPU.pxd:27-69, .pyx:27-597): ``apply``/``apply_``,
``solve``/``solve_``, ``copy``, ``emigrate``/``immigrate``, ``diagonalize``/
``undiagonalize``, ``fold_top``/``fold_bottom``, ``is_folded``/``is_foldable``,
``enable_residual``, scalar/vector scaling, operator and scalar addition, and
the ``has_low_dirichlet``/``has_high_dirichlet``/``operator_rows``/``shape``
properties with the same fold-status strings. Device arrays are torch CUDA
float64 tensors (the reference's ``SizedArrayPtr``); every computation runs in
libfdadi.so through the C ABI (include/fdadi.h).

A tridiagonal operator holds row-aligned ``sup``/``mid``/``sub`` diagonals in
the reference's block-major "cublas" layout, the residual ``R``, per-line
Dirichlet values and per-line fold slots: while an operator is CAN_FOLD the
slots hold the pentadiagonal corner entries A[0,2] / A[L-1,L-3]; once FOLDED
they hold the fold factors (the reference GPU operator uses the same slots,
BandedOperatorGPU.pyx:329-344).
"""
import ctypes

import numpy as np
import scipy.sparse
import torch

from . import _lib
from ._lib import FOLD_CODES, FOLD_NAMES

FOLDED = "FOLDED"
CAN_FOLD = "CAN_FOLD"
CANNOT_FOLD = "CANNOT_FOLD"


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev(x, device=None):
    device = device or torch.device("cuda", torch.cuda.current_device())
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device=device)


class HostOperator(object):
    """Host copy of an operator with the reference CPU operator's fields
    (FiniteDifference/BandedOperator.pyx:20-72): ``D`` (scipy DIA, offsets in
    descending order), ``R``, ``dirichlet``, ``blocks``, ``axis``, fold statuses
    and factors. Returned by ``BandedOperator.immigrate()``."""

    def __init__(self, D, R, dirichlet, blocks, axis, derivative, order, deltas,
                 is_mixed_derivative, top_fold_status, bottom_fold_status,
                 top_factors=None, bottom_factors=None):
        self.D, self.R = D, R
        self.dirichlet = list(dirichlet)
        self.blocks, self.axis = blocks, axis
        self.derivative, self.order, self.deltas = derivative, order, deltas
        self.is_mixed_derivative = is_mixed_derivative
        self.top_fold_status, self.bottom_fold_status = top_fold_status, bottom_fold_status
        self.top_factors, self.bottom_factors = top_factors, bottom_factors
        self.shape = D.shape


class BandedOperator(object):
    """A discrete derivative operator on the GPU (tridiagonal or mixed)."""

    attrs = ("deltas", "derivative", "is_mixed_derivative", "order", "axis", "blocks",
             "top_fold_status", "bottom_fold_status")

    def __init__(self, other=None, tag=""):
        self.deltas = None
        self.derivative = 1
        self.order = 2
        self.axis = 0
        self.blocks = 1
        self.is_mixed_derivative = False
        self.top_fold_status = CANNOT_FOLD
        self.bottom_fold_status = CANNOT_FOLD
        self.tag = tag
        self._scratch = None
        # tridiagonal storage
        self.diags = None          # [3, N]: sup, mid, sub
        self.R = None
        self.low_dirichlet = None
        self.high_dirichlet = None
        self.top_factors = None
        self.bottom_factors = None
        self._has_low = False
        self._has_high = False
        self.has_residual = True
        # [2, N] second off-diagonals inside the lines (A[r, r+2], A[r, r-2]) of
        # a spliced upwind scheme, or None; the corners stay in the fold slots
        self.band2 = None
        # mixed storage
        self.coeff = None
        self.w0 = None
        self.w1 = None
        self.n0 = self.n1 = 0
        if other is not None:
            self.emigrate(other, tag)

    # -- properties (BandedOperatorGPU.pyx:45-82) --
    @property
    def has_high_dirichlet(self):
        return False if self.is_mixed_derivative else self._has_high

    @has_high_dirichlet.setter
    def has_high_dirichlet(self, val):
        if self.is_mixed_derivative:
            raise NotImplementedError("Mixed derivatives cannot have dirichlet boundaries.")
        self._has_high = bool(val)

    @property
    def has_low_dirichlet(self):
        return False if self.is_mixed_derivative else self._has_low

    @has_low_dirichlet.setter
    def has_low_dirichlet(self, val):
        if self.is_mixed_derivative:
            raise NotImplementedError("Mixed derivatives cannot have dirichlet boundaries.")
        self._has_low = bool(val)

    @property
    def operator_rows(self):
        if self.is_mixed_derivative:
            return self.n0 * self.n1
        return int(self.diags.shape[1])

    @property
    def shape(self):
        return (self.operator_rows, self.operator_rows)

    @property
    def block_len(self):
        return self.operator_rows // self.blocks

    # -- C-ABI views --
    def _tri(self):
        d = self.diags
        b2 = self.band2
        return _lib.Tri(self.operator_rows, self.blocks, self.axis, int(self.has_residual),
                        int(self._has_low), int(self._has_high),
                        FOLD_CODES[self.top_fold_status], FOLD_CODES[self.bottom_fold_status],
                        d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), self.R.data_ptr(),
                        self.low_dirichlet.data_ptr(), self.high_dirichlet.data_ptr(),
                        self.top_factors.data_ptr(), self.bottom_factors.data_ptr(),
                        b2[0].data_ptr() if b2 is not None else None,
                        b2[1].data_ptr() if b2 is not None else None)

    def _mixed(self):
        return _lib.Mixed(self.n0, self.n1, int(self.has_residual), 0, self.coeff.data_ptr(),
                          self.w0.data_ptr(), self.w1.data_ptr(), self.R.data_ptr())

    def _grid_shape(self, V):
        if V.dim() == 1:
            return int(V.shape[0]), 1
        if V.dim() == 2:
            return int(V.shape[0]), int(V.shape[1])
        raise ValueError("Dimension mismatch: only 1-D and 2-D grids are supported")

    def copy_meta_data(self, other, **kwargs):
        for attr in self.attrs:
            setattr(self, attr, kwargs.get(attr, getattr(other, attr)))

    def copy(self):
        B = BandedOperator()
        B.copy_meta_data(self)
        B.has_residual = self.has_residual
        B._has_low, B._has_high = self._has_low, self._has_high
        for name in ("diags", "R", "low_dirichlet", "high_dirichlet", "top_factors",
                     "bottom_factors", "band2", "coeff", "w0", "w1"):
            t = getattr(self, name)
            setattr(B, name, None if t is None else t.clone())
        B.n0, B.n1 = self.n0, self.n1
        return B

    # -- migration (BandedOperatorGPU.pyx:157-372) --
    def emigrate(self, other, tag=""):
        """Become a GPU copy of a host operator with the reference CPU
        operator's fields (D as a scipy DIA matrix, R, dirichlet, blocks...)."""
        self.copy_meta_data(other)
        self.tag = tag
        if other.is_mixed_derivative:
            return self._emigrate_mixed(other)
        return self._emigrate_tri(other)

    def _emigrate_tri(self, other):
        D = scipy.sparse.dia_matrix(other.D)
        N = D.shape[0]
        blocks = int(other.blocks)
        L = N // blocks
        rows = np.zeros((5, N))
        for k, o in enumerate(D.offsets):
            o = int(o)
            if abs(o) > 2:
                raise ValueError("Operator is not banded within +-2: offset %d" % o)
            data = D.data[k]
            i = np.arange(max(0, -o), min(N, N - o))
            rows[2 - o, i] = data[i + o]
        top = other.top_fold_status
        bot = other.bottom_fold_status
        tops = np.zeros(blocks)
        bots = np.zeros(blocks)
        if top == FOLDED:
            tops = np.atleast_1d(np.asarray(other.top_factors, dtype=float))
        elif np.any(rows[0]):
            tops = rows[0, ::L].copy()
            top = CAN_FOLD
        if bot == FOLDED:
            bots = np.atleast_1d(np.asarray(other.bottom_factors, dtype=float))
        elif np.any(rows[4]):
            bots = rows[4, L - 1::L].copy()
            bot = CAN_FOLD
        self.top_fold_status, self.bottom_fold_status = top, bot
        # second off-diagonals inside the lines (a spliced upwind scheme)
        inner2 = rows[[0, 4]].copy()
        inner2[0, ::L] = 0.0
        inner2[1, L - 1::L] = 0.0
        self.band2 = _dev(inner2) if np.any(inner2) and not (top == FOLDED or bot == FOLDED) \
            else None
        self.diags = _dev(rows[1:4])
        R = other.R if other.R is not None else np.zeros(N)
        self.has_residual = other.R is not None
        self.R = _dev(R)
        low, high = other.dirichlet[0], other.dirichlet[1]
        self._has_low, self._has_high = low is not None, high is not None
        self.low_dirichlet = _dev(np.broadcast_to(np.atleast_1d(low if low is not None else 0.0),
                                                  (blocks,)).astype(float))
        self.high_dirichlet = _dev(np.broadcast_to(
            np.atleast_1d(high if high is not None else 0.0), (blocks,)).astype(float))
        self.top_factors = _dev(tops)
        self.bottom_factors = _dev(bots)
        self.blocks = blocks
        return self

    def _emigrate_mixed(self, other):
        """A host mixed operator must carry its factored form (``coeff``,
        ``w0``, ``w1``, ``n0``, ``n1``), as ``immigrate`` returns it."""
        for name in ("coeff", "w0", "w1"):
            if not hasattr(other, name):
                raise ValueError("mixed operator must provide the factored stencil (%s)" % name)
        self.is_mixed_derivative = True
        self.n0, self.n1 = int(other.n0), int(other.n1)
        self.coeff = _dev(other.coeff)
        self.w0 = _dev(other.w0).reshape(3, self.n0)
        self.w1 = _dev(other.w1).reshape(3, self.n1)
        R = other.R if other.R is not None else np.zeros(self.n0 * self.n1)
        self.R = _dev(R)
        return self

    def immigrate(self, tag=""):
        """Host copy with the reference CPU operator's fields."""
        if self.is_mixed_derivative:
            return self._immigrate_mixed()
        d = self.diags.cpu().numpy()
        N, L = self.operator_rows, self.block_len
        top = self.top_factors.cpu().numpy()
        bot = self.bottom_factors.cpu().numpy()
        offsets = [1, 0, -1]
        data = [d[0], d[1], d[2]]
        b2 = self.band2.cpu().numpy() if self.band2 is not None else None
        if self.top_fold_status == CAN_FOLD or b2 is not None:
            r = np.zeros(N) if b2 is None else b2[0].copy()
            if self.top_fold_status == CAN_FOLD:
                r[::L] = top
            offsets.insert(0, 2)
            data.insert(0, r)
        if self.bottom_fold_status == CAN_FOLD or b2 is not None:
            r = np.zeros(N) if b2 is None else b2[1].copy()
            if self.bottom_fold_status == CAN_FOLD:
                r[L - 1::L] = bot
            offsets.append(-2)
            data.append(r)
        dia = np.zeros((len(offsets), N))
        for k, (o, row) in enumerate(zip(offsets, data)):
            i = np.arange(max(0, -o), min(N, N - o))
            dia[k, i + o] = row[i]
        D = scipy.sparse.dia_matrix((dia, np.array(offsets)), shape=(N, N))
        low = tuple(self.low_dirichlet.cpu().numpy()) if self._has_low else None
        high = tuple(self.high_dirichlet.cpu().numpy()) if self._has_high else None
        R = self.R.cpu().numpy() if self.has_residual else np.zeros(N)
        return HostOperator(D, R, [low, high], self.blocks, self.axis, self.derivative,
                            self.order, self.deltas, False, self.top_fold_status,
                            self.bottom_fold_status,
                            top if self.top_fold_status == FOLDED else None,
                            bot if self.bottom_fold_status == FOLDED else None)

    def _immigrate_mixed(self):
        n0, n1 = self.n0, self.n1
        w0 = self.w0.cpu().numpy()
        w1 = self.w1.cpu().numpy()
        c = self.coeff.cpu().numpy()
        N = n0 * n1
        rows, cols, vals = [], [], []
        for a in (-1, 0, 1):
            for b in (-1, 0, 1):
                i, j = np.meshgrid(np.arange(1, n0 - 1), np.arange(1, n1 - 1), indexing="ij")
                val = w1[b + 1][j] * w0[a + 1][i] * c[i * n1 + j]
                rows.append((i * n1 + j).ravel())
                cols.append(((i + a) * n1 + (j + b)).ravel())
                vals.append(val.ravel())
        M = scipy.sparse.coo_matrix((np.concatenate(vals),
                                     (np.concatenate(rows), np.concatenate(cols))),
                                    shape=(N, N)).todia()
        H = HostOperator(M, self.R.cpu().numpy(), [None, None], self.blocks, self.axis,
                         self.derivative, self.order, self.deltas, True, self.top_fold_status,
                         self.bottom_fold_status)
        H.coeff, H.w0, H.w1, H.n0, H.n1 = c, w0, w1, n0, n1
        return H

    # -- fold (BandedOperatorGPU.pyx:375-401, 476-485) --
    def diagonalize(self):
        if self.is_mixed_derivative:
            raise RuntimeError("Diagonalize called on a mixed operator.")
        self._fold(self.top_fold_status == CAN_FOLD, self.bottom_fold_status == CAN_FOLD, 0)

    def undiagonalize(self):
        if self.is_mixed_derivative:
            raise RuntimeError("Undiagonalize called on a mixed operator.")
        self._fold(self.top_fold_status == FOLDED, self.bottom_fold_status == FOLDED, 1)

    def fold_top(self, unfold=False):
        self._no_mixed()
        self._fold(True, False, int(bool(unfold)))

    def fold_bottom(self, unfold=False):
        self._no_mixed()
        self._fold(False, True, int(bool(unfold)))

    def _fold(self, top, bottom, unfold):
        t = self._tri()
        _lib.call("fdadi_tri_fold", ctypes.byref(t), int(top), int(bottom), unfold, _stream())
        self.top_fold_status = FOLD_NAMES[t.top_fold_status]
        self.bottom_fold_status = FOLD_NAMES[t.bottom_fold_status]
        # a folded operator is tridiagonal: the second off-diagonals inside the
        # lines are dropped, as the reference's diagonalize drops them
        # (BandedOperator.pyx:195-198)
        if self.is_folded():
            self.band2 = None

    def is_folded(self):
        return self.top_fold_status == FOLDED or self.bottom_fold_status == FOLDED

    def is_foldable(self):
        return self.top_fold_status == CAN_FOLD or self.bottom_fold_status == CAN_FOLD

    def _no_mixed(self):
        if self.is_mixed_derivative:
            raise ValueError("Operation not supported with mixed operator.")

    # -- apply / solve (BandedOperatorGPU.pyx:404-460) --
    def apply_(self, V, overwrite=False):
        U = V if overwrite else V.clone()
        if self.is_mixed_derivative:
            src = U.clone()
            m = self._mixed()
            _lib.call("fdadi_mixed_apply", ctypes.byref(m), _ptr(src), _ptr(U), _stream())
        else:
            n0, n1 = self._grid_shape(U)
            t = self._tri()
            _lib.call("fdadi_tri_apply", ctypes.byref(t), _ptr(U), _ptr(U), n0, n1, _stream())
        return U

    def apply(self, V, overwrite=False):
        """Wrapper for host (numpy) data."""
        return self.apply_(_dev(V), overwrite=True).cpu().numpy()

    def solve_(self, V, overwrite=False):
        if self.is_mixed_derivative:
            raise NotImplementedError("The mixed operator has no solve (the reference's "
                                      "csrsv solve is marked untrustworthy and unused).")
        U = V if overwrite else V.clone()
        n0, n1 = self._grid_shape(U)
        need = self.operator_rows * (3 if self.band2 is not None else 1)
        if self._scratch is None or self._scratch.numel() != need:
            self._scratch = torch.empty(need, dtype=torch.float64, device=U.device)
        t = self._tri()
        _lib.call("fdadi_tri_solve", ctypes.byref(t), _ptr(U), n0, n1, _ptr(self._scratch),
                  _stream())
        return U

    def solve(self, V, overwrite=False):
        return self.solve_(_dev(V), overwrite=True).cpu().numpy()

    def enable_residual(self, state):
        self.has_residual = bool(state)

    # -- algebra (BandedOperatorGPU.pyx:488-596) --
    def vectorized_scale(self, vector):
        vec = _dev(vector)
        if vec.numel() != self.operator_rows:
            if vec.numel() == self.block_len and not self.is_mixed_derivative:
                vec = vec.repeat(self.blocks)
            else:
                raise ValueError("Dimension mismatch: vector of %d for %d rows"
                                 % (vec.numel(), self.operator_rows))
        self._scale(vec, 0.0)

    def vectorized_scale_from_host(self, vector):
        self.vectorized_scale(vector)

    def _scale(self, vec, scalar):
        if self.is_mixed_derivative:
            m = self._mixed()
            _lib.call("fdadi_mixed_scale", ctypes.byref(m), _ptr(vec), float(scalar), _stream())
        else:
            t = self._tri()
            _lib.call("fdadi_tri_scale", ctypes.byref(t), _ptr(vec), float(scalar), _stream())

    def mul_scalar_from_host(self, v, inplace=False):
        B = self if inplace else self.copy()
        B._scale(None, float(v))
        return B

    def __mul__(self, val):
        B = self.copy()
        B.__imul__(val)
        return B

    def __imul__(self, val):
        if isinstance(val, torch.Tensor) and val.numel() == 1:
            val = float(val.item())
        if isinstance(val, torch.Tensor) or isinstance(val, np.ndarray):
            self.vectorized_scale(val)
        else:
            self._scale(None, float(val))
        return self

    def add(self, val, inplace=False):
        if inplace:
            self += val
            return self
        return self + val

    def __add__(self, val):
        B = self.copy()
        if isinstance(val, BandedOperator):
            B.add_operator(val)
        else:
            B.add_scalar_from_host(val)
        return B

    def __iadd__(self, val):
        if isinstance(val, BandedOperator):
            self.add_operator(val)
        else:
            self.add_scalar_from_host(val)
        return self

    def add_operator(self, other):
        if self.is_mixed_derivative:
            raise NotImplementedError("No add to mixed operator")
        if other.is_mixed_derivative:
            raise NotImplementedError("No add mixed operator to this one")
        if self.axis != other.axis:
            raise ValueError("Both operators must operate on the same axis. (%s != %s)"
                             % (self.axis, other.axis))
        if self.operator_rows != other.operator_rows:
            raise ValueError("Both operators must have the same length")
        if self.is_folded():
            raise NotImplementedError("No add to diagonalized operator.")
        if other.is_folded():
            raise NotImplementedError("No add diagonalized operator.")
        if other.band2 is not None and self.band2 is None:
            self.band2 = torch.zeros_like(other.band2)
        a, b = self._tri(), other._tri()
        _lib.call("fdadi_tri_add_operator", ctypes.byref(a), ctypes.byref(b), _stream())
        self.top_fold_status = FOLD_NAMES[a.top_fold_status]
        self.bottom_fold_status = FOLD_NAMES[a.bottom_fold_status]

    def add_scalar_from_host(self, other):
        """Add a scalar to the main diagonal (not the Dirichlet rows). The
        reference declares this argument as a C float
        (BandedOperatorGPU.pyx:556; BandedOperator.pxd:32 for the CPU engine),
        so the value is rounded to binary32 first."""
        if self.is_mixed_derivative:
            raise RuntimeError("add_scalar called on a mixed operator.")
        t = self._tri()
        _lib.call("fdadi_tri_add_scalar", ctypes.byref(t), float(np.float32(other)), _stream())

    def add_scalar(self, other, index=0):
        """Add element ``index`` of a device array (full double precision, as
        the reference's device-pointer overload, _TriBandedOperatorGPU.cu:697-711)."""
        if self.is_mixed_derivative:
            raise RuntimeError("add_scalar called on a mixed operator.")
        val = float(other.reshape(-1)[index].item()) if isinstance(other, torch.Tensor) \
            else float(np.asarray(other).reshape(-1)[index])
        t = self._tri()
        _lib.call("fdadi_tri_add_scalar", ctypes.byref(t), val, _stream())


# ---------------------------------------------------------------------------
# Operator construction (host, once per engine)
# ---------------------------------------------------------------------------

def centre_rows(x, derivative):
    """Centred non-uniform 3-point stencil: (sub, mid, sup) rows of length n,
    zero on rows 0 and n-1 (centercoeffs, BandedOperator.pyx:970-1017)."""
    x = np.asarray(x, dtype=float)
    n = x.size
    sub, mid, sup = np.zeros(n), np.zeros(n), np.zeros(n)
    di = x[1:-1] - x[:-2]
    dn = x[2:] - x[1:-1]
    s = di + dn
    if derivative == 1:
        sup[1:-1] = di / (dn * s)
        mid[1:-1] = (-di + dn) / (di * dn)
        sub[1:-1] = -dn / (di * s)
    else:
        sup[1:-1] = 2 / (dn * s)
        mid[1:-1] = -2 / (di * dn)
        sub[1:-1] = 2 / (di * s)
    return sub, mid, sup


def heston_line(v, derivative, axis, barrier):
    """One line of the Heston operator the GPU reference builds in for_vector
    (_TriBandedOperatorGPU.cu:203-362, 1107-1182): (sub, mid, sup, R, extra,
    low_dirichlet, high_dirichlet, bottom CAN_FOLD)."""
    x = np.asarray(v, dtype=float)
    n = x.size
    sub, mid, sup = centre_rows(x, derivative)
    R = np.zeros(n)
    extra = 0.0
    d1, d2 = x[1] - x[0], x[2] - x[1]
    dm1, dm2 = x[-1] - x[-2], x[-2] - x[-3]
    low = high = False
    if axis == 0:
        # spot: Dirichlet U = 0 at S = 0
        sub[0], mid[0], sup[0] = 0.0, 1.0, 0.0
        low = True
        if barrier:
            sub[-1], mid[-1], sup[-1] = 0.0, 1.0, 0.0
            high = True
        elif derivative == 1:
            # dU/dS = 1 at S_max (von Neumann)
            sub[-1] = mid[-1] = sup[-1] = 0.0
            R[-1] = 1.0
        else:
            # second derivative with the first derivative fixed at 1
            xx = dm1 * dm1
            mid[-1] = -2 / xx
            sub[-1] = 2 / xx
            sup[-1] = 0.0
            R[-1] = (1.0 * 2) / dm1
    else:
        if derivative == 1:
            # one-sided first order at both ends
            sup[0], mid[0] = 1 / d1, -1 / d1
            mid[-1], sub[-1] = 1.0 / dm1, -1.0 / dm1
        else:
            # Neumann 0 at v = 0; second-order backward at v_max (offset -2)
            sub[0] = mid[0] = sup[0] = 0.0
            rd = 1.0 / (0.5 * (dm2 + dm1) * dm2 * dm1)
            extra = dm1 * rd
            sub[-1] = -(dm2 + dm1) * rd
            mid[-1] = dm2 * rd
            sup[-1] = 0.0
    return sub, mid, sup, R, extra, low, high


def upwind_rows(x, scheme, at):
    """Rows ``at`` and beyond of a first-derivative operator whose scheme
    switches there (the rows splice_with takes from the second scheme,
    BandedOperator.pyx:527-591): 'forward' (forwardcoeffs, BandedOperator.pyx:
    917-967: rows 1..n-3 use points i, i+1, i+2, row n-2 the centred
    stencil) or 'backward' (backwardcoeffs, :1020-1067: rows 2..n-2 use
    points i-2, i-1, i, row 1 the centred stencil). Returns (sup2, sup, mid,
    sub, sub2), length n each, zero outside the rows that scheme fills."""
    x = np.asarray(x, dtype=float)
    n = x.size
    e2, e1, e0, f1, f2 = (np.zeros(n) for _ in range(5))
    if scheme == "forward":
        for i in range(max(at, 1), n - 2):
            d1, d2 = x[i + 1] - x[i], x[i + 2] - x[i + 1]
            e1[i] = (d1 + d2) / (d1 * d2)
            e2[i] = -d1 / (d2 * (d1 + d2))
            e0[i] = (-2 * d1 - d2) / (d1 * (d1 + d2))
        if n - 2 >= at:
            dl, dm = x[n - 1] - x[n - 2], x[n - 2] - x[n - 3]
            e1[n - 2] = dm / (dl * (dm + dl))
            e0[n - 2] = (-dm + dl) / (dm * dl)
            f1[n - 2] = -dl / (dm * (dm + dl))
    elif scheme == "backward":
        for i in range(max(at, 2), n - 1):
            dp, di = x[i - 1] - x[i - 2], x[i] - x[i - 1]
            e0[i] = (dp + 2 * di) / (di * (dp + di))
            f1[i] = (-dp - di) / (dp * di)
            f2[i] = di / (dp * (dp + di))
        if at <= 1:
            d1, d2 = x[1] - x[0], x[2] - x[1]
            xx = d1 + d2
            e1[1] = d1 / (d2 * xx)
            e0[1] = (-d1 + d2) / (d1 * d2)
            f1[1] = -d2 / (d1 * xx)
    else:
        raise ValueError("Unknown scheme: %s" % scheme)
    return e2, e1, e0, f1, f2


def for_vector(v, blocks, derivative, axis, barrier=False, scheme=None, at=None):
    """Heston derivative operator along ``axis`` replicated over ``blocks``
    lines, as FiniteDifference.BandedOperatorGPU.for_vector builds it
    (BandedOperatorGPU.pyx:599-618): spot operators (axis 0) carry the
    Dirichlet row at S = 0 and a residual; the variance second derivative is
    CAN_FOLD at v_max.

    scheme, at: a first derivative whose rows from ``at`` on use 'forward' or
    'backward' differences (the up/down-winding schemes HestonFiniteDifference-
    Engine splices in, heston.py:414-439, FiniteDifferenceEngine.pyx:267-289).
    The operator then has a second off-diagonal inside its lines and can fold
    at that end, as the reference's spliced operator does."""
    sub, mid, sup, R, extra, low, high = heston_line(v, derivative, axis, barrier)
    band2 = None
    if scheme is not None:
        n = np.asarray(v).size
        if derivative != 1:
            raise NotImplementedError("only first derivatives switch schemes")
        if not 0 <= int(at) < n - 1:
            raise ValueError("Cannot splice beyond the end of the vector. %i >= %i"
                             % (int(at), n - 1))
        e2, e1, e0, f1, f2 = upwind_rows(v, scheme, int(at))
        # rows at.. come from the upwind scheme; the boundary rows stay
        rows = np.arange(n)
        take = (rows >= int(at)) & (rows >= 1) & (rows <= n - 2)
        sup = np.where(take, e1, sup)
        mid = np.where(take, e0, mid)
        sub = np.where(take, f1, sub)
        band2 = np.vstack([np.where(take, e2, 0.0), np.where(take, f2, 0.0)])
        band2[0, 0] = 0.0
        band2[1, n - 1] = 0.0
    B = BandedOperator()
    B.axis, B.blocks, B.derivative, B.order = int(axis), int(blocks), int(derivative), 2
    B.deltas = None
    B.diags = _dev(np.vstack([np.tile(sup, blocks), np.tile(mid, blocks), np.tile(sub, blocks)]))
    if band2 is not None:
        B.band2 = _dev(np.tile(band2, (1, blocks)))
    B.R = _dev(np.tile(R, blocks))
    B.has_residual = axis == 0
    B._has_low, B._has_high = low, high
    B.low_dirichlet = _dev(np.zeros(blocks))
    B.high_dirichlet = _dev(np.zeros(blocks))
    B.top_factors = _dev(np.zeros(blocks))
    B.bottom_factors = _dev(np.full(blocks, extra))
    B.top_fold_status = CAN_FOLD if scheme == "forward" else CANNOT_FOLD
    B.bottom_fold_status = CAN_FOLD if ((axis == 1 and derivative == 2) or scheme == "backward") \
        else CANNOT_FOLD
    return B


def mixed_for_vector(v0, v1):
    """d2/dv0dv1 operator (BandedOperatorGPU.pyx:621-641): centred first
    derivatives in both directions, zero on all four edges; coefficient 1."""
    v0 = np.asarray(v0, dtype=float)
    v1 = np.asarray(v1, dtype=float)
    B = BandedOperator()
    B.is_mixed_derivative = True
    B.derivative, B.axis, B.order, B.deltas = 1, 1, 2, None
    B.blocks = v0.size
    B.n0, B.n1 = v0.size, v1.size
    B.w0 = _dev(np.vstack(centre_rows(v0, 1)))
    B.w1 = _dev(np.vstack(centre_rows(v1, 1)))
    B.coeff = _dev(np.ones(v0.size * v1.size))
    B.R = _dev(np.zeros(v0.size * v1.size))
    B.has_residual = True
    return B
