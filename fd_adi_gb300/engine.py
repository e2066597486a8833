"""ADI engines: drop-ins for FiniteDifference.FiniteDifferenceEngineGPU.

* ``FiniteDifferenceEngineADI`` mirrors FiniteDifferenceEngineGPU.pyx:40-593:
  operators as GPU ``BandedOperator``s, ``preprocess_operators``,
  ``scale_and_combine_operators``, ``set_zero_derivative`` and the
  ``solve_implicit``/``solve_douglas``/``solve_hundsdorferverwer``/
  ``solve_smooth`` host wrappers with their ``*_`` device versions. Its time
  loops issue one operator call at a time, the reference's per-step call
  sequence -- the unfused ("plain") GPU path.
* ``HestonFiniteDifferenceEngine`` mirrors FiniteDifferenceEngineGPU.pyx:596-757
  (meshes, payoff grid, hard-coded Heston operators, ``idx``/``price``). Its
  ``solve_*`` wrappers run the fused batched engine (``HestonBatch``) by
  default; ``fused=False`` selects the per-operator path.
* ``BlackScholesFiniteDifferenceEngine`` mirrors blackscholes.py:144-239. Its
  ``solve_*`` wrappers run the fused batched engine (``BlackScholesBatch``) by
  default.

Semantics follow the reference CPU engine (the oracle): the zero-derivative
term -r/ndim is rounded to binary32 (BandedOperator.pxd:32 declares
add_scalar's argument a C float) and the implicit steps keep the boundary
residual (FiniteDifferenceEngine.pyx:631-635). The reference GPU engine
differs in both (double -r/ndim, residual disabled in its implicit steps,
FiniteDifferenceEngineGPU.pyx:187-188); set ``zero_derivative_f32=False``
and ``implicit_residual=False`` to reproduce it instead.
"""
import numpy as np
import torch

from . import _lib
from .banded_operator import BandedOperator, _dev, for_vector, mixed_for_vector
from .construct import make_operators
from . import mesh as _mesh
from .option import BarrierOption, Grid, Option


def _apply_into(L, X, src):
    X.copy_(src)
    L.apply_(X, overwrite=True)


def _axpby(y, x, a, b):
    _lib.call("fdadi_axpby", _ptr(y), _ptr(x), float(a), float(b), y.numel(),
              _stream_ptr())


def _ptr(t):
    import ctypes
    return ctypes.c_void_p(t.data_ptr())


def _stream_ptr():
    import ctypes
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class FiniteDifferenceEngine(object):
    """Base engine (FiniteDifferenceEngineGPU.pyx:40-128)."""

    def __init__(self):
        self.simple_operators = {}
        self.operators = {}
        self.t = 0
        self.n = 0
        self.barrier = 0
        self.default_scheme = "center"
        self.default_order = 2
        self.coefficients = {}
        self.boundaries = {}
        self.grid = None
        self.option = None
        self.zero_derivative_coefficient_host = None
        self.zero_derivative_f32 = True
        self.implicit_residual = True
        self.gpugrid = None
        # time-dependent coefficients: the interest rate of every step of the
        # next solve (the implicit steps of solve_smooth first), or None
        self.rates = None
        self._rate = None
        self._rate_step = 0

    @property
    def shape(self):
        return self.grid.shape

    @property
    def ndim(self):
        return self.grid.ndim

    def from_host_FiniteDifferenceEngine(self, other):
        """Move an engine whose operators are host operators (reference CPU
        BandedOperator fields) onto the GPU (FiniteDifferenceEngineGPU.pyx:100-128)."""
        if hasattr(other, "init"):
            other.init()
        self.option = getattr(other, "option", None)
        self.grid = other.grid.copy()
        self.gpugrid = _dev(self.grid.domain[-1])
        self.coefficients = other.coefficients
        ops = dict(other.operators)
        simple = dict(getattr(other, "simple_operators", {}))
        try:
            if self.option is not None and self.option.correlation == 0:
                ops.pop((0, 1), None)
                simple.pop((0, 1), None)
        except AttributeError:
            pass
        self.operators = {k: BandedOperator(v) for k, v in ops.items()}
        self.simple_operators = {k: BandedOperator(v) for k, v in simple.items()
                                 if not getattr(v, "is_mixed_derivative", False)
                                 or hasattr(v, "coeff")}
        return self


class FiniteDifferenceEngineADI(FiniteDifferenceEngine):
    """GPU ADI engine on per-operator kernels.

    With ``grid``, ``coefficients`` and ``boundaries`` (the reference CPU
    engine's dicts, FiniteDifferenceEngine.pyx:72-152) the operators are built
    once on the host and moved to the GPU."""

    def __init__(self, grid=None, coefficients=None, boundaries=None, schemes=None,
                 force_bandwidth=None):
        FiniteDifferenceEngine.__init__(self)
        if grid is not None:
            self.grid = grid
            self.gpugrid = _dev(grid.domain[-1])
            self.coefficients = coefficients or {}
            self.boundaries = boundaries or {}
            if coefficients:
                host = make_operators(grid.mesh, coefficients, boundaries or {}, self.t)
                self.operators = {k: v.to_gpu() for k, v in host.items()}

    def init(self):
        return

    # -- operator preparation (FiniteDifferenceEngineGPU.pyx:163-361) --
    def set_zero_derivative(self):
        if self.zero_derivative_coefficient_host is None:
            if isinstance(self.coefficients, dict) and () in self.coefficients:
                val = self.coefficients[()](self.t) / float(self.grid.ndim)
            elif self.option is not None:
                val = -self.option.interest_rate.value / self.grid.ndim
            else:
                raise RuntimeError("Zero derivative coefficient has not been set.")
            self.zero_derivative_coefficient_host = np.atleast_1d(val)
        return self.zero_derivative_coefficient_host

    def _add_zero_derivative(self, op):
        val = float(np.asarray(self.set_zero_derivative()).reshape(-1)[0])
        if self.zero_derivative_f32:
            op.add_scalar_from_host(val)
        else:
            op.add_scalar(np.atleast_1d(val), 0)

    def scale_and_combine_operators(self, operators=None):
        """Scale each single-derivative operator by its PDE coefficient and
        sum them per dimension (FiniteDifferenceEngineGPU.pyx:193-280)."""
        if operators is None:
            if hasattr(self, "make_operator_templates"):
                self.make_operator_templates()
            operators = self.simple_operators
        if not operators:
            return
        self.operators = {}
        for d, op in sorted(operators.items()):
            op = op.copy()
            dim = op.axis
            vec = self.coefficient_vector(d, dim)
            if vec is not None:
                op.vectorized_scale(vec)
            if len(set(d)) > 1:
                self.operators[d] = op
            elif dim not in self.operators:
                self.operators[dim] = op
                self._add_zero_derivative(op)
            else:
                self.operators[dim] += op

    def coefficient_vector(self, d, dim):
        if isinstance(self.coefficients, dict) and d in self.coefficients:
            from .construct import coefficient_vector
            return coefficient_vector(self.grid.mesh, self.coefficients[d], self.t, dim)
        return None

    def preprocess_operators(self, dt, theta):
        """Firsts = dt*A, Les = theta*dt*A, Lis = 1 - theta*dt*A with the
        residual disabled on Les and Lis (FiniteDifferenceEngineGPU.pyx:163-190)."""
        dt = float(np.asarray(dt).reshape(-1)[0]) if not np.isscalar(dt) else float(dt)
        theta = float(np.asarray(theta).reshape(-1)[0]) if not np.isscalar(theta) else float(theta)
        if not self.operators:
            self.scale_and_combine_operators()
        Firsts = [o.mul_scalar_from_host(dt) for d, o in self.operators.items()]
        dims = [(d, o) for d, o in sorted(self.operators.items(), key=lambda kv: str(kv[0]))
                if not isinstance(d, tuple)]
        Les = [o.mul_scalar_from_host(theta).mul_scalar_from_host(dt, inplace=True)
               for d, o in dims]
        Lis = [o.mul_scalar_from_host(theta * -dt).add(1, inplace=True) for d, o in dims]
        for L in Les + Lis:
            L.enable_residual(False)
        return Firsts, Les, Lis

    def _dims(self):
        return [(d, o) for d, o in sorted(self.operators.items(), key=lambda kv: str(kv[0]))
                if not isinstance(d, tuple)]

    def _next_rate(self):
        """With per-step rates (self.rates): take the next step's rate and
        rebuild the combined operators for it, as preprocess_operators is
        meant to run per step for time-dependent parameters
        (FiniteDifferenceEngineGPU.pyx:163-167). Returns True if it did."""
        if self.rates is None:
            return False
        rates = np.asarray(self.rates, dtype=np.float64).reshape(-1)
        if self._rate_step >= rates.size:
            raise ValueError("rates holds %d steps; the solve needs more" % rates.size)
        self._rate = float(rates[self._rate_step])
        self._rate_step += 1
        self.zero_derivative_coefficient_host = np.atleast_1d(-self._rate / self.grid.ndim)
        self.operators = {}
        self.scale_and_combine_operators()
        return True

    def _start_rates(self):
        """Start of a solve: step 0 of self.rates. Operators left at the last
        step's rate by an earlier time-dependent solve are dropped."""
        self._rate_step = 0
        if self._rate is not None:
            self._rate = None
            self.operators = {}
            self.zero_derivative_coefficient_host = None

    def _split_ops(self, dt, theta):
        """Firsts, Les, Lis for one (dt, theta), folded where foldable."""
        Firsts = [o.mul_scalar_from_host(dt) for d, o in self.operators.items()]
        dims = self._dims()
        Les = [o.mul_scalar_from_host(theta).mul_scalar_from_host(dt, inplace=True)
               for d, o in dims]
        Lis = [o.mul_scalar_from_host(theta * -dt).add(1, inplace=True) for d, o in dims]
        for L in Les + Lis:
            L.enable_residual(False)
        for L in Les + Lis + Firsts:
            if L.is_foldable():
                L.diagonalize()
        return Firsts, Les, Lis

    # -- host wrappers --
    def _initial(self, initial):
        if initial is not None:
            return _dev(initial)
        return _dev(self.grid.domain[-1])

    def solve_implicit(self, n, dt, initial=None, callback=None, numpy=False):
        if callback or numpy:
            raise NotImplementedError("Callbacks and Numpy not available for GPU solver.")
        V = self._initial(initial)
        self._start_rates()
        self.solve_implicit_(int(n), dt, V)
        return V.cpu().numpy()

    def solve_douglas(self, n, dt, initial=None, theta=0.5, callback=None, numpy=False):
        if callback or numpy:
            raise NotImplementedError("Callbacks and Numpy not available for GPU solver.")
        V = self._initial(initial)
        self._start_rates()
        self.solve_douglas_(int(n), dt, V, theta)
        return V.cpu().numpy()

    def solve_hundsdorferverwer(self, n, dt, initial=None, theta=0.5, callback=None, numpy=False):
        if callback or numpy:
            raise NotImplementedError("Callbacks and Numpy not available for GPU solver.")
        V = self._initial(initial)
        self._start_rates()
        self.solve_hundsdorferverwer_(int(n), dt, V, theta)
        return V.cpu().numpy()

    def solve_smooth(self, n, dt, initial=None, callback=None, smoothing_steps=2, scheme=None):
        if scheme:
            raise NotImplementedError("Changing smoothing schemes not supported on GPU.")
        V = self._initial(initial)
        self._start_rates()
        self.solve_smooth_(int(n), dt, V, smoothing_steps)
        return V.cpu().numpy()

    # -- device loops: the reference's per-step call sequence --
    def solve_implicit_(self, n, dt, V, callback=None, numpy=False):
        """Fully implicit steps (FiniteDifference.pyx:617-659): an explicit
        mixed step, then the per-dimension solves in the order 1, 0."""
        if callback or numpy:
            raise NotImplementedError("Callbacks and Numpy not available for GPU solver.")
        dt = float(dt)
        if not self.operators:
            self.scale_and_combine_operators()

        def prep():
            Lis = [o.mul_scalar_from_host(-dt).add(1, inplace=True) for d, o in self._dims()]
            for L in Lis:
                L.enable_residual(self.implicit_residual and True)
            Lis = Lis[1:] + Lis[:1]
            cross = self.operators.get((0, 1))
            cross = cross.mul_scalar_from_host(dt) if cross is not None else None
            for L in Lis:
                # folding the corner rows is the same system; an operator with
                # second off-diagonals inside its lines (a switched scheme) is
                # solved as a band, as the reference solves every implicit line
                if L.is_foldable() and L.band2 is None:
                    L.diagonalize()
            return Lis, cross

        timedep = self.rates is not None
        if not timedep:
            Lis, cross = prep()
        U = torch.empty_like(V)
        for _ in range(int(n)):
            if timedep and self._next_rate():
                Lis, cross = prep()
            if cross is not None:
                _apply_into(cross, U, V)
                _axpby(V, U, 1.0, 1.0)
            for L in Lis:
                L.solve_(V, overwrite=True)
        return V

    def solve_douglas_(self, n, dt, V, theta=0.5):
        """Douglas (FiniteDifferenceEngineGPU.pyx:435-481)."""
        dt, theta = float(dt), float(theta)
        if not self.operators:
            self.scale_and_combine_operators()
        timedep = self.rates is not None
        if not timedep:
            Firsts, Les, Lis = self._split_ops(dt, theta)
        Y = V.clone()
        X = torch.empty_like(V)
        for _ in range(int(n)):
            if timedep and self._next_rate():
                Firsts, Les, Lis = self._split_ops(dt, theta)
            for L in Firsts:
                _apply_into(L, X, Y)
                _axpby(V, X, 1.0, 1.0)
            for Le, Li in zip(Les, Lis):
                _apply_into(Le, X, Y)
                _axpby(V, X, 1.0, -1.0)
                Li.solve_(V, overwrite=True)
            Y.copy_(V)
        return V

    def solve_hundsdorferverwer_(self, n, dt, V, theta=0.5):
        """Hundsdorfer-Verwer (FiniteDifferenceEngineGPU.pyx:502-562)."""
        dt, theta = float(dt), float(theta)
        if not self.operators:
            self.scale_and_combine_operators()
        timedep = self.rates is not None
        if not timedep:
            Firsts, Les, Lis = self._split_ops(dt, theta)
        X = torch.empty_like(V)
        Y = torch.empty_like(V)
        Z = torch.empty_like(V)
        for _ in range(int(n)):
            if timedep and self._next_rate():
                Firsts, Les, Lis = self._split_ops(dt, theta)
            Y.copy_(V)
            for L in Firsts:
                _apply_into(L, X, Y)
                _axpby(V, X, 1.0, 1.0)
            Z.copy_(V)
            for Le, Li in zip(Les, Lis):
                _apply_into(Le, X, Y)
                _axpby(Z, X, 1.0, -1.0)
                Li.solve_(Z, overwrite=True)
            _axpby(Y, Z, 0.5, -0.5)      # Y = (Y - Z) / 2
            for L in Firsts:
                keep = L.has_residual
                L.enable_residual(False)
                _apply_into(L, X, Y)
                _axpby(V, X, 1.0, -1.0)
                L.enable_residual(keep)
            for Le, Li in zip(Les, Lis):
                _apply_into(Le, X, Z)
                _axpby(V, X, 1.0, -1.0)
                Li.solve_(V, overwrite=True)
        return V

    def solve_craigsneyd_(self, n, dt, V, theta=0.5, modified=False):
        """Craig-Sneyd (FiniteDifference.pyx:843-898) or, with modified, the
        modified Craig-Sneyd scheme (:779-841), on device arrays. Per step:
        Y0 = V + sum F_k V; Y2 from the Douglas sweep; then Z = Y0 +
        (dt/2) M (Y2 - V) (modified: theta dt M (Y2 - V) + (1/2 - theta)
        sum F_k.apply(Y2 - V), residuals included as the reference applies
        them), and the same sweep from Z. The reference has these on the CPU
        engine only; they run here on the per-operator kernels."""
        dt, theta = float(dt), float(theta)
        if not self.operators:
            self.scale_and_combine_operators()
        Firsts = [o.mul_scalar_from_host(dt) for d, o in self.operators.items()]
        dims = self._dims()
        Les = [o.mul_scalar_from_host(theta).mul_scalar_from_host(dt, inplace=True)
               for d, o in dims]
        Lis = [o.mul_scalar_from_host(theta * -dt).add(1, inplace=True) for d, o in dims]
        for L in Les + Lis:
            L.enable_residual(False)
        # the reference's Craig-Sneyd keeps full bandwidth; folding the corner
        # rows is the same operator, a switched scheme's inner band is not
        for L in Les + Lis + Firsts:
            if L.is_foldable() and L.band2 is None:
                L.diagonalize()
        cross = self.operators.get((0, 1))
        c = theta * dt if modified else 0.5 * dt
        X = torch.empty_like(V)
        Y = torch.empty_like(V)
        Y0 = torch.empty_like(V)
        D = torch.empty_like(V)
        for _ in range(int(n)):
            Y.copy_(V)
            for L in Firsts:
                _apply_into(L, X, V)
                _axpby(Y, X, 1.0, 1.0)
            Y0.copy_(Y)
            for Le, Li in zip(Les, Lis):
                _apply_into(Le, X, V)
                _axpby(Y, X, 1.0, -1.0)
                Li.solve_(Y, overwrite=True)
            D.copy_(Y)
            _axpby(D, V, 1.0, -1.0)          # D = Y2 - V
            Y.copy_(Y0)
            if cross is not None:
                _apply_into(cross, X, D)
                _axpby(Y, X, 1.0, c)
            if modified:
                for L in Firsts:
                    _apply_into(L, X, D)
                    _axpby(Y, X, 1.0, 0.5 - theta)
            for Le, Li in zip(Les, Lis):
                _apply_into(Le, X, V)
                _axpby(Y, X, 1.0, -1.0)
                Li.solve_(Y, overwrite=True)
            V.copy_(Y)
        return V

    def solve_craigsneyd2_(self, n, dt, V, theta=0.5):
        """Modified Craig-Sneyd (FiniteDifference.pyx:779-841)."""
        return self.solve_craigsneyd_(n, dt, V, theta, modified=True)

    def solve_craigsneyd(self, n, dt, initial=None, theta=0.5, callback=None, numpy=False):
        if callback or numpy:
            raise NotImplementedError("Callbacks and Numpy not available for GPU solver.")
        V = self._initial(initial)
        self.solve_craigsneyd_(int(n), dt, V, theta)
        return V.cpu().numpy()

    def solve_craigsneyd2(self, n, dt, initial=None, theta=0.5, callback=None, numpy=False):
        if callback or numpy:
            raise NotImplementedError("Callbacks and Numpy not available for GPU solver.")
        V = self._initial(initial)
        self.solve_craigsneyd_(int(n), dt, V, theta, modified=True)
        return V.cpu().numpy()

    def solve_smooth_(self, n, dt, V, smoothing_steps=2):
        """Rannacher start: 2*s implicit half-steps, then HV at theta = 0.6
        (FiniteDifferenceEngine.pyx:1010-1016)."""
        self.solve_implicit_(smoothing_steps * 2, float(dt) * 0.5, V)
        self.solve_hundsdorferverwer_(int(n) - smoothing_steps, dt, V, 0.60)
        return V


class HestonFiniteDifferenceEngine(FiniteDifferenceEngineADI):
    """Heston engine (FiniteDifferenceEngineGPU.pyx:596-757)."""

    def __init__(self, option, grid=None, spot_max=1500.0, spot_min=0.0, spots=None, vars=None,
                 var_max=10.0, nspots=100, nvols=100, spotdensity=7.0, varexp=4.0,
                 force_exact=True, flip_idx_var=False, flip_idx_spot=False, schemes=None,
                 coefficients=None, boundaries=None, cache=True, verbose=True,
                 force_bandwidth=None, fused=True):
        FiniteDifferenceEngineADI.__init__(self)
        if schemes is not None:
            raise NotImplementedError("Only central differencing (with the flip_idx_spot / "
                                      "flip_idx_var switches) is supported on GPU")
        assert isinstance(option, Option)
        self.option = option
        self.fused = fused
        self.coefficients = [(0,), (0, 0), (1,), (1, 1), (0, 1), ()]
        if isinstance(option, BarrierOption):
            if option.top:
                if option.top[0]:
                    raise NotImplementedError("Knockin barriers are not supported.")
                spot_max = option.top[1]
                if grid:
                    assert np.allclose(spot_max, max(grid.mesh[0]))
            if option.bottom:
                raise NotImplementedError("Bottom barriers are not supported for GPU creation.")
        if grid:
            self.spots = np.array(grid.mesh[0], dtype=float)
            self.vars = np.array(grid.mesh[1], dtype=float)
        else:
            if vars is None:
                vars = _mesh.exponential_space(0.00, option.variance.value, var_max, varexp,
                                               nvols, force_exact=force_exact)
            self.vars = np.array(vars, dtype=float)
            if spots is None:
                if isinstance(option, BarrierOption) and option.top and not option.top[0]:
                    spots = _mesh.exponential_space(0.00, option.strike, spot_max, 1.0 / 3,
                                                    nspots, force_exact=force_exact)
                    self.barrier = option.top[1]
                else:
                    spots = _mesh.sinh_space(option.strike - spot_min, spot_max - spot_min,
                                             spotdensity, nspots,
                                             force_exact=force_exact) + spot_min
            self.spots = np.array(spots, dtype=float)
            K = option.strike
            grid = Grid([self.spots, self.vars], initializer=lambda *x: np.maximum(x[0] - K, 0))
        self.spots[np.argmin(np.abs(self.spots - option.spot))] = option.spot
        # up/down-winding (heston.py:414-439): forward differences in S from the
        # strike on, backward differences in v from the mean variance on
        from bisect import bisect_left
        if flip_idx_var is True:
            flip_idx_var = bisect_left(list(np.round(self.vars, decimals=5)),
                                       np.round(option.variance.mean, decimals=5))
        if flip_idx_spot is True:
            flip_idx_spot = bisect_left(list(np.round(self.spots, decimals=5)),
                                        np.round(option.strike, decimals=5))
        self.flip_idx_spot = None if flip_idx_spot is False or flip_idx_spot is None \
            else int(flip_idx_spot)
        self.flip_idx_var = None if flip_idx_var is False or flip_idx_var is None \
            else int(flip_idx_var)
        if self.flip_idx_spot is not None or self.flip_idx_var is not None:
            # the fused engine builds centred stencils only; the switched
            # schemes run on the per-operator kernels (the reference GPU engine
            # does not run them at all, FiniteDifferenceEngineGPU.pyx:634)
            self.fused = False
        grid._mesh = (self.spots, self.vars)
        self.grid = grid
        self.gpugrid = _dev(self.grid.domain[-1])
        self.zero_derivative_coefficient_host = np.atleast_1d(
            -self.option.interest_rate.value / self.grid.ndim)

    def make_operator_templates(self):
        """Single-derivative Heston operators (FiniteDifferenceEngineGPU.pyx:697-724)."""
        m0, m1 = self.spots, self.vars
        bar = bool(self.barrier)
        fs, fv = getattr(self, "flip_idx_spot", None), getattr(self, "flip_idx_var", None)
        self.simple_operators[(0,)] = for_vector(m0, m1.size, 1, 0, bar,
                                                 "forward" if fs is not None else None, fs)
        self.simple_operators[(0, 0)] = for_vector(m0, m1.size, 2, 0, bar)
        self.simple_operators[(1,)] = for_vector(m1, m0.size, 1, 1, bar,
                                                 "backward" if fv is not None else None, fv)
        self.simple_operators[(1, 1)] = for_vector(m1, m0.size, 2, 1, bar)
        if getattr(self.option, "correlation", 0) != 0:
            self.simple_operators[(0, 1)] = mixed_for_vector(m0, m1)

    def coefficient_vector(self, d, dim):
        """Per-point Heston coefficients in the operator's block-major order
        (heston.py:303-325; GPU: _coefficients.cu:19-115)."""
        r, kappa, theta, sigma, rho = self.option.params()
        if self._rate is not None:
            r = self._rate          # this step's rate (time-dependent coefficients)
        S, v = self.spots, self.vars
        if dim == 0:
            Sg, vg = np.meshgrid(S, v)          # [nv, nS]: spot fastest
        else:
            vg, Sg = np.meshgrid(v, S)          # [nS, nv]: variance fastest
        Sg, vg = Sg.ravel(), vg.ravel()
        if d == (0,):
            return r * Sg
        if d == (0, 0):
            return 0.5 * vg * Sg ** 2
        if d == (1,):
            out = kappa * (theta - vg)
            out[Sg == 0] = 0
            return out
        if d == (1, 1):
            out = 0.5 * sigma ** 2 * vg
            out[Sg == 0] = 0
            return out
        if d == (0, 1):
            return rho * sigma * Sg * vg
        return None

    @property
    def idx(self):
        return _mesh.price_index(self.spots, self.vars, self.option.spot,
                                 self.option.variance.value)

    @property
    def price(self):
        return self.grid.domain[-1][self.idx]

    # -- fused path --
    def _batch(self, scheme, n_steps, dt, theta, implicit_steps=0, factor=0.5):
        from .batch import HestonBatch
        rates = None
        if self.rates is not None:
            total = int(implicit_steps) + int(n_steps)
            r = np.asarray(self.rates, dtype=np.float64).reshape(-1)
            if r.size < total:
                raise ValueError("rates holds %d steps; the solve needs %d" % (r.size, total))
            rates = r[:total].reshape(1, total)
        return HestonBatch([self.option], [(self.spots, self.vars)], scheme=scheme,
                           n_steps=n_steps, dt=[dt], theta=theta, implicit_steps=implicit_steps,
                           implicit_dt_factor=factor, barrier=[bool(self.barrier)], rates=rates)

    def _fused_run(self, initial, scheme, n_steps, dt, theta, implicit_steps=0, factor=0.5):
        V0 = self.grid.domain[-1] if initial is None else initial
        b = self._batch(scheme, n_steps, dt, theta, implicit_steps, factor)
        out = b.solve([np.asarray(V0, dtype=float)])[0]
        self.grid.domain.append(out.copy())
        return out

    def solve_implicit(self, n, dt, initial=None, callback=None, numpy=False):
        if not self.fused:
            return FiniteDifferenceEngineADI.solve_implicit(self, n, dt, initial, callback, numpy)
        return self._fused_run(initial, "douglas", 0, dt, 0.5, int(n), 1.0)

    def solve_douglas(self, n, dt, initial=None, theta=0.5, callback=None, numpy=False):
        if not self.fused:
            return FiniteDifferenceEngineADI.solve_douglas(self, n, dt, initial, theta)
        return self._fused_run(initial, "douglas", int(n), dt, theta)

    def solve_hundsdorferverwer(self, n, dt, initial=None, theta=0.5, callback=None,
                                numpy=False):
        if not self.fused:
            return FiniteDifferenceEngineADI.solve_hundsdorferverwer(self, n, dt, initial, theta)
        return self._fused_run(initial, "hv", int(n), dt, theta)

    def solve_smooth(self, n, dt, initial=None, callback=None, smoothing_steps=2, scheme=None):
        if not self.fused:
            return FiniteDifferenceEngineADI.solve_smooth(self, n, dt, initial, callback,
                                                          smoothing_steps, scheme)
        if scheme:
            raise NotImplementedError("Changing smoothing schemes not supported on GPU.")
        return self._fused_run(initial, "hv", int(n) - smoothing_steps, dt, 0.60,
                               2 * smoothing_steps, 0.5)


class BlackScholesFiniteDifferenceEngine(FiniteDifferenceEngineADI):
    """1-D Black-Scholes engine (blackscholes.py:144-239), non-log mesh.

    ``solve_*`` run the fused batched engine (``BlackScholesBatch``, the
    whole schedule in one launch) by default; ``fused=False``, or custom
    coefficients or boundaries, select the per-operator path."""

    def __init__(self, option, grid=None, spot_max=1500.0, nspots=100, spotdensity=7.0,
                 force_exact=True, coefficients=None, boundaries=None, fused=True, **kwargs):
        self.fused = bool(fused) and not coefficients and not boundaries
        self.option = option
        r = option.interest_rate.value
        var = option.variance.value
        if grid is None:
            spots = _mesh.sinh_space(option.spot, spot_max, spotdensity, nspots,
                                     force_exact=force_exact)
            K = option.strike
            grid = Grid([spots], initializer=lambda x: np.maximum(x - K, 0))
        self.spots = np.asarray(grid.mesh[0])
        if not coefficients:
            coefficients = {(): lambda t: -r, (0,): lambda t, *d: r * d[0],
                            (0, 0): lambda t, *d: 0.5 * var * d[0] ** 2}
        if not boundaries:
            boundaries = {(0,): ((0, lambda *a: 0.0), (1, lambda t, x: 1.0)),
                          (0, 0): ((0, lambda *a: 0.0), (None, lambda t, x: 1.0))}
        FiniteDifferenceEngineADI.__init__(self, grid, coefficients, boundaries)
        self.option = option

    @property
    def idx(self):
        return int(np.argmin(np.abs(self.spots - self.option.spot)))

    @property
    def price(self):
        return self.grid.domain[-1][self.idx]

    # -- fused path --
    def _fused_run(self, initial, scheme, n_steps, dt, theta, implicit_steps=0, factor=0.5):
        from .batch import BlackScholesBatch
        V0 = self.grid.domain[-1] if initial is None else initial
        b = BlackScholesBatch([self.option], [self.spots], scheme=scheme, n_steps=n_steps,
                              dt=[dt], theta=theta, implicit_steps=implicit_steps,
                              implicit_dt_factor=factor)
        out = b.solve([np.asarray(V0, dtype=float)])[0]
        self.grid.domain.append(out.copy())
        return out

    def solve_implicit(self, n, dt, initial=None, callback=None, numpy=False):
        if not self.fused:
            return FiniteDifferenceEngineADI.solve_implicit(self, n, dt, initial, callback, numpy)
        return self._fused_run(initial, "douglas", 0, dt, 0.5, int(n), 1.0)

    def solve_douglas(self, n, dt, initial=None, theta=0.5, callback=None, numpy=False):
        if not self.fused:
            return FiniteDifferenceEngineADI.solve_douglas(self, n, dt, initial, theta)
        return self._fused_run(initial, "douglas", int(n), dt, theta)

    def solve_hundsdorferverwer(self, n, dt, initial=None, theta=0.5, callback=None,
                                numpy=False):
        if not self.fused:
            return FiniteDifferenceEngineADI.solve_hundsdorferverwer(self, n, dt, initial, theta)
        return self._fused_run(initial, "hv", int(n), dt, theta)

    def solve_craigsneyd(self, n, dt, initial=None, theta=0.5, callback=None, numpy=False):
        if not self.fused:
            return FiniteDifferenceEngineADI.solve_craigsneyd(self, n, dt, initial, theta)
        return self._fused_run(initial, "cs", int(n), dt, theta)

    def solve_craigsneyd2(self, n, dt, initial=None, theta=0.5, callback=None, numpy=False):
        if not self.fused:
            return FiniteDifferenceEngineADI.solve_craigsneyd2(self, n, dt, initial, theta)
        return self._fused_run(initial, "mcs", int(n), dt, theta)

    def solve_smooth(self, n, dt, initial=None, callback=None, smoothing_steps=2, scheme=None):
        if not self.fused:
            return FiniteDifferenceEngineADI.solve_smooth(self, n, dt, initial, callback,
                                                          smoothing_steps, scheme)
        if scheme:
            raise NotImplementedError("Changing smoothing schemes not supported on GPU.")
        return self._fused_run(initial, "hv", int(n) - smoothing_steps, dt, 0.60,
                               2 * smoothing_steps, 0.5)


def heston_coefficients(r, kappa, theta, sigma, rho):
    """The Heston PDE coefficient dict of heston.py:303-333."""
    def mu_s(t, *dim):
        return r * dim[0]

    def gamma2_s(t, *dim):
        return 0.5 * dim[1] * dim[0] ** 2

    def mu_v(t, *dim):
        if np.isscalar(dim[0]):
            if dim[0] == 0:
                return 0
        ret = kappa * (theta - dim[1])
        ret[dim[0] == 0] = 0
        return ret

    def gamma2_v(t, *dim):
        if np.isscalar(dim[0]):
            if dim[0] == 0:
                return 0
        ret = 0.5 * sigma ** 2 * dim[1]
        ret[dim[0] == 0] = 0
        return ret

    def cross(t, *dim):
        return rho * sigma * dim[0] * dim[1]

    return {(): lambda t: -r, (0,): mu_s, (0, 0): gamma2_s, (1,): mu_v, (1, 1): gamma2_v,
            (0, 1): cross}


def heston_boundaries():
    """The Heston boundary dict of heston.py:335-359."""
    return {(0,): ((0, lambda t, *dim: 0.0), (1, lambda t, *dim: 1.0)),
            (0, 0): ((0, lambda t, *dim: 0.0), (None, lambda t, *dim: 1.0)),
            (1,): ((None, lambda t, *dim: None), (None, lambda t, *dim: None)),
            (1, 1): ((1, lambda t, *dim: 0), (None, lambda t, *dim: None))}
