"""Batched Heston pricing on the fused engine (fdadi_heston_* in include/fdadi.h).

Thousands of options with different parameters and uneven grids are packed
into one arena and advanced together: every time step is a handful of
launches over the whole batch, optionally replayed from a CUDA graph. The
reference prices one option per engine with dozens of launches per step
(FiniteDifferenceEngineGPU.pyx:502-562); this has no reference counterpart
beyond the per-option results, which match the reference CPU engine.
"""
import ctypes
import hashlib
import json
import os

import numpy as np
import torch

from . import _lib
from . import mesh as _mesh

SCHEMES = {"douglas": _lib.SCHEME_DOUGLAS, "hv": _lib.SCHEME_HV,
           "hundsdorferverwer": _lib.SCHEME_HV, "cs": _lib.SCHEME_CS,
           "craigsneyd": _lib.SCHEME_CS, "mcs": _lib.SCHEME_MCS, "craigsneyd2": _lib.SCHEME_MCS}
HV_THETA = 0.5 + np.sqrt(3.0) / 6.0


# Launch shapes the engine implements (fdadi_heston_plan_t fields): spot solve
# (kind 0: line per thread, rows prefetched, threads per block; kind 1:
# partitioned lines, lines per block, segments per line) and variance solve
# (kind 0: one tile per warp, factors loaded in the recurrence; kind 1: two
# tiles, pipelined copies, factors by shuffle; kind 2: one tile, factors by
# shuffle; warps per block; kind 3: partitioned lines, one 32-row task per
# block split into column segments, warps per block).
SPOT_PLANS = [(0, 1, 128), (0, 1, 64), (0, 1, 256), (0, 4, 32), (0, 8, 32), (0, 8, 64),
              (1, 32, 4), (1, 32, 8), (1, 32, 16), (1, 32, 32), (1, 16, 16), (1, 16, 32),
              (1, 16, 64), (1, 8, 32), (1, 8, 64), (1, 8, 128), (0, 2, 64), (0, 2, 128),
              (0, 4, 64), (0, 4, 128)]
VAR_PLANS = [(0, 4), (0, 2), (1, 1), (1, 2), (1, 4), (2, 1), (2, 2), (2, 4), (3, 4), (3, 8),
             (3, 16)]


def make_plan(spot, var, groups=1, expl_per_sm=0):
    """Plan dict from a SPOT_PLANS and a VAR_PLANS entry, a number of option
    groups (1..4) whose explicit stages and line solves overlap, and the
    explicit stage's blocks per SM (0: one block per tile)."""
    return {"spot_kind": spot[0], "spot_a": spot[1], "spot_b": spot[2],
            "var_kind": var[0], "var_warps": var[1], "groups": groups,
            "expl_per_sm": expl_per_sm}


# Tuned launch plans by batch shape (this process); FDADI_TUNE_CACHE names a
# JSON file that keeps them across processes.
_PLANS = {}


def _cache_path():
    return os.environ.get("FDADI_TUNE_CACHE")


def _load_plans():
    path = _cache_path()
    if path and os.path.exists(path):
        try:
            with open(path) as f:
                for k, v in json.load(f).items():
                    _PLANS.setdefault(k, v)
        except (OSError, ValueError):
            pass


def _save_plans():
    path = _cache_path()
    if path:
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(_PLANS, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def option_params(opt):
    """(r, kappa, theta, sigma, rho) of a HestonOption or a 5-sequence."""
    if hasattr(opt, "params"):
        return opt.params()
    return tuple(float(x) for x in opt)


class HestonBatch(object):
    """A prepared batch: operators and line-solve factors of every option
    built on the device once; ``run`` advances a packed state arena.

    options: HestonOption objects or (r, kappa, theta, sigma, rho) tuples.
    meshes:  list of (spots, vars) numpy arrays, one per option.
    dt:      per-option main step (scalar or sequence).
    Schedule: ``implicit_steps`` fully implicit steps of dt*implicit_dt_factor,
    then ``n_steps`` of ``scheme`` ("douglas", "hv", "cs" or "mcs") at ``theta``.
    plan:    launch plan of the line solves: None (size heuristic), "auto"
             (measured by the autotuner on this batch, cached by batch shape)
             or a dict of fdadi_heston_plan_t fields.
    rates:   time-dependent coefficients: [n, implicit_steps + n_steps] interest
             rate of every step of every option (the implicit steps first), or
             None to use each option's constant r. With rates, the operators and
             line-solve factors are rebuilt before every step."""

    def __init__(self, options, meshes, scheme="hv", n_steps=1, dt=0.01, theta=HV_THETA,
                 implicit_steps=0, implicit_dt_factor=0.5, barrier=None, drop_zero_mixed=True,
                 graph=False, device=None, stream=None, plan=None, rates=None):
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        n = len(options)
        if n == 0 or len(meshes) != n:
            raise ValueError("need one mesh per option")
        self.options = options
        self.n = n
        self.n0 = np.array([np.asarray(m[0]).size for m in meshes], dtype=np.int32)
        self.n1 = np.array([np.asarray(m[1]).size for m in meshes], dtype=np.int32)
        self.sizes = self.n0.astype(np.int64) * self.n1
        self.p_off = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        self.total_points = int(self.p_off[-1])
        dev = self.device
        self.spots = torch.as_tensor(np.concatenate([np.asarray(m[0], np.float64) for m in meshes]),
                                     device=dev)
        self.vars = torch.as_tensor(np.concatenate([np.asarray(m[1], np.float64) for m in meshes]),
                                    device=dev)
        self.params = torch.as_tensor(np.array([option_params(o) for o in options],
                                               dtype=np.float64).reshape(n, 5), device=dev)
        self.dt = torch.as_tensor(np.broadcast_to(np.asarray(dt, dtype=np.float64), (n,)).copy(),
                                  device=dev)
        bar = np.zeros(n, dtype=np.int32) if barrier is None else np.asarray(barrier, np.int32)
        self.barrier = torch.as_tensor(bar, device=dev)
        self.rates = None
        if rates is not None:
            total = int(implicit_steps) + int(n_steps)
            r = np.ascontiguousarray(rates, dtype=np.float64)
            if r.shape != (n, total):
                raise ValueError("rates must have shape (%d, %d) (options, implicit_steps + "
                                 "n_steps), got %s" % (n, total, r.shape))
            self.rates = torch.as_tensor(r, device=dev)
        self.graph = bool(graph)
        if stream is None:
            stream = torch.cuda.Stream(device=dev) if self.graph else torch.cuda.current_stream(dev)
        self.stream = stream
        flags = (_lib.HESTON_DROP_ZERO_MIXED if drop_zero_mixed else 0) | \
                (_lib.HESTON_GRAPH if self.graph else 0)
        self._n0_host = self.n0.copy()
        self._n1_host = self.n1.copy()
        self.struct = _lib.HestonBatch(
            n, SCHEMES[scheme], int(n_steps), int(implicit_steps), float(theta),
            float(implicit_dt_factor), flags, 0,
            self._n0_host.ctypes.data, self._n1_host.ctypes.data,
            self.spots.data_ptr(), self.vars.data_ptr(), self.params.data_ptr(),
            self.dt.data_ptr(), self.barrier.data_ptr(), None,
            self.rates.data_ptr() if self.rates is not None else None)
        self._plan = None
        lib = _lib.load()
        nbytes = lib.fdadi_heston_workspace_bytes(ctypes.byref(self.struct))
        if nbytes < 0:
            raise ValueError("bad batch: " + _lib.last_error())
        self.workspace_bytes = int(nbytes)
        self.workspace = torch.empty(self.workspace_bytes, dtype=torch.uint8, device=dev)
        self._prepare()
        if isinstance(plan, str):
            if plan != "auto":
                raise ValueError("plan must be None, 'auto' or a dict")
            self.tune()
        elif plan is not None:
            self.set_plan(plan)

    @property
    def shape_key(self):
        """Key of the batch shape the launch plan depends on."""
        h = hashlib.sha1(self.n0.tobytes() + self.n1.tobytes()).hexdigest()[:16]
        return "%d:%d:%s" % (self.n, self.total_points, h)

    def set_plan(self, plan):
        """Use this launch plan (dict of fdadi_heston_plan_t fields) from now on."""
        self._plan = _lib.HestonPlan.from_dict(plan)
        self.struct.plan = ctypes.cast(ctypes.pointer(self._plan), ctypes.c_void_p)

    @property
    def plan(self):
        """The launch plan in use (the size heuristic's when none was set)."""
        if self._plan is not None:
            return self._plan.as_dict()
        p = _lib.HestonPlan()
        _lib.call("fdadi_heston_default_plan", ctypes.byref(self.struct), ctypes.byref(p))
        return p.as_dict()

    def tune(self, reps=3, force=False):
        """Measure every launch plan of the line solves on this batch and keep
        the fastest (cached by batch shape). Overwrites the stage buffers
        only; the state is untouched."""
        _load_plans()
        key = self.shape_key
        if force or key not in _PLANS:
            p = _lib.HestonPlan()
            with torch.cuda.stream(self.stream):
                _lib.call("fdadi_heston_tune", ctypes.byref(self.struct),
                          ctypes.c_void_p(self.workspace.data_ptr()), self.workspace_bytes,
                          int(reps), ctypes.byref(p), self._sptr())
            _PLANS[key] = p.as_dict()
            _save_plans()
        self.set_plan(_PLANS[key])
        return self.plan

    @classmethod
    def from_options(cls, options, nspots, nvols, spot_max_factor=8.0, var_max=5.0,
                     spotdensity=7.0, varexp=4.0, **kw):
        """Meshes as the reference Heston engine builds them
        (heston.py:384-406) with S_max = spot_max_factor * K."""
        ns = np.broadcast_to(np.asarray(nspots), (len(options),))
        nv = np.broadcast_to(np.asarray(nvols), (len(options),))
        meshes = [_mesh.heston_meshes(o.spot, o.strike, o.variance.value, int(a), int(b),
                                      spot_max_factor * o.strike, var_max, spotdensity, varexp)
                  for o, a, b in zip(options, ns, nv)]
        return cls(options, meshes, **kw), meshes

    def _sptr(self):
        return ctypes.c_void_p(self.stream.cuda_stream)

    def price_calls(self, spot, strikes, variance, params, dt, V=None, put=False,
                    spot_max_factor=8.0, var_max=5.0, spotdensity=7.0, varexp=4.0,
                    threads=0):
        """Price a new set of options on this batch's grid sizes, from their
        parameters (host arrays in, host prices out), as the reference engine
        does per option (FiniteDifferenceEngineGPU.pyx:662-686 builds the
        meshes, heston.py:402 the payoff, :461-469 reads the price).

        Host: every option's meshes (spot: sinh mesh on [0, ~spot_max_factor
        K] clustered at K; variance: exponential mesh on [0, ~var_max]; the
        grid point nearest the spot moved onto it), bit-identical to
        mesh.heston_meshes, and each price's arena index. Device: the meshes,
        parameters, steps and strikes copied from pinned memory on the batch's
        stream, the operators and factors rebuilt, the payoff, the time loop
        and the price gather; the prices come back to pinned memory.

        spot, variance: scalars or [n]; strikes, dt: [n]; params: [n, 5] of
        (r, kappa, theta, sigma, rho). V: the device state arena to use
        (allocated on first use). Returns a numpy array of n prices."""
        mesh_kw = dict(spot_max_factor=spot_max_factor, var_max=var_max,
                       spotdensity=spotdensity, varexp=varexp, threads=threads)
        slot = self._stage(0, spot, strikes, variance, params, dt, **mesh_kw)
        self._launch(slot, V, put)
        return self._finish(slot)

    def price_calls_many(self, sets, V=None, put=False, spot_max_factor=8.0, var_max=5.0,
                         spotdensity=7.0, varexp=4.0, threads=0):
        """price_calls over a sequence of option sets (each a tuple (spot,
        strikes, variance, params, dt) on this batch's grid sizes), pipelined:
        the host builds set k+1's meshes and indices into a second pinned
        staging area while the device prices set k, so the host's share of a
        set costs no device time. Returns a list of price arrays, in order."""
        mesh_kw = dict(spot_max_factor=spot_max_factor, var_max=var_max,
                       spotdensity=spotdensity, varexp=varexp, threads=threads)
        out = []
        it = iter(sets)
        first = next(it, None)
        if first is None:
            return out
        cur = self._stage(0, *first, **mesh_kw)
        k = 1
        for nxt in it:
            self._launch(cur, V, put)
            # set k's host work runs while the device prices set k - 1; the
            # other slot's copies finished when its set was read back
            staged = self._stage(k % 2, *nxt, **mesh_kw)
            out.append(self._finish(cur))
            cur = staged
            k += 1
        self._launch(cur, V, put)
        out.append(self._finish(cur))
        return out

    def _slot(self, i):
        """Pinned host staging area i (two, for price_calls_many)."""
        if not hasattr(self, "_h"):
            n = self.n
            pin = lambda t: t.pin_memory()
            self._h = [dict(spots=pin(torch.empty(self.spots.numel(), dtype=torch.float64)),
                            vars=pin(torch.empty(self.vars.numel(), dtype=torch.float64)),
                            params=pin(torch.empty(n * 5, dtype=torch.float64)),
                            dt=pin(torch.empty(n, dtype=torch.float64)),
                            K=pin(torch.empty(n, dtype=torch.float64)),
                            idx=pin(torch.empty(n, dtype=torch.int64)),
                            prices=pin(torch.empty(n, dtype=torch.float64)))
                       for _ in range(2)]
            self._d = dict(K=torch.empty(n, dtype=torch.float64, device=self.device),
                           idx=torch.empty(n, dtype=torch.int64, device=self.device),
                           prices=torch.empty(n, dtype=torch.float64, device=self.device))
        return self._h[i]

    def _stage(self, i, spot, strikes, variance, params, dt, spot_max_factor=8.0, var_max=5.0,
               spotdensity=7.0, varexp=4.0, threads=0):
        """Host part of price_calls into staging area i: meshes, price indices
        and the per-option inputs."""
        n = self.n
        strikes = np.ascontiguousarray(strikes, dtype=np.float64).reshape(-1)
        if strikes.size != n:
            raise ValueError("need %d strikes, got %d" % (n, strikes.size))
        params = np.ascontiguousarray(params, dtype=np.float64).reshape(n, 5)
        dt = np.broadcast_to(np.asarray(dt, dtype=np.float64), (n,))
        spot = np.broadcast_to(np.asarray(spot, dtype=np.float64), (n,))
        variance = np.broadcast_to(np.asarray(variance, dtype=np.float64), (n,))
        spots, vars_ = _mesh.heston_meshes_batch(spot, strikes, variance, self.n0, self.n1,
                                                 spot_max_factor * strikes, var_max,
                                                 spotdensity, varexp, threads=threads)
        flat = self.p_off[:-1] + _mesh.price_index_batch(spots, vars_, self.n0, self.n1, spot,
                                                         variance)
        h = self._slot(i)
        h["spots"].numpy()[:] = spots
        h["vars"].numpy()[:] = vars_
        h["params"].numpy()[:] = params.reshape(-1)
        h["dt"].numpy()[:] = dt
        h["K"].numpy()[:] = strikes
        h["idx"].numpy()[:] = flat
        return h

    def _launch(self, h, V=None, put=False):
        """Device part of price_calls from a staging area, queued on the
        batch's stream (the operator build waits for its own copies)."""
        if V is None:
            if getattr(self, "_V", None) is None:
                self._V = torch.empty(self.total_points, dtype=torch.float64, device=self.device)
            V = self._V
        self._check_state(V)
        d = self._d
        with torch.cuda.stream(self.stream):
            self.stream.wait_stream(torch.cuda.current_stream(self.device))
            self.spots.copy_(h["spots"], non_blocking=True)
            self.vars.copy_(h["vars"], non_blocking=True)
            self.params.view(-1).copy_(h["params"], non_blocking=True)
            self.dt.copy_(h["dt"], non_blocking=True)
            d["K"].copy_(h["K"], non_blocking=True)
            d["idx"].copy_(h["idx"], non_blocking=True)
            self._prepare()
            self.payoff(d["K"], V, put=put)
            self.run(V)
            self.gather(V, d["idx"], d["prices"])
            h["prices"].copy_(d["prices"], non_blocking=True)
        self._last = h

    def _finish(self, h):
        self.stream.synchronize()
        return h["prices"].numpy().copy()

    def price_calls_last(self):
        """The prices of the last price_calls() (a copy)."""
        return self._last["prices"].numpy().copy()

    @property
    def price_calls_h2d_bytes(self):
        """Host-to-device bytes one price_calls() copies."""
        return 8 * (int(self.spots.numel()) + int(self.vars.numel()) + 5 * self.n + 4 * self.n)

    def _prepare(self):
        with torch.cuda.stream(self.stream):
            _lib.call("fdadi_heston_prepare", ctypes.byref(self.struct),
                      ctypes.c_void_p(self.workspace.data_ptr()), self.workspace_bytes,
                      self._sptr())

    @property
    def launches_per_run(self):
        return int(_lib.load().fdadi_heston_launch_count(ctypes.byref(self.struct)))

    def pack(self, grids):
        """Host grids (one [n0, n1] array per option) -> device arena."""
        flat = np.concatenate([np.asarray(g, dtype=np.float64).reshape(-1) for g in grids])
        if flat.size != self.total_points:
            raise ValueError("Dimension mismatch: %d grid points for a %d-point batch"
                             % (flat.size, self.total_points))
        return torch.as_tensor(flat, device=self.device)

    def unpack(self, V):
        h = V.detach().cpu().numpy()
        return [h[self.p_off[k]:self.p_off[k + 1]].reshape(self.n0[k], self.n1[k])
                for k in range(self.n)]

    def _check_state(self, V):
        """The kernels index V by the arena's offsets: refuse anything else."""
        if (V.dtype != torch.float64 or not V.is_cuda or V.numel() != self.total_points
                or not V.is_contiguous()):
            raise ValueError("state must be a contiguous CUDA float64 tensor of %d points"
                             % self.total_points)

    @staticmethod
    def _check_index(idx, n=None):
        if (idx.dtype != torch.int64 or not idx.is_cuda or not idx.is_contiguous()
                or (n is not None and idx.numel() != n)):
            raise ValueError("indices must be a contiguous CUDA int64 tensor%s"
                             % ("" if n is None else " of %d values" % n))

    def run(self, V):
        """Advance the packed state arena V (device, float64) in place."""
        self._check_state(V)
        if self.graph:
            self.stream.wait_stream(torch.cuda.current_stream(self.device))
        _lib.call("fdadi_heston_run", ctypes.byref(self.struct),
                  ctypes.c_void_p(self.workspace.data_ptr()), self.workspace_bytes,
                  ctypes.c_void_p(V.data_ptr()), self._sptr())
        if self.graph:
            torch.cuda.current_stream(self.device).wait_stream(self.stream)
        return V

    def payoff(self, strikes, V=None, put=False):
        """Initial state built on the device: max(S - K, 0) (or the put's
        max(K - S, 0)) on every option's mesh. strikes: device float64 [n].

        The payoff is taken on the batch's own spots. The reference takes it
        before a grid point is moved onto the spot (heston.py:402-406); for
        that order, build the grids on the host and use pack()."""
        if (strikes.dtype != torch.float64 or not strikes.is_cuda or strikes.numel() != self.n
                or not strikes.is_contiguous()):
            raise ValueError("strikes must be a contiguous CUDA float64 tensor of %d values"
                             % self.n)
        if V is None:
            V = torch.empty(self.total_points, dtype=torch.float64, device=self.device)
        self._check_state(V)
        cur = torch.cuda.current_stream(self.device)
        _lib.call("fdadi_heston_payoff", ctypes.byref(self.struct),
                  ctypes.c_void_p(self.workspace.data_ptr()), self.workspace_bytes,
                  ctypes.c_void_p(strikes.data_ptr()), 1 if put else 0,
                  ctypes.c_void_p(V.data_ptr()), ctypes.c_void_p(cur.cuda_stream))
        return V

    def greeks(self, V, flat_idx):
        """(price, delta, gamma) device tensors: each option's value at its
        arena index and the centred non-uniform S-derivatives there."""
        self._check_state(V)
        self._check_index(flat_idx, self.n)
        out = [torch.empty(self.n, dtype=torch.float64, device=self.device) for _ in range(3)]
        cur = torch.cuda.current_stream(self.device)
        _lib.call("fdadi_heston_greeks", ctypes.byref(self.struct),
                  ctypes.c_void_p(self.workspace.data_ptr()), self.workspace_bytes,
                  ctypes.c_void_p(V.data_ptr()), ctypes.c_void_p(flat_idx.data_ptr()),
                  *[ctypes.c_void_p(t.data_ptr()) for t in out], ctypes.c_void_p(cur.cuda_stream))
        return tuple(out)

    def status(self, V):
        """Per-option status words (numpy int32): bit 1 = a line-solve pivot
        was zero or non-finite when the operators were built, bit 2 = the
        option's grid in V holds a NaN or infinity."""
        self._check_state(V)
        out = torch.empty(self.n, dtype=torch.int32, device=self.device)
        with torch.cuda.stream(self.stream):
            _lib.call("fdadi_heston_status", ctypes.byref(self.struct),
                      ctypes.c_void_p(self.workspace.data_ptr()), self.workspace_bytes,
                      ctypes.c_void_p(V.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                      self._sptr())
        self.stream.synchronize()
        return out.cpu().numpy()

    def check(self, V):
        """Raise ValueError naming the options whose solve failed (the
        reference raises from DIE() on a failed solve)."""
        st = self.status(V)
        bad = np.nonzero(st)[0]
        if bad.size:
            what = []
            for k in bad[:8]:
                why = []
                if st[k] & _lib.STATUS_PIVOT:
                    why.append("zero or non-finite pivot")
                if st[k] & _lib.STATUS_NONFINITE:
                    why.append("non-finite values")
                what.append("option %d: %s" % (k, ", ".join(why)))
            raise ValueError("%d of %d options failed (%s%s)"
                             % (bad.size, self.n, "; ".join(what), "; ..." if bad.size > 8 else ""))
        return st

    def solve(self, grids):
        """Host grids in, host grids out."""
        V = self.pack(grids)
        self.run(V)
        return self.unpack(V)

    def flat_index(self, points=None):
        """Arena index of each option's (spot, variance) grid point, by the
        reference's rounded bisection (FiniteDifferenceEngineGPU.pyx:727-734).
        points: per-option (spot, variance); default: the options' own."""
        if points is None:
            points = [(o.spot, o.variance.value) for o in self.options]
        idx = np.zeros(self.n, dtype=np.int64)
        spots = self.spots.cpu().numpy()
        vars_ = self.vars.cpu().numpy()
        s0 = np.concatenate([[0], np.cumsum(self.n0)])
        v0 = np.concatenate([[0], np.cumsum(self.n1)])
        for k, (spot, variance) in enumerate(points):
            S = spots[s0[k]:s0[k + 1]]
            v = vars_[v0[k]:v0[k + 1]]
            i, j = _mesh.price_index(S, v, spot, variance)
            idx[k] = self.p_off[k] + i * self.n1[k] + j
        return torch.as_tensor(idx, device=self.device)

    def gather(self, V, flat_idx, out=None):
        """V[flat_idx] on the device (the price read-out); flat_idx are arena
        indices as flat_index() returns them."""
        self._check_state(V)
        self._check_index(flat_idx)
        if out is None:
            out = torch.empty(flat_idx.numel(), dtype=torch.float64, device=self.device)
        _lib.call("fdadi_gather", ctypes.c_void_p(V.data_ptr()),
                  ctypes.c_void_p(flat_idx.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                  flat_idx.numel(),
                  ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream))
        return out


def payoff_grids(options, meshes):
    """Call payoff max(S - K, 0) on each option's grid (heston.py:402)."""
    return [np.maximum(np.asarray(m[0])[:, None] - o.strike, 0.0)
            * np.ones((1, np.asarray(m[1]).size)) for o, m in zip(options, meshes)]


def bs_meshes_batch(spot, sizes, spot_max=1500.0, spotdensity=7.0, force_exact=True, out=None):
    """The Black-Scholes engine's meshes for a batch (blackscholes.py:181-183:
    sinh_space(spot, spot_max, spotdensity, n, force_exact)), one per distinct
    (spot, size) and laid out option after option into out (a new array if
    None), bit-identical to building each option's; and each option's price
    index into that layout, the mesh point nearest its spot
    (blackscholes.py:222-228). Returns the indices."""
    sizes = np.asarray(sizes, dtype=np.int64).reshape(-1)
    spot = np.broadcast_to(np.asarray(spot, dtype=np.float64), sizes.shape)
    p_off = np.concatenate([[0], np.cumsum(sizes)])
    if out is None:
        out = np.empty(int(p_off[-1]))
    su, si = np.unique(spot, return_inverse=True)
    mx = int(sizes.max()) + 1
    ku, inv = np.unique(si.reshape(-1).astype(np.int64) * mx + sizes, return_inverse=True)
    inv = inv.reshape(-1)
    uniq = [(float(su[k // mx]), int(k % mx)) for k in ku]
    ms = [np.asarray(_mesh.sinh_space(s0, spot_max, spotdensity, m, force_exact=force_exact),
                     dtype=np.float64) for s0, m in uniq]
    at = np.array([int(np.argmin(np.abs(S - s0))) for S, (s0, _) in zip(ms, uniq)])
    np.concatenate([ms[u] for u in inv], out=out)
    return p_off[:-1] + at[inv]


def bs_params(opt):
    """(r, variance) of a Black-Scholes Option or a 2-sequence."""
    if hasattr(opt, "interest_rate"):
        return float(opt.interest_rate.value), float(opt.variance.value)
    r, var = opt
    return float(r), float(var)


class BlackScholesBatch(object):
    """Batched Black-Scholes on the fused engine (fdadi_bs_* in
    include/fdadi.h): every option's operators and Thomas factors built on
    the device once; ``run`` advances every option's whole schedule in one
    launch (each option is one independent line).

    options: Black-Scholes Option objects or (r, variance) tuples.
    meshes:  list of spot meshes (numpy arrays, >= 4 points each).
    dt:      per-option main step (scalar or sequence).
    Schedule: ``implicit_steps`` fully implicit steps of dt*implicit_dt_factor,
    then ``n_steps`` of ``scheme`` ("douglas", "hv", "cs" or "mcs") at ``theta``.
    The operator is the reference's (blackscholes.py:144-239): r S D_S +
    1/2 var S^2 D_SS - r, U = 0 at the first mesh point, dU/dS = 1 at S_max.
    prefetch: rows each thread keeps in flight in its sweeps (2, 4 or 8; 0
    chooses by batch size); the results do not depend on it."""

    def __init__(self, options, meshes, scheme="hv", n_steps=1, dt=0.01, theta=HV_THETA,
                 implicit_steps=0, implicit_dt_factor=0.5, device=None, stream=None,
                 prefetch=0):
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        n = len(options)
        if n == 0 or len(meshes) != n:
            raise ValueError("need one mesh per option")
        self.options = options
        self.n = n
        self.sizes = np.array([np.asarray(m).size for m in meshes], dtype=np.int32)
        if (self.sizes < 4).any():
            raise ValueError("every spot mesh needs at least 4 points")
        self.p_off = np.concatenate([[0], np.cumsum(self.sizes.astype(np.int64))]).astype(np.int64)
        self.total_points = int(self.p_off[-1])
        dev = self.device
        self.spots = torch.as_tensor(np.concatenate([np.asarray(m, np.float64) for m in meshes]),
                                     device=dev)
        self.params = torch.as_tensor(np.array([bs_params(o) for o in options],
                                               dtype=np.float64).reshape(n, 2), device=dev)
        self.dt = torch.as_tensor(np.broadcast_to(np.asarray(dt, dtype=np.float64), (n,)).copy(),
                                  device=dev)
        self.stream = stream if stream is not None else torch.cuda.current_stream(dev)
        if scheme not in SCHEMES:
            raise ValueError("unknown scheme %r" % (scheme,))
        self._n_host = self.sizes.copy()
        self.struct = _lib.BsBatch(n, SCHEMES[scheme], int(n_steps), int(implicit_steps),
                                   float(theta), float(implicit_dt_factor),
                                   self._n_host.ctypes.data, self.spots.data_ptr(),
                                   self.params.data_ptr(), self.dt.data_ptr(), int(prefetch), 0)
        nbytes = _lib.load().fdadi_bs_workspace_bytes(ctypes.byref(self.struct))
        if nbytes < 0:
            raise ValueError("bad batch: " + _lib.last_error())
        self.workspace_bytes = int(nbytes)
        self.workspace = torch.empty(self.workspace_bytes, dtype=torch.uint8, device=dev)
        self._prepare()

    @classmethod
    def from_options(cls, options, nspots=100, spot_max=1500.0, spotdensity=7.0,
                     force_exact=True, **kw):
        """Meshes as the reference engine builds them (blackscholes.py:181-183):
        sinh meshes on [0, ~spot_max] clustered at each option's spot."""
        ns = np.broadcast_to(np.asarray(nspots), (len(options),))
        meshes = [_mesh.sinh_space(o.spot, spot_max, spotdensity, int(k), force_exact=force_exact)
                  for o, k in zip(options, ns)]
        return cls(options, meshes, **kw), meshes

    def _sptr(self):
        return ctypes.c_void_p(self.stream.cuda_stream)

    def _ws(self):
        return ctypes.c_void_p(self.workspace.data_ptr())

    def _prepare(self):
        with torch.cuda.stream(self.stream):
            _lib.call("fdadi_bs_prepare", ctypes.byref(self.struct), self._ws(),
                      self.workspace_bytes, self._sptr())

    def _check_state(self, V):
        if (V.dtype != torch.float64 or not V.is_cuda or V.numel() != self.total_points
                or not V.is_contiguous()):
            raise ValueError("state must be a contiguous CUDA float64 tensor of %d points"
                             % self.total_points)

    def pack(self, grids):
        """Host grids (one 1-D array per option) -> device state."""
        flat = np.concatenate([np.asarray(g, dtype=np.float64).reshape(-1) for g in grids])
        if flat.size != self.total_points:
            raise ValueError("Dimension mismatch: %d grid points for a %d-point batch"
                             % (flat.size, self.total_points))
        return torch.as_tensor(flat, device=self.device)

    def unpack(self, V):
        h = V.detach().cpu().numpy()
        return [h[self.p_off[k]:self.p_off[k + 1]].copy() for k in range(self.n)]

    def run(self, V):
        """Advance the packed state V (device, float64) in place: one launch."""
        self._check_state(V)
        self.stream.wait_stream(torch.cuda.current_stream(self.device))
        _lib.call("fdadi_bs_run", ctypes.byref(self.struct), self._ws(), self.workspace_bytes,
                  ctypes.c_void_p(V.data_ptr()), self._sptr())
        torch.cuda.current_stream(self.device).wait_stream(self.stream)
        return V

    def solve(self, grids):
        """Host grids in, host grids out."""
        V = self.pack(grids)
        self.run(V)
        return self.unpack(V)

    def payoff(self, strikes, V=None, put=False):
        """Initial state max(S - K, 0) (or max(K - S, 0)) built on the device;
        strikes: device float64 [n]."""
        if (strikes.dtype != torch.float64 or not strikes.is_cuda or strikes.numel() != self.n
                or not strikes.is_contiguous()):
            raise ValueError("strikes must be a contiguous CUDA float64 tensor of %d values"
                             % self.n)
        if V is None:
            V = torch.empty(self.total_points, dtype=torch.float64, device=self.device)
        self._check_state(V)
        _lib.call("fdadi_bs_payoff", ctypes.byref(self.struct), self._ws(), self.workspace_bytes,
                  ctypes.c_void_p(strikes.data_ptr()), 1 if put else 0,
                  ctypes.c_void_p(V.data_ptr()),
                  ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream))
        return V

    def flat_index(self, spots=None):
        """State index of each option's price point: the mesh point nearest its
        spot (blackscholes.py:222-228, argmin |S - spot|)."""
        if spots is None:
            spots = [o.spot for o in self.options]
        S = self.spots.cpu().numpy()
        idx = np.array([self.p_off[k] + int(np.argmin(np.abs(S[self.p_off[k]:self.p_off[k + 1]]
                                                              - spots[k])))
                        for k in range(self.n)], dtype=np.int64)
        return torch.as_tensor(idx, device=self.device)

    def gather(self, V, flat_idx, out=None):
        """V[flat_idx] on the device (the price read-out)."""
        self._check_state(V)
        HestonBatch._check_index(flat_idx)
        if out is None:
            out = torch.empty(flat_idx.numel(), dtype=torch.float64, device=self.device)
        _lib.call("fdadi_gather", ctypes.c_void_p(V.data_ptr()),
                  ctypes.c_void_p(flat_idx.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                  flat_idx.numel(),
                  ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream))
        return out

    def status(self, V):
        """Per-option status words (numpy int32), as HestonBatch.status."""
        self._check_state(V)
        out = torch.empty(self.n, dtype=torch.int32, device=self.device)
        with torch.cuda.stream(self.stream):
            _lib.call("fdadi_bs_status", ctypes.byref(self.struct), self._ws(),
                      self.workspace_bytes, ctypes.c_void_p(V.data_ptr()),
                      ctypes.c_void_p(out.data_ptr()), self._sptr())
        self.stream.synchronize()
        return out.cpu().numpy()

    def price_calls(self, spot, strikes, params, dt, put=False, spot_max=1500.0,
                    spotdensity=7.0, force_exact=True):
        """Price a new set of options on this batch's mesh sizes, from their
        parameters (host arrays in, host prices out), as the reference engine
        does per option (blackscholes.py:181-183 builds the mesh, :222-232
        reads the price): the sinh meshes (one per distinct spot and size),
        the copies to the device, the operator build, payoff, run and price
        read-out. spot: scalar or [n]; strikes, dt: [n]; params: [n, 2] of
        (r, variance). Returns a numpy array of n prices."""
        n = self.n
        strikes = np.ascontiguousarray(strikes, dtype=np.float64).reshape(-1)
        if strikes.size != n:
            raise ValueError("need %d strikes, got %d" % (n, strikes.size))
        spot = np.broadcast_to(np.asarray(spot, dtype=np.float64), (n,))
        params = np.ascontiguousarray(params, dtype=np.float64).reshape(n, 2)
        dt = np.broadcast_to(np.asarray(dt, dtype=np.float64), (n,))
        if not hasattr(self, "_h"):
            pin = lambda t: t.pin_memory()
            self._h = dict(spots=pin(torch.empty(self.total_points, dtype=torch.float64)),
                           params=pin(torch.empty(2 * n, dtype=torch.float64)),
                           dt=pin(torch.empty(n, dtype=torch.float64)),
                           K=pin(torch.empty(n, dtype=torch.float64)),
                           idx=pin(torch.empty(n, dtype=torch.int64)),
                           prices=pin(torch.empty(n, dtype=torch.float64)))
            self._d = dict(K=torch.empty(n, dtype=torch.float64, device=self.device),
                           idx=torch.empty(n, dtype=torch.int64, device=self.device),
                           prices=torch.empty(n, dtype=torch.float64, device=self.device),
                           V=torch.empty(self.total_points, dtype=torch.float64,
                                         device=self.device))
        h, d = self._h, self._d
        idx = bs_meshes_batch(spot, self.sizes, spot_max, spotdensity, force_exact,
                              out=h["spots"].numpy())
        h["params"].numpy()[:] = params.reshape(-1)
        h["dt"].numpy()[:] = dt
        h["K"].numpy()[:] = strikes
        h["idx"].numpy()[:] = idx
        with torch.cuda.stream(self.stream):
            self.stream.wait_stream(torch.cuda.current_stream(self.device))
            self.spots.copy_(h["spots"], non_blocking=True)
            self.params.view(-1).copy_(h["params"], non_blocking=True)
            self.dt.copy_(h["dt"], non_blocking=True)
            d["K"].copy_(h["K"], non_blocking=True)
            d["idx"].copy_(h["idx"], non_blocking=True)
            self._prepare()
            self.payoff(d["K"], d["V"], put=put)
            self.run(d["V"])
            self.gather(d["V"], d["idx"], d["prices"])
            h["prices"].copy_(d["prices"], non_blocking=True)
        self.stream.synchronize()
        return h["prices"].numpy().copy()

    @property
    def price_calls_h2d_bytes(self):
        """Host-to-device bytes one price_calls() copies."""
        return 8 * (self.total_points + 2 * self.n + 3 * self.n)
