"""ctypes binding of libfdadi.so (the C ABI in include/fdadi.h).

The library is the only compute path: if it cannot be loaded the import of
any op raises, there is no fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfdadi.so")

FDADI_CANNOT_FOLD, FDADI_CAN_FOLD, FDADI_FOLDED = 0, 1, 2
FOLD_CODES = {"CANNOT_FOLD": 0, "CAN_FOLD": 1, "FOLDED": 2}
FOLD_NAMES = {v: k for k, v in FOLD_CODES.items()}
SCHEME_IMPLICIT, SCHEME_DOUGLAS, SCHEME_HV, SCHEME_CS, SCHEME_MCS = 0, 1, 2, 3, 4
HESTON_DROP_ZERO_MIXED, HESTON_GRAPH = 1, 2
NOALLOC_MAX_ROWS = 1 << 20

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int32_p = ctypes.POINTER(ctypes.c_int32)
c_int64_p = ctypes.POINTER(ctypes.c_int64)


class Tri(ctypes.Structure):
    """fdadi_tri_t"""
    _fields_ = [("operator_rows", ctypes.c_int64), ("blocks", ctypes.c_int64),
                ("axis", ctypes.c_int32), ("has_residual", ctypes.c_int32),
                ("has_low_dirichlet", ctypes.c_int32), ("has_high_dirichlet", ctypes.c_int32),
                ("top_fold_status", ctypes.c_int32), ("bottom_fold_status", ctypes.c_int32),
                ("sup", ctypes.c_void_p), ("mid", ctypes.c_void_p), ("sub", ctypes.c_void_p),
                ("R", ctypes.c_void_p), ("low_dirichlet", ctypes.c_void_p),
                ("high_dirichlet", ctypes.c_void_p), ("top_factors", ctypes.c_void_p),
                ("bottom_factors", ctypes.c_void_p), ("sup2", ctypes.c_void_p),
                ("sub2", ctypes.c_void_p)]


class Mixed(ctypes.Structure):
    """fdadi_mixed_t"""
    _fields_ = [("n0", ctypes.c_int64), ("n1", ctypes.c_int64),
                ("has_residual", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("coeff", ctypes.c_void_p), ("w0", ctypes.c_void_p), ("w1", ctypes.c_void_p),
                ("R", ctypes.c_void_p)]


STATUS_PIVOT = 1        # a line-solve pivot was zero or non-finite
STATUS_NONFINITE = 2    # the option's grid holds a NaN or infinity


class MlpNet(ctypes.Structure):
    """fdadi_mlp_net_t"""
    _fields_ = [("W", ctypes.c_void_p * 5), ("b", ctypes.c_void_p * 5),
                ("K", ctypes.c_int32 * 5), ("N", ctypes.c_int32 * 5),
                ("members", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class HestonPlan(ctypes.Structure):
    """fdadi_heston_plan_t"""
    _fields_ = [("spot_kind", ctypes.c_int32), ("spot_a", ctypes.c_int32),
                ("spot_b", ctypes.c_int32), ("var_kind", ctypes.c_int32),
                ("var_warps", ctypes.c_int32), ("groups", ctypes.c_int32),
                ("expl_per_sm", ctypes.c_int32), ("reserved", ctypes.c_int32 * 1)]

    FIELDS = ("spot_kind", "spot_a", "spot_b", "var_kind", "var_warps", "groups", "expl_per_sm")

    def as_dict(self):
        return {k: int(getattr(self, k)) for k in self.FIELDS}

    @classmethod
    def from_dict(cls, d):
        return cls(*[int(d.get(k, 1 if k == "groups" else 0)) for k in cls.FIELDS])


class HestonBatch(ctypes.Structure):
    """fdadi_heston_batch_t"""
    _fields_ = [("n_options", ctypes.c_int32), ("scheme", ctypes.c_int32),
                ("n_steps", ctypes.c_int32), ("implicit_steps", ctypes.c_int32),
                ("theta", ctypes.c_double), ("implicit_dt_factor", ctypes.c_double),
                ("flags", ctypes.c_int32),
                ("reserved", ctypes.c_int32),
                ("n0", ctypes.c_void_p), ("n1", ctypes.c_void_p),
                ("spots", ctypes.c_void_p), ("vars", ctypes.c_void_p),
                ("params", ctypes.c_void_p), ("dt", ctypes.c_void_p),
                ("barrier", ctypes.c_void_p), ("plan", ctypes.c_void_p),
                ("rates", ctypes.c_void_p)]


class BsBatch(ctypes.Structure):
    """fdadi_bs_batch_t"""
    _fields_ = [("n_options", ctypes.c_int32), ("scheme", ctypes.c_int32),
                ("n_steps", ctypes.c_int32), ("implicit_steps", ctypes.c_int32),
                ("theta", ctypes.c_double), ("implicit_dt_factor", ctypes.c_double),
                ("n", ctypes.c_void_p), ("spots", ctypes.c_void_p),
                ("params", ctypes.c_void_p), ("dt", ctypes.c_void_p),
                ("prefetch", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Gemm(ctypes.Structure):
    """fdadi_gemm_t"""
    _fields_ = [("A", ctypes.c_void_p), ("lda", ctypes.c_int64), ("strideA", ctypes.c_int64),
                ("B", ctypes.c_void_p), ("ldb", ctypes.c_int64), ("strideB", ctypes.c_int64),
                ("bias", ctypes.c_void_p), ("strideBias", ctypes.c_int64),
                ("aux", ctypes.c_void_p), ("ldaux", ctypes.c_int64), ("strideAux", ctypes.c_int64),
                ("out_f32", ctypes.c_void_p), ("ldo", ctypes.c_int64), ("strideO", ctypes.c_int64),
                ("out_bf16", ctypes.c_void_p), ("ldh", ctypes.c_int64), ("strideH", ctypes.c_int64),
                ("M", ctypes.c_int32), ("N", ctypes.c_int32), ("K", ctypes.c_int32),
                ("act", ctypes.c_int32), ("problems", ctypes.c_int32), ("variant", ctypes.c_int32),
                ("status", ctypes.c_void_p), ("wait_cycles", ctypes.c_int64)]


# name -> (restype, argtypes); every symbol include/fdadi.h declares
SIGNATURES = {
    "fdadi_version": (ctypes.c_int, []),
    "fdadi_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "fdadi_exponential_space": (ctypes.c_int, [ctypes.c_double, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                               ctypes.c_int32, ctypes.c_void_p]),
    "fdadi_heston_var_meshes": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                               ctypes.c_int32, ctypes.c_void_p]),
    "fdadi_tri_apply": (ctypes.c_int, [ctypes.POINTER(Tri), ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]),
    "fdadi_tri_solve": (ctypes.c_int, [ctypes.POINTER(Tri), ctypes.c_void_p, ctypes.c_int64,
                                       ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]),
    "fdadi_tri_solve_noalloc": (ctypes.c_int, [ctypes.POINTER(Tri), ctypes.c_void_p,
                                               ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]),
    "fdadi_tri_scale": (ctypes.c_int, [ctypes.POINTER(Tri), ctypes.c_void_p, ctypes.c_double,
                                       ctypes.c_void_p]),
    "fdadi_tri_add_scalar": (ctypes.c_int, [ctypes.POINTER(Tri), ctypes.c_double,
                                            ctypes.c_void_p]),
    "fdadi_tri_add_operator": (ctypes.c_int, [ctypes.POINTER(Tri), ctypes.POINTER(Tri),
                                              ctypes.c_void_p]),
    "fdadi_tri_fold": (ctypes.c_int, [ctypes.POINTER(Tri), ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_void_p]),
    "fdadi_mixed_apply": (ctypes.c_int, [ctypes.POINTER(Mixed), ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p]),
    "fdadi_mixed_scale": (ctypes.c_int, [ctypes.POINTER(Mixed), ctypes.c_void_p, ctypes.c_double,
                                         ctypes.c_void_p]),
    "fdadi_axpby": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_int64, ctypes.c_void_p]),
    "fdadi_heston_workspace_bytes": (ctypes.c_int64, [ctypes.POINTER(HestonBatch)]),
    "fdadi_heston_prepare": (ctypes.c_int, [ctypes.POINTER(HestonBatch), ctypes.c_void_p,
                                            ctypes.c_int64, ctypes.c_void_p]),
    "fdadi_heston_run": (ctypes.c_int, [ctypes.POINTER(HestonBatch), ctypes.c_void_p,
                                        ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]),
    "fdadi_gather": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_int64, ctypes.c_void_p]),
    "fdadi_heston_launch_count": (ctypes.c_int64, [ctypes.POINTER(HestonBatch)]),
    "fdadi_heston_tune": (ctypes.c_int, [ctypes.POINTER(HestonBatch), ctypes.c_void_p,
                                         ctypes.c_int64, ctypes.c_int32,
                                         ctypes.POINTER(HestonPlan), ctypes.c_void_p]),
    "fdadi_heston_default_plan": (ctypes.c_int, [ctypes.POINTER(HestonBatch),
                                                 ctypes.POINTER(HestonPlan)]),
    "fdadi_mlp_infer": (ctypes.c_int, [ctypes.POINTER(MlpNet), ctypes.c_void_p, ctypes.c_int32,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fdadi_heston_greeks": (ctypes.c_int, [ctypes.POINTER(HestonBatch), ctypes.c_void_p,
                                           ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    "fdadi_heston_payoff": (ctypes.c_int, [ctypes.POINTER(HestonBatch), ctypes.c_void_p,
                                           ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32,
                                           ctypes.c_void_p, ctypes.c_void_p]),
    "fdadi_heston_status": (ctypes.c_int, [ctypes.POINTER(HestonBatch), ctypes.c_void_p,
                                           ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    "fdadi_bs_workspace_bytes": (ctypes.c_int64, [ctypes.POINTER(BsBatch)]),
    "fdadi_bs_prepare": (ctypes.c_int, [ctypes.POINTER(BsBatch), ctypes.c_void_p,
                                        ctypes.c_int64, ctypes.c_void_p]),
    "fdadi_bs_run": (ctypes.c_int, [ctypes.POINTER(BsBatch), ctypes.c_void_p, ctypes.c_int64,
                                    ctypes.c_void_p, ctypes.c_void_p]),
    "fdadi_bs_payoff": (ctypes.c_int, [ctypes.POINTER(BsBatch), ctypes.c_void_p,
                                       ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32,
                                       ctypes.c_void_p, ctypes.c_void_p]),
    "fdadi_bs_status": (ctypes.c_int, [ctypes.POINTER(BsBatch), ctypes.c_void_p,
                                       ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p]),
    "fdadi_heston_stage": (ctypes.c_int, [ctypes.POINTER(HestonBatch), ctypes.c_void_p,
                                          ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32,
                                          ctypes.c_void_p]),
    "fdadi_mlp_gemm": (ctypes.c_int, [ctypes.POINTER(Gemm), ctypes.c_void_p]),
    "fdadi_transpose_bf16": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                            ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                            ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.c_void_p]),
    "fdadi_mlp_mse": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                     ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                     ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                     ctypes.c_void_p, ctypes.c_void_p]),
    "fdadi_mlp_colsum": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                        ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "fdadi_mlp_adam": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float, ctypes.c_float, ctypes.c_int32,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fdadi_mlp_featurize": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fdadi_mlp_combine": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                         ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]),
    "fdadi_fp64_probe": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_int32,
                                        ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]),
}

STAGE = {"explicit_douglas": 0, "explicit_hv0": 1, "explicit_hv3": 2, "explicit_implicit": 3,
         "spot_solve": 4, "var_solve_y2": 5, "var_solve_v": 6, "var_solve_implicit": 7,
         "spot_solve_implicit": 8}

_lib = None


def load(build_if_missing=True):
    """Load libfdadi.so (building it first if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        from . import build as _build
        if _build.stale():
            _build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libfdadi.so is not built (%s); run fd_adi_gb300.build.build()"
                           % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    buf = ctypes.create_string_buffer(1024)
    load().fdadi_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


class FdadiError(RuntimeError):
    pass


def check(rc, what=""):
    """Raise for a nonzero status: ValueError for argument/shape errors (the
    reference surfaces its DIE() messages as ValueError through `except +`),
    RuntimeError otherwise."""
    if rc == 0:
        return
    msg = last_error()
    if rc == 1:
        raise ValueError("%s%s" % (what + ": " if what else "", msg))
    raise FdadiError("%s%s (code %d)" % (what + ": " if what else "", msg, rc))


def call(name, *args):
    rc = getattr(load(), name)(*args)
    check(rc, name)
    return rc
