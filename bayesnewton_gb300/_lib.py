"""ctypes binding of libbnx.so (the C ABI declared in include/bnx.h).

The library is the only compute path: if it is missing or cannot be loaded, every
entry point raises; there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbnx.so")

MAX_COMPONENTS = 8
MAX_STATE = 8
MAX_CUB = 32

KIND_MATERN12, KIND_MATERN32, KIND_MATERN52, KIND_MATERN72, KIND_FEEDBACK = 1, 2, 3, 4, 5
COMBINE_SUM, COMBINE_INDEPENDENT = 0, 1
LIK_GAUSSIAN, LIK_BERNOULLI_LOGIT, LIK_BERNOULLI_PROBIT, LIK_POISSON_EXP = 1, 2, 3, 4
LIK_HETERO_EXP, LIK_HETERO_SOFTPLUS = 5, 6
METHOD_VI, METHOD_NEWTON, METHOD_EP, METHOD_PL = 0, 1, 2, 3
DTYPE_F32, DTYPE_F64 = 0, 1
OK, ERR_ARG, ERR_UNSUPPORTED, ERR_CUDA = 0, -1, -2, -3
STATUS_NONPD, STATUS_SINGULAR, STATUS_SITE_KEPT, STATUS_SITE_CLAMPED = 1, 2, 4, 8
RES_ENERGY, RES_LOGLIK, RES_SUM1, RES_SUM2, RES_DIFF1, RES_DIFF2 = 0, 1, 2, 3, 4, 5
RES_SURR_PSD, RES_SURR_SPOT = 6, 7
NRESULT = 8

EXPORTS = ("bn_model_create", "bn_model_destroy", "bn_model_set_prior", "bn_model_set_likelihood",
           "bn_model_info", "bn_update_posterior", "bn_newton_step", "bn_model_result",
           "bn_kalman_filter", "bn_rts_smoother", "bn_model_set_series", "bn_model_series_energy",
           "bn_model_set_profiling", "bn_model_kernel_times",
           "bn_mlp_create", "bn_mlp_destroy", "bn_mlp_num_params", "bn_mlp_set_params", "bn_mlp_get_params",
           "bn_mlp_prepare", "bn_mlp_sites", "bn_mlp_forward", "bn_mlp_loss_grad", "bn_mlp_train", "bn_model_set_surrogate",
           "bn_dense_gemm", "bn_dense_inverse", "bn_model_set_segment", "bn_model_element_sizes", "bn_segment_step", "bn_segment_filter_state",
           "bn_segment_smoother_state",
           "bn_st_create", "bn_st_destroy", "bn_st_set_prior", "bn_st_set_likelihood", "bn_st_update_posterior",
           "bn_st_newton_step", "bn_st_result", "bn_st_latent_posterior", "bn_st_set_profiling", "bn_st_step_time",
           "bn_temporal_conditional", "bn_model_predict", "bn_model_log_density", "bn_model_predict_y",
           "bn_model_energy_grad", "bn_st_predict",
           "bn_ih_create", "bn_ih_destroy", "bn_ih_set_prior", "bn_ih_set_likelihood", "bn_ih_update_posterior",
           "bn_ih_site_update", "bn_ih_log_lik", "bn_ih_result", "bn_ih_dare_state",
           "bn_bounded_wait_probe", "bn_gauss_hermite", "bn_build_info")
KERNELS = ("filter_reduce", "filter_blocks", "filter_rerun", "smoother_blocks", "smoother_rerun", "site_tail")


class PriorDesc(ctypes.Structure):
    _fields_ = [("num_components", ctypes.c_int32), ("combine", ctypes.c_int32),
                ("kind", ctypes.c_int32 * MAX_COMPONENTS), ("size", ctypes.c_int32 * MAX_COMPONENTS),
                ("variance", ctypes.c_double * MAX_COMPONENTS), ("lengthscale", ctypes.c_double * MAX_COMPONENTS),
                ("feedback", ctypes.c_double * (MAX_STATE * MAX_STATE)),
                ("pinf", ctypes.c_double * (MAX_STATE * MAX_STATE))]


class LikDesc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("method", ctypes.c_int32), ("num_cub", ctypes.c_int32),
                ("ensure_psd", ctypes.c_int32), ("score_form", ctypes.c_int32), ("variance", ctypes.c_double),
                ("binsize", ctypes.c_double), ("power", ctypes.c_double)]


class StDesc(ctypes.Structure):
    _fields_ = [("temporal_kind", ctypes.c_int32), ("temporal_variance", ctypes.c_double),
                ("temporal_lengthscale", ctypes.c_double), ("spatial_kind", ctypes.c_int32),
                ("spatial_variance", ctypes.c_double), ("spatial_lengthscale", ctypes.c_double),
                ("num_inducing", ctypes.c_int32), ("spatial_dim", ctypes.c_int32),
                ("z", ctypes.POINTER(ctypes.c_double)), ("conditional", ctypes.c_int32)]


class SiteState(ctypes.Structure):
    _fields_ = [("nat1", ctypes.c_void_p), ("nat2", ctypes.c_void_p), ("post_mean", ctypes.c_void_p),
                ("post_var", ctypes.c_void_p), ("grad", ctypes.c_void_p), ("hess", ctypes.c_void_p),
                ("lin", ctypes.c_void_p)]


class BnError(RuntimeError):
    pass


_LIB = None


def load():
    """Load libbnx.so once.  Raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise BnError("libbnx.so is not built (run bayesnewton_gb300/build.py or __graft_entry__.build())")
    lib = ctypes.CDLL(LIB_PATH)
    vp, i32, i64, dbl = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    P = ctypes.POINTER
    lib.bn_model_create.argtypes = [P(PriorDesc), P(LikDesc), i64, i32, i32, i32, P(vp)]
    lib.bn_model_destroy.argtypes = [vp]
    lib.bn_model_set_prior.argtypes = [vp, P(PriorDesc)]
    lib.bn_model_set_likelihood.argtypes = [vp, P(LikDesc)]
    lib.bn_model_info.argtypes = [vp, P(i32), P(i32), P(i32), P(i32)]
    lib.bn_update_posterior.argtypes = [vp, vp, i32, vp, vp, P(SiteState)]
    lib.bn_newton_step.argtypes = [vp, vp, i32, dbl, vp, vp, P(SiteState)]
    lib.bn_model_result.argtypes = [vp, vp, P(dbl), P(i32)]
    lib.bn_kalman_filter.argtypes = [vp, vp, i32, i32, vp, vp, vp, vp, vp, vp]
    lib.bn_rts_smoother.argtypes = [vp, vp, i32, i32, vp, vp, vp, vp, vp, vp]
    lib.bn_model_set_series.argtypes = [vp, i64, P(ctypes.c_int64), P(dbl), P(dbl), P(i32), P(dbl)]
    lib.bn_model_series_energy.argtypes = [vp, vp, P(dbl)]
    lib.bn_model_set_profiling.argtypes = [vp, i32]
    lib.bn_model_kernel_times.argtypes = [vp, P(ctypes.c_float), i32]
    fp = P(ctypes.c_float)
    lib.bn_mlp_create.argtypes = [i32, P(vp)]
    lib.bn_mlp_destroy.argtypes = [vp]
    lib.bn_mlp_num_params.argtypes = []
    lib.bn_mlp_set_params.argtypes = [vp, fp, fp]
    lib.bn_mlp_get_params.argtypes = [vp, fp, fp]
    lib.bn_mlp_prepare.argtypes = [vp, vp, i32, i32, vp, vp, vp, vp]
    lib.bn_mlp_sites.argtypes = [vp, vp, i64, vp, vp, vp, i32, i32, dbl, i32, vp, P(ctypes.c_uint32)]
    lib.bn_mlp_forward.argtypes = [vp, vp, i32, vp, vp]
    lib.bn_mlp_loss_grad.argtypes = [vp, vp, i32, vp, vp, P(dbl), fp]
    lib.bn_mlp_train.argtypes = [vp, vp, i32, vp, vp, i32, i32, ctypes.c_float, ctypes.c_uint32, P(dbl)]
    lib.bn_model_set_surrogate.argtypes = [vp, vp, i32, dbl]
    lib.bn_bounded_wait_probe.argtypes = [vp, ctypes.c_uint32, vp]
    lib.bn_dense_gemm.argtypes = [vp, i32, i32, i32, i32, i32, i32, i32, ctypes.c_float, vp, vp, ctypes.c_float, vp,
                                  vp]
    lib.bn_dense_inverse.argtypes = [vp, i32, i32, i32, vp, vp, vp]
    lib.bn_model_set_segment.argtypes = [vp, i32, i32, dbl]
    lib.bn_model_element_sizes.argtypes = [vp, P(i32), P(i32), P(i32)]
    lib.bn_segment_step.argtypes = [vp, vp, i32, i32, dbl, vp, vp, P(SiteState), P(dbl), P(dbl)]
    lib.bn_segment_filter_state.argtypes = [i32, P(dbl), P(dbl), P(dbl)]
    lib.bn_segment_smoother_state.argtypes = [i32, P(dbl), P(dbl), P(dbl)]
    lib.bn_st_create.argtypes = [P(StDesc), P(LikDesc), i64, i32, vp, P(vp)]
    lib.bn_st_destroy.argtypes = [vp]
    lib.bn_st_set_prior.argtypes = [vp, P(StDesc)]
    lib.bn_st_set_likelihood.argtypes = [vp, P(LikDesc)]
    lib.bn_st_update_posterior.argtypes = [vp, vp, vp, vp, P(SiteState)]
    lib.bn_st_newton_step.argtypes = [vp, vp, dbl, vp, vp, P(SiteState)]
    lib.bn_st_result.argtypes = [vp, vp, P(dbl), P(i32)]
    lib.bn_st_latent_posterior.argtypes = [vp, vp, vp, vp]
    lib.bn_st_set_profiling.argtypes = [vp, i32]
    lib.bn_st_predict.argtypes = [vp, vp, vp, i64, vp, i32, vp, vp, vp]
    lib.bn_st_step_time.argtypes = [vp, P(ctypes.c_float)]
    lib.bn_temporal_conditional.argtypes = [vp, vp, vp, i64, vp, vp, vp, vp, i32, vp, vp]
    lib.bn_model_predict.argtypes = [vp, vp, i32, vp, vp, P(SiteState), vp, i64, vp, vp, vp]
    lib.bn_model_log_density.argtypes = [vp, vp, i64, vp, vp, vp, vp, P(dbl)]
    lib.bn_model_predict_y.argtypes = [vp, vp, i64, vp, vp, vp, vp]
    lib.bn_model_energy_grad.argtypes = [vp, vp, i32, vp, vp, P(SiteState), P(dbl), P(dbl)]
    lib.bn_ih_create.argtypes = [P(PriorDesc), P(LikDesc), i64, i32, i32, P(vp)]
    lib.bn_ih_destroy.argtypes = [vp]
    lib.bn_ih_set_prior.argtypes = [vp, P(PriorDesc)]
    lib.bn_ih_set_likelihood.argtypes = [vp, P(LikDesc)]
    lib.bn_ih_update_posterior.argtypes = [vp, vp, dbl, i32, vp, P(SiteState)]
    lib.bn_ih_site_update.argtypes = [vp, vp, dbl, P(SiteState)]
    lib.bn_ih_log_lik.argtypes = [vp, vp, dbl, i32, vp, P(SiteState)]
    lib.bn_ih_result.argtypes = [vp, vp, P(dbl), P(i32)]
    lib.bn_ih_dare_state.argtypes = [vp, vp, P(dbl), P(dbl)]
    lib.bn_gauss_hermite.argtypes = [i32, P(dbl), P(dbl)]
    lib.bn_build_info.argtypes = []
    lib.bn_build_info.restype = ctypes.c_char_p
    for name in EXPORTS:
        if name != "bn_build_info":
            getattr(lib, name).restype = ctypes.c_int
    lib.bn_st_destroy.restype = None
    lib.bn_mlp_destroy.restype = None
    _LIB = lib
    return lib


def check(code, what):
    if code != OK:
        names = {ERR_ARG: "invalid argument", ERR_UNSUPPORTED: "unsupported configuration", ERR_CUDA: "CUDA error"}
        raise BnError("%s failed: %s (%d)" % (what, names.get(code, "error"), code))
