"""ctypes binding of include/dyn.h (libdynamite_gb300.so, built in-tree).

The library is the product: there is no Python or CPU fallback for any call
that needs it, and loading fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
i64p = C.POINTER(C.c_int64)
szp = C.POINTER(C.c_size_t)

DYN_OK = 0
DYN_RK54, DYN_SSPRK104 = 1, 2
DYN_FP64, DYN_MIXED = 0, 1
DYN_SEARCH_BINARY, DYN_SEARCH_LOWER_BOUND = 0, 1
DYN_SPARSIFY_CPU, DYN_SPARSIFY_CUDA_HOST, DYN_SPARSIFY_GPU = 0, 1, 2
DYN_RINT, DYN_POSB1X, DYN_POSB2X = 16, 17, 18


class Config(C.Structure):
    _fields_ = [
        ("p", C.c_int), ("p2", C.c_int), ("lam", C.c_double), ("T0", C.c_double), ("Gamma", C.c_double),
        ("len", C.c_size_t), ("depth", C.c_size_t), ("delta_t_min", C.c_double), ("delta_max", C.c_double),
        ("precision", C.c_int), ("search", C.c_int), ("history_capacity", C.c_size_t), ("device", C.c_int),
        ("stream", C.c_void_p), ("use_graph", C.c_int), ("log_response", C.c_int),
    ]


class Tables(C.Structure):
    _fields_ = [
        ("theta", dp), ("phi2", dp), ("integ", dp),
        ("indsA1y", i64p), ("indsA2y", i64p), ("indsB2y", i64p),
        ("weightsA1y", dp), ("weightsA2y", dp), ("weightsB2y", dp),
    ]


class StateC(C.Structure):
    _fields_ = [
        ("n", C.c_size_t), ("t1grid", dp), ("delta_t_ratio", dp), ("QK", dp), ("QR", dp), ("dQK", dp),
        ("dQR", dp), ("rvec", dp), ("drvec", dp),
    ]


class Controller(C.Structure):
    _fields_ = [("delta_t", C.c_double), ("delta", C.c_double), ("delta_old", C.c_double), ("loop", C.c_int),
                ("method", C.c_int)]


class StepResult(C.Structure):
    _fields_ = [("delta", C.c_double), ("t", C.c_double), ("r", C.c_double), ("energy", C.c_double),
                ("qk0", C.c_double), ("dr", C.c_double)]


class RunParams(C.Structure):
    _fields_ = [
        ("nsteps", C.c_int), ("tmax", C.c_double), ("dt_schedule", dp), ("method_schedule", ip),
        ("gpu_rollback", C.c_int), ("out_dt", dp), ("out_method", ip), ("out_delta", dp), ("out_t", dp),
        ("out_energy", dp), ("out_qk0", dp), ("out_r", dp),
        ("sparsify_every", C.c_longlong), ("sparsify_sweeps", C.c_int), ("sparsify_variant", C.c_int),
        ("tail_fit", C.c_int), ("use_serk2", C.c_int),
    ]


class TailInfo(C.Structure):
    _fields_ = [("alpha_raw", C.c_double), ("alpha", C.c_double), ("j0", C.c_int), ("applied", C.c_int)]


class NoAllocRHS(C.Structure):
    """dyn_noalloc_rhs: every pointer is a device address owned by the caller."""

    _fields_ = [
        ("p", C.c_int), ("p2", C.c_int), ("lam", C.c_double), ("T0", C.c_double), ("Gamma", C.c_double),
        ("len", C.c_size_t), ("depth", C.c_size_t), ("rows", C.c_size_t), ("search", C.c_int),
        ("theta", C.c_void_p), ("phi2", C.c_void_p), ("integ", C.c_void_p),
        ("indsA1y", C.c_void_p), ("indsA2y", C.c_void_p), ("indsB2y", C.c_void_p),
        ("weightsA1y", C.c_void_p), ("weightsA2y", C.c_void_p), ("weightsB2y", C.c_void_p),
        ("KR", C.c_void_p), ("dKR", C.c_void_p), ("t1grid", C.c_void_p), ("delta_t_ratio", C.c_void_p),
        ("rvec", C.c_void_p), ("drvec", C.c_void_p), ("out", C.c_void_p),
    ]


class BatchGrid(C.Structure):
    _fields_ = [("len", C.c_size_t), ("depth", C.c_size_t), ("tables", Tables)]


class BatchQuench(C.Structure):
    _fields_ = [
        ("grid", C.c_int), ("p", C.c_int), ("p2", C.c_int), ("lam", C.c_double), ("T0", C.c_double),
        ("Gamma", C.c_double), ("delta_t_min", C.c_double), ("delta_max", C.c_double), ("delta_t", C.c_double),
        ("t_stop", C.c_double), ("max_steps", C.c_longlong), ("capacity", C.c_size_t),
    ]


class BatchConfig(C.Structure):
    _fields_ = [
        ("device", C.c_int), ("stream", C.c_void_p), ("search", C.c_int), ("gpu_rollback", C.c_int),
        ("ticks_per_launch", C.c_int), ("threads", C.c_int), ("targets", C.c_int), ("ctas_per_sm", C.c_int),
        ("sparsify_every", C.c_longlong), ("sparsify_sweeps", C.c_int), ("sparsify_variant", C.c_int),
        ("precision", C.c_int), ("use_serk2", C.c_int),
    ]


class BatchInfo(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("method", C.c_int), ("loop", C.c_int), ("pad", C.c_int), ("steps", C.c_longlong),
        ("n", C.c_size_t), ("t", C.c_double), ("delta_t", C.c_double), ("delta", C.c_double),
        ("delta_old", C.c_double), ("energy", C.c_double), ("r", C.c_double), ("qk0", C.c_double),
    ]


class AdjointObjective(C.Structure):
    _fields_ = [("w_energy", C.c_double), ("w_r", C.c_double), ("c_K", dp), ("c_R", dp), ("c_dK", dp),
                ("c_dR", dp), ("w_dr", C.c_double)]


class AdjointStats(C.Structure):
    _fields_ = [("ms_forward", C.c_double), ("ms_backward", C.c_double), ("device_bytes", C.c_size_t),
                ("steps", C.c_int), ("recompute_mismatch", C.c_longlong)]


DYN_QUENCH_RUNNING, DYN_QUENCH_DONE, DYN_QUENCH_MAXSTEPS, DYN_QUENCH_FULL = 0, 1, 2, 3

_lib = None


class StateDev(C.Structure):
    """dyn_state_dev: the history in the reference's device layout (device pointers)."""

    _fields_ = [("n", C.c_size_t)] + [(f, C.c_void_p) for f in ("t1grid", "delta_t_ratio", "QK", "QR", "dQK", "dQR",
                                                                 "rvec", "drvec")]


class DynError(RuntimeError):
    """A dyn_status other than DYN_OK; `status` holds the code."""

    def __init__(self, msg: str, status: int = 0):
        super().__init__(msg)
        self.status = status


DYN_ERR_INVALID, DYN_ERR_CUDA, DYN_ERR_NOMEM, DYN_ERR_STATE, DYN_ERR_UNSUPPORTED, DYN_ERR_NONFINITE = (
    -1, -2, -3, -4, -5, -6)


def lib():
    """Load the native library; raise if it is missing (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise DynError(f"{LIB_PATH} is missing: build it with `python -m dynamite_gb300.build`")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        sigs = {
            "dyn_abi_version": ([], C.c_int),
            "dyn_energy_history": ([vp, dp, C.c_size_t], C.c_int),
            "dyn_tail_fit": ([vp, C.c_int, C.POINTER(TailInfo)], C.c_int),
            "dyn_tail_fit_reset": ([vp], C.c_int),
            "dyn_last_error": ([], C.c_char_p),
            "dyn_ctx_create": ([C.POINTER(Config), C.POINTER(Tables), C.POINTER(vp)], C.c_int),
            "dyn_check_tables": ([C.c_size_t, C.c_size_t, C.POINTER(Tables)], C.c_int),
            "dyn_ctx_destroy": ([vp], C.c_int),
            "dyn_sync": ([vp], C.c_int),
            "dyn_state_init": ([vp, C.c_double], C.c_int),
            "dyn_state_upload": ([vp, C.POINTER(StateC)], C.c_int),
            "dyn_state_rows": ([vp, szp], C.c_int),
            "dyn_state_time": ([vp, dp], C.c_int),
            "dyn_state_download": ([vp, C.POINTER(StateC)], C.c_int),
            "dyn_controller_get": ([vp, C.POINTER(Controller)], C.c_int),
            "dyn_controller_set": ([vp, C.POINTER(Controller)], C.c_int),
            "dyn_interpolate": ([vp, dp, dp], C.c_int),
            "dyn_get_interp": ([vp, C.c_int, dp], C.c_int),
            "dyn_qkr_step": ([vp, dp, dp], C.c_int),
            "dyn_rhs": ([vp, dp, dp], C.c_int),
            "dyn_rstep": ([vp, dp], C.c_int),
            "dyn_drstep2": ([vp, dp, dp, dp, dp, C.c_double, dp], C.c_int),
            "dyn_energy": ([vp, dp], C.c_int),
            "dyn_conv_dev": ([vp, C.c_int, vp, vp, C.c_size_t, C.c_double, vp], C.c_int),
            "dyn_search_dev": ([vp, vp, C.c_size_t, vp, C.c_size_t, vp], C.c_int),
            "dyn_update": ([vp, C.c_int, C.c_double, C.POINTER(StepResult)], C.c_int),
            "dyn_run": ([vp, C.POINTER(RunParams), C.POINTER(StepResult)], C.c_int),
            "dyn_sparsify": ([vp, C.c_double, C.c_int, szp], C.c_int),
            "dyn_rollback": ([vp, C.c_int], C.c_int),
            "dyn_last_row": ([vp, dp, dp], C.c_int),
            "dyn_profile_stage": ([vp, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)], C.c_int),
            "dyn_probe_fp64": ([C.c_int, dp], C.c_int),
            "dyn_rhs_noalloc": ([C.POINTER(NoAllocRHS), vp], C.c_int),
            "dyn_state_upload_dev": ([vp, C.POINTER(StateDev)], C.c_int),
            "dyn_state_rows_load_dev": ([vp, C.c_size_t, C.c_size_t, C.POINTER(StateDev)], C.c_int),
            "dyn_state_rows_store_dev": ([vp, C.c_size_t, C.c_size_t, C.POINTER(StateDev)], C.c_int),
            "dyn_get_interp_dev": ([vp, C.c_int, vp], C.c_int),
            "dyn_interp_b1_dev": ([vp, vp, vp], C.c_int),
            "dyn_batch_create": ([C.POINTER(BatchConfig), C.POINTER(BatchGrid), C.c_int, C.POINTER(BatchQuench),
                                  C.c_int, C.POINTER(vp)], C.c_int),
            "dyn_batch_destroy": ([vp], C.c_int),
            "dyn_batch_upload": ([vp, C.c_int, C.POINTER(StateC), C.POINTER(Controller)], C.c_int),
            "dyn_batch_download": ([vp, C.c_int, C.POINTER(StateC)], C.c_int),
            "dyn_batch_get_info": ([vp, C.c_int, C.POINTER(BatchInfo)], C.c_int),
            "dyn_batch_set_limits": ([vp, C.c_int, C.c_double, C.c_longlong], C.c_int),
            "dyn_batch_run": ([vp, C.c_longlong, C.POINTER(C.c_longlong)], C.c_int),
            "dyn_batch_enqueue": ([vp, C.c_longlong], C.c_int),
            "dyn_batch_sync": ([vp], C.c_int),
            "dyn_batch_last_row": ([vp, C.c_int, dp, dp], C.c_int),
            "dyn_batch_tune": ([vp, C.c_int, ip, ip, ip, C.POINTER(C.c_float)], C.c_int),
            "dyn_batch_profile": ([vp, C.c_int, C.POINTER(C.c_float)], C.c_int),
            "dyn_adjoint_forward": ([vp, C.POINTER(RunParams), C.POINTER(StepResult)], C.c_int),
            "dyn_adjoint_backward": ([vp, C.POINTER(AdjointObjective), dp, C.POINTER(AdjointStats)], C.c_int),
            "dyn_adjoint_history_grad": ([vp, C.POINTER(StateC)], C.c_int),
            "dyn_grid_generate": ([C.c_size_t, C.c_double, C.c_int, C.c_int, C.c_double, C.c_double, dp, dp, dp,
                                   dp, i64p, dp, i64p, dp, i64p, dp], C.c_int),
            "dyn_grid_rational_depth": ([C.c_size_t, C.c_int, C.c_int], C.c_int),
            "dyn_grid_positions": ([C.c_size_t, C.c_double, C.c_double, C.c_double, dp, dp, dp], C.c_int),
            "dyn_grid_generate_rational": ([C.c_size_t, C.c_double, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                            dp, dp, dp, dp, i64p, dp, i64p, dp, i64p, dp], C.c_int),
        }
        for name, (args, res) in sigs.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def check(status: int, what: str = "") -> None:
    if status != DYN_OK:
        msg = lib().dyn_last_error().decode(errors="replace")
        raise DynError(f"{what} failed (status {status}): {msg}", status)


def ptr(a):
    return None if a is None else a.ctypes.data_as(dp)
