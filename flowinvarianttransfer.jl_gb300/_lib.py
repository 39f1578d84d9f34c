"""ctypes binding of libfit_gb300.so (the C ABI in include/fit_gb300.h).

The library is the only compute path: there is no CPU fallback, and loading fails loudly when the
shared object is missing or does not export every declared entry point."""
from __future__ import annotations

import ctypes as C
import os

from . import _build

EXPORTS = [
    "fit_plan_create", "fit_plan_destroy", "fit_last_error", "fit_plan_set_stream", "fit_plan_info",
    "fit_launch_count", "fit_nonlinear_term", "fit_assign_shells", "fit_transfer_density",
    "fit_spectral_flux", "fit_shell_to_shell", "fit_helical_decompose", "fit_helmholtz_decompose", "fit_toroidal_poloidal_decompose",
    "fit_partial_fluxes", "fit_mode_to_mode", "fit_prof_enable", "fit_prof_read", "fit_prof_kind_name",
    "fit_coarse_graining_flux", "fit_forward_spectrum", "fit_ns_evolve", "fit_mlp_nparams", "fit_mlp_forward", "fit_mlp_status",
    "fit_mlp_train_grad", "fit_mlp_adam", "fit_gradient_model_flux", "fit_field_moments", "fit_field_compare",
    "fit_batch_create", "fit_batch_destroy", "fit_batch_add_flux", "fit_batch_run", "fit_batch_run_eager", "fit_batch_info",
    "fit_autotune_enable", "fit_autotune_clear", "fit_autotune_info", "fit_autotune_entry",
    "fit_partial_fluxes_batched", "fit_band_to_band", "fit_stress_residual",
    "fit_set_shell_index", "fit_shell_to_shell_indexed", "fit_bench_fused_pass",
]

PTR_HOST, PTR_DEVICE = 0, 1
DEALIAS = {"none": 0, "two_thirds": 1, "three_halves": 2}
S2S_PLAIN, S2S_BATCHED = 0, 1
ERRORS = {-1: "argument", -2: "size", -3: "cuda", -4: "allocation", -5: "state"}

_lib = None


class FitError(RuntimeError):
    """A failure inside libfit_gb300 (CUDA, allocation or state)."""


def _declare(lib):
    vp, i32, i64, u32, dp = C.c_void_p, C.c_int, C.c_int64, C.c_uint32, C.POINTER(C.c_double)
    lib.fit_plan_create.argtypes = [C.POINTER(vp), i32, C.POINTER(i64), i32, i32, i32, i32, i32, C.POINTER(dp)]
    lib.fit_plan_destroy.argtypes = [vp]
    lib.fit_last_error.restype = C.c_char_p
    lib.fit_last_error.argtypes = []
    lib.fit_plan_set_stream.argtypes = [vp, vp]
    lib.fit_plan_info.argtypes = [vp, C.POINTER(i64), i32]
    lib.fit_launch_count.restype = C.c_longlong
    lib.fit_launch_count.argtypes = []
    lib.fit_nonlinear_term.argtypes = [vp, vp, vp, vp, i32]
    lib.fit_assign_shells.argtypes = [vp, dp, i32, u32, i32, vp, i32]
    lib.fit_transfer_density.argtypes = [vp, i32, vp, vp, vp, i32]
    lib.fit_spectral_flux.argtypes = [vp, vp, vp, vp, dp, i32, u32, i32, i32, vp, vp, i32]
    lib.fit_shell_to_shell.argtypes = [vp, vp, vp, dp, i32, u32, i32, i32, i32, i32, vp, vp, vp, i32]
    lib.fit_set_shell_index.argtypes = [vp, vp, i32, i32]
    lib.fit_shell_to_shell_indexed.argtypes = [vp, vp, vp, i32, i32, i32, vp, vp, vp, i32]
    lib.fit_helical_decompose.argtypes = [vp, vp, vp, vp, i32]
    lib.fit_toroidal_poloidal_decompose.argtypes = [vp, vp, vp, vp, i32]
    lib.fit_helmholtz_decompose.argtypes = [vp, vp, vp, vp, i32]
    lib.fit_partial_fluxes.argtypes = [vp, vp, i32, i32, dp, i32, u32, i32, vp, i32]
    lib.fit_mode_to_mode.argtypes = [vp, vp, vp, i32, i32, vp, vp, i32]
    lib.fit_prof_enable.argtypes = [i32]
    lib.fit_prof_read.argtypes = [i32, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    lib.fit_prof_kind_name.restype = C.c_char_p
    lib.fit_prof_kind_name.argtypes = [i32]
    f32 = C.c_float
    lib.fit_coarse_graining_flux.argtypes = [vp, vp, C.c_double, i32, vp, vp, vp, dp, i32]
    lib.fit_forward_spectrum.argtypes = [vp, vp, vp, i32]
    lib.fit_ns_evolve.argtypes = [vp, vp, i32, C.c_double, C.c_double, C.c_double, C.c_double, i32]
    lib.fit_mlp_nparams.argtypes = []
    lib.fit_mlp_status.argtypes = [C.POINTER(i32)]
    lib.fit_mlp_forward.argtypes = [vp, vp, i64, i64, vp, vp, i32, C.c_double, vp, vp, vp]
    lib.fit_stress_residual.argtypes = [vp, vp, i64, i64, C.c_double, vp, vp]
    lib.fit_mlp_train_grad.argtypes = [vp, vp, vp, i64, i64, i64, vp, vp, i32, vp, vp, vp]
    lib.fit_gradient_model_flux.argtypes = [vp, i64, i64, C.c_double, vp, vp, vp]
    lib.fit_field_moments.argtypes = [vp, i64, i64, i32, vp, vp]
    lib.fit_field_compare.argtypes = [vp, vp, i64, vp, vp]
    lib.fit_batch_create.argtypes = [C.POINTER(vp), i32]
    lib.fit_batch_destroy.argtypes = [vp]
    lib.fit_batch_add_flux.argtypes = [vp, vp, vp, vp, dp, i32, u32, i32, i32, vp, vp]
    lib.fit_batch_run.argtypes = [vp, vp]
    lib.fit_batch_run_eager.argtypes = [vp, vp]
    lib.fit_batch_info.argtypes = [vp, C.POINTER(i64), i32]
    lib.fit_autotune_enable.argtypes = [i32]
    lib.fit_autotune_clear.argtypes = []
    lib.fit_autotune_info.argtypes = [C.POINTER(i64), C.POINTER(i64), dp, dp]
    lib.fit_autotune_entry.argtypes = [i64, C.POINTER(i64), dp]
    lib.fit_bench_fused_pass.argtypes = [i32, i32, C.c_longlong, i32, dp, dp]
    lib.fit_band_to_band.argtypes = [vp, vp, vp, dp, i32, C.c_double, u32, i32, i32, vp, vp, vp, i32]
    lib.fit_partial_fluxes_batched.argtypes = [vp, vp, i32, C.POINTER(i32), i32, dp, i32, u32, i32, vp, i32]
    lib.fit_mlp_adam.argtypes = [vp, vp, vp, vp, i32, f32, f32, f32, f32, vp]
    for name in EXPORTS:
        if name not in ("fit_last_error", "fit_launch_count", "fit_prof_kind_name"):
            getattr(lib, name).restype = C.c_int


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) the shared library; raises if any export is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise FitError(f"libfit_gb300.so not found at {path}; run __graft_entry__.build()")
    lib = C.CDLL(path)
    missing = [n for n in EXPORTS if not hasattr(lib, n)]
    if missing:
        raise FitError(f"libfit_gb300.so lacks exports {missing}")
    _declare(lib)
    _lib = lib
    return lib


def check(rc: int):
    if rc == 0:
        return
    msg = _lib.fit_last_error().decode(errors="replace")
    if rc in (-1, -2):
        raise ValueError(msg)
    raise FitError(f"libfit_gb300 {ERRORS.get(rc, rc)} error: {msg}")


def launch_count() -> int:
    return int(load().fit_launch_count())


def mlp_status() -> int:
    """1 when a clock-bounded wait inside an earlier MLP forward gave up (clears the flag)."""
    v = C.c_int(0)
    check(load().fit_mlp_status(C.byref(v)))
    return int(v.value)


def prof_enable(on: bool):
    check(load().fit_prof_enable(int(on)))


def prof_read_all():
    """{kind name: (ms_total, algorithmic_bytes_total, launches)} since the last prof_enable."""
    lib = load()
    out = {}
    for k in range(64):
        if not lib.fit_prof_kind_name(k):
            break
        ms, by, n = C.c_double(), C.c_double(), C.c_longlong()
        check(lib.fit_prof_read(k, C.byref(ms), C.byref(by), C.byref(n)))
        if n.value:
            out[lib.fit_prof_kind_name(k).decode()] = (ms.value, by.value, n.value)
    return out
