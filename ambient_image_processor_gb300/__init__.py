"""GB300-native TGV-DCT shading correction (sm_103a), drop-in for the reference path.

This package is a thin Python view of the C ABI in ``include/tgvdct.h``
(``_build/libtgvdct.so``).  It mirrors the reference's operator surface for the
path — the raw launchers of ``source/modules/tgv_deshade`` and
``source/modules/cuda_image_operations`` and the ``TGVDeshadeProcessor`` methods
that call them — with numpy arrays in (depth, height, width) order, x fastest.
Every compute call goes to the CUDA library; if it is missing, the call raises.
"""
from __future__ import annotations

import ctypes
import os
import numpy as np

from . import phantoms  # noqa: F401  (re-exported for users and benchmarks)

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libtgvdct.so")

# enums of include/tgvdct.h
OK, ERR_BAD_ARG, ERR_OOM, ERR_CUDA, ERR_NO_DEVICE, ERR_UNSUPPORTED, STOPPED, ERR_TIMEOUT = range(8)
DATA_L1, DATA_L2 = 0, 1
GEOMETRY_3D, GEOMETRY_2D = 0, 1
STATE_FP32, STATE_BF16_DUAL, STATE_FX16_DUAL = 0, 1, 2
DCT_FP32, DCT_TF32, DCT_BF16X3 = 0, 1, 2
EIGEN_REFERENCE, EIGEN_ACCURATE = 0, 1
KERNEL_AUTO, KERNEL_TWO_PASS, KERNEL_FUSED, KERNEL_FUSED_REGISTER = 0, 1, 2, 3
KERNEL_FUSED_SHIFTED = 4

_STATUS_NAMES = {OK: "ok", ERR_BAD_ARG: "bad argument", ERR_OOM: "out of memory",
                 ERR_CUDA: "CUDA error", ERR_NO_DEVICE: "no suitable CUDA device",
                 ERR_UNSUPPORTED: "unsupported mode", STOPPED: "stopped early",
                 ERR_TIMEOUT: "a bounded wait in a kernel ran out"}


class TgvdctError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Params(ctypes.Structure):
    """tgvdct_params."""
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("depth", ctypes.c_uint32), ("lambda_", ctypes.c_float),
                ("alpha0", ctypes.c_float), ("alpha1", ctypes.c_float),
                ("iteration_count", ctypes.c_uint32), ("tau", ctypes.c_float),
                ("sigma", ctypes.c_float), ("theta", ctypes.c_float),
                ("data_term", ctypes.c_int32), ("geometry", ctypes.c_int32),
                ("state_precision", ctypes.c_int32), ("dct_mode", ctypes.c_int32),
                ("poisson_eigen", ctypes.c_int32),
                ("paint_iteration_interval", ctypes.c_uint32),
                ("callback_on_device", ctypes.c_int32),
                ("iteration_kernel", ctypes.c_int32), ("z_chunk", ctypes.c_int32),
                ("energy_check_interval", ctypes.c_uint32),
                ("energy_tolerance", ctypes.c_float)]


CALLBACK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32,
                            ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                            ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                            ctypes.c_void_p)

_lib = None
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_u32 = ctypes.c_uint32
_i32 = ctypes.c_int32
_flt = ctypes.c_float

# name -> argtypes (restype tgvdct_status unless noted)
_SIGS = {
    "tgvdct_params_init": [ctypes.POINTER(Params)],
    "tgvdct_workspace_bytes": [ctypes.POINTER(Params)],
    "tgvdct_create": [ctypes.POINTER(Params), ctypes.POINTER(_vp)],
    "tgvdct_destroy": [_vp],
    "tgvdct_set_params": [_vp, ctypes.POINTER(Params)],
    "tgvdct_iterations_run": [_vp],
    "tgvdct_loop_launches": [_vp],
    "tgvdct_tgv2_l1_deshade_launch": [_f32p, _u32, _u32, _u32, _flt, _u32, _u32, ctypes.c_int,
                                      CALLBACK, _vp, _flt, _flt, _f32p, _f32p, _f32p, _f32p],
    "tgvdct_tgv2_l1_deshade_launch_2d": [_f32p, _u32, _u32, _flt, _u32, _u32, CALLBACK, _vp,
                                         _flt, _flt, _f32p, _f32p, _f32p],
    "tgvdct_tgv2_denoise_launch": [_f32p, _u32, _u32, _u32, _i32, _flt, _u32, _flt, _flt, _f32p],
    "tgvdct_tgv2_run_dev": [_vp, _vp, _vp, _vp, _vp, _vp, CALLBACK, _vp, _vp],
    "tgvdct_tgv2_forward_checkpointed_dev": [_vp, _vp, _vp, _vp, _vp, _vp, _u32, _vp],
    "tgvdct_tgv2_backward_dev": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "tgvdct_divergence_launch": [_f32p, _f32p, _vp, _u32, _u32, _u32, _f32p],
    "tgvdct_divergence_dev": [_vp, _vp, _vp, _u32, _u32, _u32, _vp, _vp],
    "tgvdct_set_domain_mask_dev": [_vp, _vp, _vp],
    "tgvdct_poisson_integrate_adjoint_dev": [_vp, _vp, _vp, _vp, _vp, _vp],
    "tgvdct_convergence_test": [ctypes.POINTER(Params), _f32p, _vp, _u32, _vp, _vp, _u32,
                                ctypes.POINTER(_u32), _vp],
    "tgvdct_convergence_optimization": [ctypes.POINTER(Params), _f32p, _vp, _i32,
                                        ctypes.POINTER(ctypes.c_float),
                                        ctypes.POINTER(ctypes.c_float), _f32p, _f32p, _f32p],
    "tgvdct_process_tgv2_l1_masked": [ctypes.POINTER(Params), _f32p, _f32p, _i32, _i32, _i32,
                                      CALLBACK, _vp, _f32p, _f32p, _f32p],
    "tgvdct_tgv2_l1_deshade_masked_launch": [_f32p, _f32p, _u32, _u32, _u32, _flt, _u32, _u32,
                                             ctypes.c_int, CALLBACK, _vp, _flt, _flt, _f32p,
                                             _f32p, _f32p, _vp],
    "tgvdct_device_alloc": [ctypes.c_size_t, ctypes.POINTER(_vp)],
    "tgvdct_device_free": [_vp],
    "tgvdct_host_to_device": [_vp, _vp, ctypes.c_size_t],
    "tgvdct_device_to_host": [_vp, _vp, ctypes.c_size_t],
    "tgvdct_tgv2_run": [ctypes.POINTER(Params), _f32p, _f32p, _vp, _vp, _vp, CALLBACK, _vp],
    "tgvdct_cosine_transform_launch": [_f32p, _u32, _u32, _u32, _i32, _f32p],
    "tgvdct_inverse_cosine_transform_launch": [_f32p, _u32, _u32, _u32, _i32, _f32p],
    "tgvdct_solve_poisson_in_cosine_domain_launch": [_f32p, _u32, _u32, _u32, _i32, _f32p],
    "tgvdct_integrate_image_gradients_poisson_cosine_transform": [_f32p, _f32p, _vp, _u32, _u32,
                                                                  _u32, _i32, _i32, _f32p],
    "tgvdct_poisson_integrate_dev": [_vp, _vp, _vp, _vp, _vp, _vp],
    "tgvdct_poisson_solve_dev": [_vp, _vp, _vp, _vp],
    "tgvdct_check_device_error": [_vp, _vp],
    "tgvdct_set_pipeline_wait_limit": [_vp, ctypes.c_uint64],
    "tgvdct_integrate_poisson_noalloc_dev": [_vp, _vp, _vp, _u32, _u32, _u32, _i32, _i32, _vp,
                                             _vp],
    "tgvdct_deshade_epilogue_dev": [_vp, _vp, _vp, ctypes.c_uint64, _i32, _i32, _i32, _vp, _vp],
    "tgvdct_process_tgv2_l1": [ctypes.POINTER(Params), _f32p, _vp, _i32, _i32, _i32, CALLBACK,
                               _vp, _f32p, _f32p, _f32p],
    "tgvdct_process_dev": [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp, _vp, CALLBACK, _vp, _vp],
    "tgvdct_tgv2_energy": [ctypes.POINTER(Params), _f32p, _f32p, _f32p, _f32p, _vp,
                           np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")],
    "tgvdct_tgv2_energy_dev": [ctypes.POINTER(Params), _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "tgvdct_energy_history": [_vp, _vp, _u32, ctypes.POINTER(_u32)],
    "tgvdct_request_stop": [_vp],
    "tgvdct_release_cached": [],
    "tgvdct_state_bytes": [_vp],
    "tgvdct_bounds_check": [ctypes.POINTER(ctypes.c_uint64)],
    "tgvdct_state_save_dev": [_vp, _vp, _vp],
    "tgvdct_state_load_dev": [_vp, _vp, _vp],
    "tgvdct_tgv2_resume_dev": [_vp, _vp, _vp, _vp, _vp, CALLBACK, _vp, _vp],
    "tgvdct_state_init_dev": [_vp, _vp, _vp],
    "tgvdct_tgv2_step_dev": [_vp, _u32, _vp],
    "tgvdct_state_planes_bytes": [_vp, _u32, _u32],
    "tgvdct_state_read_dev": [_vp, _u32, _u32, _u32, _vp, _vp],
    "tgvdct_state_write_dev": [_vp, _u32, _u32, _u32, _vp, _vp],
    "tgvdct_slab_poisson_xy_dev": [_vp, _vp, _vp, _vp, _vp, _vp],
    "tgvdct_slab_poisson_inverse_yx_dev": [_vp, _vp, _vp, _u32, _u32, _vp],
    "tgvdct_pencil_create": [_u32, _u32, _u32, ctypes.c_uint64, ctypes.POINTER(_vp)],
    "tgvdct_pencil_destroy": [_vp],
    "tgvdct_pencil_poisson_z_dev": [_vp, _vp, _vp, ctypes.c_uint64, _i32, _vp],
    "tgvdct_resize_bspline3": [_f32p, _u32, _u32, _u32, _f32p, _u32, _u32, _u32],
    "tgvdct_resize_bspline3_dev": [_vp, _u32, _u32, _u32, _vp, _u32, _u32, _u32, _vp],
    "tgvdct_resize_factor_extent": [_u32, _flt],
    "tgvdct_process_tgvk_l1_downsampled": [_f32p, _vp, _u32, _u32, _u32, _flt, _flt, _u32, _f32p,
                                           _u32, _i32, _i32, _i32, _u32, CALLBACK, _vp, _f32p,
                                           _f32p, _f32p, _vp],
    "tgvdct_process_tgvk_l1_downsampled_dev": [_vp, _vp, _u32, _u32, _u32, _flt, _flt, _u32,
                                               _f32p, _u32, _i32, _i32, _i32, _u32, CALLBACK,
                                               _vp, _vp, _vp, _vp, _vp, _vp],
}
_RESTYPES = {"tgvdct_params_init": None, "tgvdct_workspace_bytes": ctypes.c_size_t,
             "tgvdct_iterations_run": ctypes.c_uint32, "tgvdct_version": ctypes.c_char_p,
             "tgvdct_loop_launches": ctypes.c_uint64,
             "tgvdct_last_error": ctypes.c_char_p, "tgvdct_status_string": ctypes.c_char_p,
             "tgvdct_resize_factor_extent": ctypes.c_uint32,
             "tgvdct_state_bytes": ctypes.c_size_t,
             "tgvdct_state_planes_bytes": ctypes.c_size_t}

# symbols of include/tgvdct.h (checked by the CPU test suite)
EXPORTED = sorted(set(_SIGS) | {"tgvdct_version", "tgvdct_last_error", "tgvdct_status_string"})


def lib() -> ctypes.CDLL:
    """The CUDA library; raises if it has not been built (there is no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run "
                              "`python -m ambient_image_processor_gb300.build` first")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        for name in ("tgvdct_version", "tgvdct_last_error"):
            getattr(L, name).restype = ctypes.c_char_p
            getattr(L, name).argtypes = []
        L.tgvdct_status_string.restype = ctypes.c_char_p
        L.tgvdct_status_string.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


_lib_checked = None


def lib_checked() -> ctypes.CDLL:
    """The bounds-checking build of the library (libtgvdct_checked.so), compiled on
    first use; same entry points as lib(), plus a working tgvdct_bounds_check."""
    global _lib_checked
    if _lib_checked is None:
        from . import build as _build
        path = _build.build(checked=True)
        L = ctypes.CDLL(path)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        L.tgvdct_last_error.restype = ctypes.c_char_p
        L.tgvdct_last_error.argtypes = []
        _lib_checked = L
    return _lib_checked


def version() -> str:
    return lib().tgvdct_version().decode()


def release_cached() -> None:
    """Frees the context and device buffers the host-buffer one-shot calls keep
    between calls (tgvdct_release_cached)."""
    _check(lib().tgvdct_release_cached(), allow_stop=False)


def _check(status: int, allow_stop: bool = True) -> int:
    if status == OK or (allow_stop and status == STOPPED):
        return status
    raise TgvdctError(status, lib().tgvdct_last_error().decode())


def default_params(**kw) -> Params:
    p = Params()
    lib().tgvdct_params_init(ctypes.byref(p))
    for k, v in kw.items():
        if k == "lambda":
            k = "lambda_"
        if not hasattr(p, k):
            raise AttributeError(f"tgvdct_params has no field {k}")
        setattr(p, k, v)
    return p


def _dims(a: np.ndarray):
    if a.ndim == 2:
        return a.shape[1], a.shape[0], 1
    if a.ndim == 3:
        return a.shape[2], a.shape[1], a.shape[0]
    raise ValueError("expected a 2-D (H, W) or 3-D (D, H, W) array")


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _make_callback(fn, shape, n_out):
    """Wraps a Python callable(iteration_index, iteration_count, *images) -> stop?"""
    if fn is None:
        return CALLBACK(), None
    size = int(np.prod(shape))

    def trampoline(it, count, a, b, c, d, _user):
        arrs = []
        for ptr in (a, b, c, d)[:n_out]:
            if ptr:
                arrs.append(np.ctypeslib.as_array(ptr, shape=(size,)).reshape(shape).copy())
            else:
                arrs.append(None)
        try:
            return 1 if fn(int(it), int(count), *arrs) else 0
        except Exception:  # a raising callback stops the loop
            return 1

    cb = CALLBACK(trampoline)
    return cb, cb


# ---------------------------------------------------------------------------
# Raw launchers (reference: tgv_deshade/*.cu, tgv_cuda/*.cu, cuda_image_operations/*.cu)

def tgv2_l1_deshade_launch(f, lambda_, iteration_count, paint_iteration_interval=0,
                           cuda_block_dimension=-1, iteration_finished_callback=None,
                           alpha0=2.0, alpha1=1.0):
    """tgv2_l1_deshade_launch<float> (tgv_deshade/tgv2_l1_deshade.cu:33-41).

    Returns (u, v_x, v_y, v_z).  The callback gets (iteration_index,
    iteration_count, u, v_x, v_y, v_z) and stops the loop by returning True.
    """
    f = _f32(f)
    w, h, d = _dims(f)
    u, vx, vy, vz = (np.empty_like(f) for _ in range(4))
    cb, keep = _make_callback(iteration_finished_callback, f.shape, 4)
    _check(lib().tgvdct_tgv2_l1_deshade_launch(f, w, h, d, lambda_, iteration_count,
                                               paint_iteration_interval, cuda_block_dimension,
                                               cb, None, alpha0, alpha1, u, vx, vy, vz))
    del keep
    return u, vx, vy, vz


def tgv2_l1_deshade_launch_2d(f, lambda_, iteration_count, paint_iteration_interval=0,
                              iteration_finished_callback=None, alpha0=2.0, alpha1=1.0):
    """tgv2_l1_deshade_launch_2d<float> (tgv_deshade/tgv2_l1_deshade_2d.cu:29-36)."""
    f = _f32(f)
    if f.ndim != 2:
        raise ValueError("the 2-D launcher takes an (H, W) image")
    h, w = f.shape
    u, vx, vy = (np.empty_like(f) for _ in range(3))
    cb, keep = _make_callback(iteration_finished_callback, f.shape, 3)
    _check(lib().tgvdct_tgv2_l1_deshade_launch_2d(f, w, h, lambda_, iteration_count,
                                                  paint_iteration_interval, cb, None, alpha0,
                                                  alpha1, u, vx, vy))
    del keep
    return u, vx, vy


def tgv2_denoise_launch(f, lambda_, iteration_count, alpha0=2.0, alpha1=1.0, data_term=DATA_L1):
    """tgv2_l1_launch / tgv2_l2_launch (tgv_cuda/tgv2_l1.cu:64, tgv_cuda/tgv2_l2.cu:60)."""
    f = _f32(f)
    w, h, d = _dims(f)
    u = np.empty_like(f)
    _check(lib().tgvdct_tgv2_denoise_launch(f, w, h, d, data_term, lambda_, iteration_count,
                                            alpha0, alpha1, u), allow_stop=False)
    return u


def divergence_kernel_launch(dx, dy, dz=None):
    """divergence_kernel_launch (cuda_image_operations/divergence.cu:59-61)."""
    dx, dy = _f32(dx), _f32(dy)
    w, h, d = _dims(dx)
    dzp = None
    if d > 1:
        dz = _f32(dz)
        dzp = dz.ctypes.data_as(_vp)
    out = np.empty_like(dx)
    _check(lib().tgvdct_divergence_launch(dx, dy, dzp, w, h, d, out), allow_stop=False)
    return out


def cosine_transform_kernel_launch(x, dct_mode=DCT_FP32):
    """cosine_transform_kernel_launch (cuda_image_operations/cosine_transform.cu:226-227)."""
    x = _f32(x)
    w, h, d = _dims(x)
    out = np.empty_like(x)
    _check(lib().tgvdct_cosine_transform_launch(x, w, h, d, dct_mode, out), allow_stop=False)
    return out


def inverse_cosine_transform_kernel_launch(x, dct_mode=DCT_FP32):
    """inverse_cosine_transform_kernel_launch (inverse_cosine_transform.cu:167-168)."""
    x = _f32(x)
    w, h, d = _dims(x)
    out = np.empty_like(x)
    _check(lib().tgvdct_inverse_cosine_transform_launch(x, w, h, d, dct_mode, out),
           allow_stop=False)
    return out


def solve_poisson_in_cosine_domain_kernel_launch(x, poisson_eigen=EIGEN_REFERENCE):
    """solve_poisson_in_cosine_domain_kernel_launch (solve_poisson_in_cosine_domain.cu:86-87)."""
    x = _f32(x)
    w, h, d = _dims(x)
    out = np.empty_like(x)
    _check(lib().tgvdct_solve_poisson_in_cosine_domain_launch(x, w, h, d, poisson_eigen, out),
           allow_stop=False)
    return out


# ---------------------------------------------------------------------------
class TGVDeshadeProcessor:
    """Mirror of the reference's TGVDeshadeProcessor static API
    (tgv_deshade/TGVDeshadeProcessor.h:23-183) over numpy images."""

    @staticmethod
    def integrate_image_gradients_poisson_cosine_transform(gradient_x, gradient_y,
                                                           gradient_z=None, dct_mode=DCT_FP32,
                                                           poisson_eigen=EIGEN_REFERENCE):
        """TGVDeshadeProcessor.cpp:386-408 (2-D inputs: :410-431)."""
        gx, gy = _f32(gradient_x), _f32(gradient_y)
        w, h, d = _dims(gx)
        gzp = None
        if d > 1:
            gz = _f32(gradient_z)
            gzp = gz.ctypes.data_as(_vp)
        out = np.empty_like(gx)
        _check(lib().tgvdct_integrate_image_gradients_poisson_cosine_transform(
            gx, gy, gzp, w, h, d, dct_mode, poisson_eigen, out), allow_stop=False)
        return out

    @staticmethod
    def processTGV2L1GPUCuda(input_image, lambda_, alpha0, alpha1, iteration_count,
                             cuda_block_dimension=-1, mask_image=None,
                             set_negative_values_to_zero=True, *, paint_iteration_interval=0,
                             iteration_finished_callback=None, add_background_back=False,
                             log_domain=False, data_term=DATA_L1, two_d=False,
                             state_precision=STATE_FP32, dct_mode=DCT_FP32,
                             poisson_eigen=EIGEN_REFERENCE, tau=None, sigma=None,
                             iteration_kernel=KERNEL_AUTO, z_chunk=0):
        """TGVDeshadeProcessor::processTGV2L1GPUCuda (TGVDeshadeProcessor.cpp:122-166; the
        GUI overload with mask, callback and add-back: :285-314).

        Returns (denoised_image, shading_image, deshaded_image).  The callback gets
        (iteration_index, iteration_count, u, l, r) — the reference's
        IterationFinishedThreeImages (TGVDeshadeProcessor.h:34-36).
        """
        f = _f32(input_image)
        w, h, d = _dims(f)
        p = default_params(width=w, height=h, depth=d, lambda_=lambda_, alpha0=alpha0,
                           alpha1=alpha1, iteration_count=iteration_count,
                           data_term=data_term,
                           geometry=GEOMETRY_2D if two_d else GEOMETRY_3D,
                           state_precision=state_precision, dct_mode=dct_mode,
                           poisson_eigen=poisson_eigen,
                           paint_iteration_interval=paint_iteration_interval,
                           iteration_kernel=iteration_kernel, z_chunk=z_chunk)
        if tau is not None:
            p.tau = tau
        if sigma is not None:
            p.sigma = sigma
        mptr, mask = None, None
        if mask_image is not None:
            mask = _f32(mask_image)
            mptr = mask.ctypes.data_as(_vp)
        u, l, r = (np.empty_like(f) for _ in range(3))
        cb, keep = _make_callback(iteration_finished_callback, f.shape, 3)
        _check(lib().tgvdct_process_tgv2_l1(ctypes.byref(p), f, mptr,
                                            int(set_negative_values_to_zero),
                                            int(add_background_back), int(log_domain), cb, None,
                                            u, l, r))
        del keep
        return u, l, r


def convergence_test(input_image, lambda_, alpha0, alpha1, iteration_count,
                     check_iteration_interval=1, mask=None, **params):
    """TGVDeshadeProcessor::processTGV2L1DeshadeCuda_convergenceTest and ...Metric
    (TGVDeshadeProcessor.cpp:479-568).  Returns (ncc history, time-TV history,
    metric TVs (2,)) as FP64 numpy arrays."""
    f = _f32(input_image)
    w, h, d = _dims(f)
    p = default_params(width=w, height=h, depth=d, lambda_=lambda_, alpha0=alpha0,
                       alpha1=alpha1, iteration_count=iteration_count, **params)
    cap = iteration_count // max(check_iteration_interval, 1) + 1
    ncc, tv, mt = np.zeros(cap), np.zeros(cap), np.zeros(2)
    cnt = _u32()
    mptr, m = None, None
    if mask is not None:
        m = _f32(mask)
        mptr = m.ctypes.data_as(_vp)
    _check(lib().tgvdct_convergence_test(ctypes.byref(p), f, mptr, check_iteration_interval,
                                         ncc.ctypes.data_as(_vp), tv.ctypes.data_as(_vp), cap,
                                         ctypes.byref(cnt), mt.ctypes.data_as(_vp)),
           allow_stop=False)
    k = min(int(cnt.value), cap)
    return ncc[:k], tv[:k], mt


def convergence_optimization(input_image, lambda_, mask=None, set_negative_values_to_zero=True,
                             **params):
    """TGVDeshadeProcessor::processTGV2L1DeshadeCuda_convergenceOptimization
    (TGVDeshadeProcessor.cpp:571-646): returns (alpha0, alpha1, u, l, r)."""
    f = _f32(input_image)
    w, h, d = _dims(f)
    p = default_params(width=w, height=h, depth=d, lambda_=lambda_, **params)
    a0, a1 = ctypes.c_float(), ctypes.c_float()
    u, l, r = (np.empty_like(f) for _ in range(3))
    mptr, m = None, None
    if mask is not None:
        m = _f32(mask)
        mptr = m.ctypes.data_as(_vp)
    _check(lib().tgvdct_convergence_optimization(ctypes.byref(p), f, mptr,
                                                 int(set_negative_values_to_zero),
                                                 ctypes.byref(a0), ctypes.byref(a1), u, l, r),
           allow_stop=False)
    return a0.value, a1.value, u, l, r


# ---------------------------------------------------------------------------
class TGVDeshadeMaskedProcessor:
    """Mirror of the reference's TGVDeshadeMaskedProcessor
    (tgv_deshade_masked/TGVDeshadeMaskedProcessor.h) over numpy images: the TGV loop
    runs on the voxels with mask >= 1 only."""

    @staticmethod
    def processTGV2L1GPUCuda(input_image, lambda_, alpha0, alpha1, iteration_count,
                             cuda_block_dimension=-1, paint_iteration_interval=0,
                             iteration_finished_callback=None, mask=None,
                             set_negative_values_to_zero=True, add_background_back=False, *,
                             log_domain=False, state_precision=STATE_FP32, dct_mode=DCT_FP32,
                             poisson_eigen=EIGEN_REFERENCE, iteration_kernel=KERNEL_AUTO,
                             z_chunk=0):
        """TGVDeshadeMaskedProcessor::processTGV2L1GPUCuda
        (TGVDeshadeMaskedProcessor.cpp:77-212; 2-D operators when depth == 1, :214-330).
        A missing mask means every voxel (the reference substitutes an all-ones mask).
        Returns (denoised_image, shading_image, deshaded_image); the callback gets
        (iteration_index, iteration_count, u, l, r)."""
        f = _f32(input_image)
        w, h, d = _dims(f)
        m = np.ones_like(f) if mask is None else _f32(mask)
        if m.shape != f.shape:
            raise ValueError("mask shape differs from the image shape")
        p = default_params(width=w, height=h, depth=d, lambda_=lambda_, alpha0=alpha0,
                           alpha1=alpha1, iteration_count=iteration_count,
                           state_precision=state_precision, dct_mode=dct_mode,
                           poisson_eigen=poisson_eigen,
                           paint_iteration_interval=paint_iteration_interval,
                           iteration_kernel=iteration_kernel, z_chunk=z_chunk)
        u, l, r = (np.empty_like(f) for _ in range(3))
        cb, keep = _make_callback(iteration_finished_callback, f.shape, 3)
        _check(lib().tgvdct_process_tgv2_l1_masked(ctypes.byref(p), f, m,
                                                   int(set_negative_values_to_zero),
                                                   int(add_background_back), int(log_domain), cb,
                                                   None, u, l, r))
        del keep
        return u, l, r


def tgv2_l1_deshade_masked_launch(f, mask, lambda_, iteration_count, alpha0, alpha1):
    """tgv2_l1_deshade_masked_launch / _2d_launch (tgv_deshade_masked/): the masked loop.
    Returns (u, v_x, v_y, v_z); v_z is zero when depth == 1."""
    f = _f32(f)
    m = _f32(mask)
    w, h, d = _dims(f)
    u, vx, vy, vz = (np.empty_like(f) for _ in range(4))
    _check(lib().tgvdct_tgv2_l1_deshade_masked_launch(f, m, w, h, d, lambda_, iteration_count, 0,
                                                      -1, CALLBACK(), None, alpha0, alpha1, u,
                                                      vx, vy, vz.ctypes.data_as(_vp)))
    return u, vx, vy, vz


def tgv2_energy(f, u, v_x, v_y, v_z=None, *, lambda_=1.0, alpha0=2.0, alpha1=1.0,
                data_term=DATA_L1, geometry=None):
    """TGV2 primal energy of (u, v) for f (tgvdct_tgv2_energy): returns
    [lambda-weighted data term, alpha1 sum |F u - v|, alpha0 sum |E v|, total], FP64
    sums of the FP32 per-voxel terms on the device.  No counterpart in the reference."""
    f = _f32(f)
    w, h, d = _dims(f)
    if geometry is None:
        geometry = GEOMETRY_2D if d == 1 and v_z is None else GEOMETRY_3D
    p = default_params(width=w, height=h, depth=d, lambda_=lambda_, alpha0=alpha0,
                       alpha1=alpha1, data_term=data_term, geometry=geometry)
    out = np.zeros(4, dtype=np.float64)
    vz = None if v_z is None else _f32(v_z)
    _check(lib().tgvdct_tgv2_energy(ctypes.byref(p), f, _f32(u), _f32(v_x), _f32(v_y),
                                    None if vz is None else vz.ctypes.data_as(_vp), out))
    return out


# ---------------------------------------------------------------------------
# Down-sampled deshade (reference: resize/ResizeProcessor.cpp,
# tgvk_deshade_downsampled/TGVKDeshadeDownsampled*Processor.cpp)
BSPLINE3 = "BSpline3"


def _shape_of(a: np.ndarray):
    """(depth, height, width) of a 2-D (H, W) or 3-D (D, H, W) image."""
    return (1,) + a.shape if a.ndim == 2 else a.shape


class ResizeProcessor:
    """Mirror of the reference's ResizeProcessor (resize/ResizeProcessor.h) for its
    BSpline3 interpolation method, over numpy images."""

    InterpolationMethod = type("InterpolationMethod", (), {"BSpline3": BSPLINE3})

    @staticmethod
    def size_for_factor(shape, size_factor):
        """(depth, height, width) of process(image, size_factor) (ResizeProcessor.cpp:35-47)."""
        e = lib().tgvdct_resize_factor_extent
        return tuple(int(e(int(n), float(size_factor))) for n in shape)

    @staticmethod
    def process(image, size_factor_or_width, height=None, depth=None,
                interpolation_method=BSPLINE3):
        """process(image, size_factor, method) or process(image, width, height, depth,
        method) (ResizeProcessor.cpp:35-143), cubic B-spline through the GPU.  A 2-D
        (H, W) image stays 2-D when depth is 1."""
        if interpolation_method != BSPLINE3:
            raise ValueError("only the BSpline3 interpolation method is built")
        x = _f32(image)
        w, h, d = _dims(x)
        if height is None:
            D, H, W = ResizeProcessor.size_for_factor((d, h, w), size_factor_or_width)
        else:
            W, H, D = int(size_factor_or_width), int(height), int(depth if depth else 1)
        out = np.empty((H, W) if (x.ndim == 2 and D == 1) else (D, H, W), dtype=np.float32)
        _check(lib().tgvdct_resize_bspline3(x, w, h, d, out, W, H, D))
        return out


def _downsampled(not_masked, input_image, downsampling_factor, lambda_, order, alpha,
                 iteration_count, mask, set_negative_values_to_zero, add_background_back,
                 paint_iteration_interval, iteration_finished_callback, calculate_div_v):
    f = _f32(input_image)
    w, h, d = _dims(f)
    m = None if mask is None else _f32(mask)
    if m is not None and m.shape != f.shape:
        raise ValueError("mask shape differs from the image shape")
    a = _f32(np.asarray(alpha, dtype=np.float32).reshape(-1))
    if a.size < 2:
        raise ValueError("alpha needs order entries")
    u, l, r = (np.empty_like(f) for _ in range(3))
    dv = np.empty_like(f) if calculate_div_v else None
    if downsampling_factor == 1:
        small = _shape_of(f)
    else:
        small = ResizeProcessor.size_for_factor(_shape_of(f), downsampling_factor)
    cb, keep = _make_callback(iteration_finished_callback,
                              small if f.ndim == 3 else small[1:], 3)
    _check(lib().tgvdct_process_tgvk_l1_downsampled(
        f, None if m is None else m.ctypes.data_as(_vp), w, h, d, float(downsampling_factor),
        float(lambda_), int(order), a, int(iteration_count), int(set_negative_values_to_zero),
        int(add_background_back), int(not_masked), int(paint_iteration_interval), cb, None, u, l,
        r, None if dv is None else dv.ctypes.data_as(_vp)))
    del keep
    return u, l, r, dv


class TGVKDeshadeDownsampledProcessor:
    """Mirror of the reference's TGVKDeshadeDownsampledProcessor
    (tgvk_deshade_downsampled/TGVKDeshadeDownsampledProcessor.h) over numpy images."""

    @staticmethod
    def processTGVKL1Cuda(input_image, downsampling_factor, lambda_, order, alpha,
                          iteration_count, mask=None, set_negative_values_to_zero=True,
                          add_background_back=False, paint_iteration_interval=0,
                          iteration_finished_callback=None, calculate_div_v=False):
        """processTGVKL1Cuda (TGVKDeshadeDownsampledProcessor.cpp:30-129): the image
        (times the mask) and the mask are resized by downsampling_factor with cubic
        B-splines, deshaded there by the masked TGV2 processor (order 2; alpha0 =
        alpha[1], alpha1 = alpha[0]), and the denoised image and the shading resized
        back.  Returns (denoised_image, shading_image, deshaded_image, div_v_image or
        None); the callback gets the down-sampled (iteration, count, u, l, r)."""
        return _downsampled(False, input_image, downsampling_factor, lambda_, order, alpha,
                            iteration_count, mask, set_negative_values_to_zero,
                            add_background_back, paint_iteration_interval,
                            iteration_finished_callback, calculate_div_v)


class TGVKDeshadeDownsampledNotMaskedProcessor:
    """Mirror of the reference's TGVKDeshadeDownsampledNotMaskedProcessor
    (tgvk_deshade_downsampled/TGVKDeshadeDownsampledNotMaskedProcessor.h)."""

    @staticmethod
    def processTGVKL1Cuda(input_image, downsampling_factor, lambda_, order, alpha,
                          iteration_count, mask=None, set_negative_values_to_zero=True,
                          add_background_back=False, paint_iteration_interval=0,
                          iteration_finished_callback=None, calculate_div_v=False):
        """processTGVKL1Cuda (TGVKDeshadeDownsampledNotMaskedProcessor.cpp:30-129): as
        the masked variant, but the TGV2 loop runs on every voxel of the resized image
        and the mask only weights the results."""
        return _downsampled(True, input_image, downsampling_factor, lambda_, order, alpha,
                            iteration_count, mask, set_negative_values_to_zero,
                            add_background_back, paint_iteration_interval,
                            iteration_finished_callback, calculate_div_v)


# ---------------------------------------------------------------------------
class Context:
    """A device workspace for one volume shape (tgvdct_context).

    Device buffers are passed as raw pointers (ints), e.g. ``tensor.data_ptr()``,
    and streams as raw handles (``torch.cuda.Stream.cuda_stream``) or None.
    """

    def __init__(self, params: Params):
        self.params = params
        self._ctx = _vp()
        _check(lib().tgvdct_create(ctypes.byref(params), ctypes.byref(self._ctx)),
               allow_stop=False)

    def close(self):
        if self._ctx:
            lib().tgvdct_destroy(self._ctx)
            self._ctx = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def iterations_run(self) -> int:
        return int(lib().tgvdct_iterations_run(self._ctx))

    def loop_launches(self) -> int:
        """Iteration kernels the context's last loop launched (graph replays included)."""
        return int(lib().tgvdct_loop_launches(self._ctx))

    def set_params(self, params: Params):
        _check(lib().tgvdct_set_params(self._ctx, ctypes.byref(params)), allow_stop=False)
        self.params = params

    def run_dev(self, f_ptr, u_ptr, vx_ptr, vy_ptr, vz_ptr=None, stream=None,
                callback=None) -> int:
        return _check(lib().tgvdct_tgv2_run_dev(self._ctx, f_ptr, u_ptr, vx_ptr, vy_ptr, vz_ptr,
                                                callback or CALLBACK(), None, stream))

    def forward_checkpointed_dev(self, f_ptr, u_ptr, vx_ptr, vy_ptr, vz_ptr, checkpoint_every,
                                 stream=None):
        _check(lib().tgvdct_tgv2_forward_checkpointed_dev(self._ctx, f_ptr, u_ptr, vx_ptr, vy_ptr,
                                                          vz_ptr, checkpoint_every, stream),
               allow_stop=False)

    def backward_dev(self, grad_u_ptr, grad_vx_ptr, grad_vy_ptr, grad_vz_ptr, grad_f_ptr,
                     grad_params_ptr, stream=None):
        _check(lib().tgvdct_tgv2_backward_dev(self._ctx, grad_u_ptr, grad_vx_ptr, grad_vy_ptr,
                                              grad_vz_ptr, grad_f_ptr, grad_params_ptr, stream),
               allow_stop=False)

    def poisson_integrate_dev(self, vx_ptr, vy_ptr, vz_ptr, l_ptr, stream=None):
        _check(lib().tgvdct_poisson_integrate_dev(self._ctx, vx_ptr, vy_ptr, vz_ptr, l_ptr,
                                                  stream), allow_stop=False)

    def poisson_integrate_adjoint_dev(self, grad_l_ptr, gvx_ptr, gvy_ptr, gvz_ptr, stream=None):
        _check(lib().tgvdct_poisson_integrate_adjoint_dev(self._ctx, grad_l_ptr, gvx_ptr, gvy_ptr,
                                                          gvz_ptr, stream), allow_stop=False)

    def poisson_solve_dev(self, rhs_ptr, l_ptr, stream=None):
        _check(lib().tgvdct_poisson_solve_dev(self._ctx, rhs_ptr, l_ptr, stream),
               allow_stop=False)

    def set_domain_mask_dev(self, mask_ptr, stream=None):
        """Restrict the loop to voxels with mask >= 1 (None clears); see
        tgvdct_set_domain_mask_dev."""
        _check(lib().tgvdct_set_domain_mask_dev(self._ctx, mask_ptr, stream), allow_stop=False)

    def energy_history(self) -> np.ndarray:
        """The weighted TGV2 energies of the last loop's energy checks, in order."""
        n = _u32()
        _check(lib().tgvdct_energy_history(self._ctx, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.float64)
        if n.value:
            _check(lib().tgvdct_energy_history(self._ctx, out.ctypes.data_as(_vp), n.value,
                                               ctypes.byref(n)))
        return out

    def state_bytes(self) -> int:
        return int(lib().tgvdct_state_bytes(self._ctx))

    def save_state_dev(self, dst_ptr, stream=None):
        """Snapshot of the loop state into a device buffer of state_bytes()."""
        _check(lib().tgvdct_state_save_dev(self._ctx, dst_ptr, stream), allow_stop=False)

    def load_state_dev(self, src_ptr, stream=None):
        _check(lib().tgvdct_state_load_dev(self._ctx, src_ptr, stream), allow_stop=False)

    def resume_dev(self, u_ptr, vx_ptr, vy_ptr, vz_ptr=None, stream=None, callback=None) -> int:
        """iteration_count more iterations from the current state."""
        return _check(lib().tgvdct_tgv2_resume_dev(self._ctx, u_ptr, vx_ptr, vy_ptr, vz_ptr,
                                                   callback or CALLBACK(), None, stream))

    def request_stop(self):
        """Ask the loop running on this context (or the next one) to stop; thread-safe."""
        _check(lib().tgvdct_request_stop(self._ctx))

    def set_pipeline_wait_limit(self, limit_ns: int):
        """Limit of the pipelines' bounded waits (tgvdct_set_pipeline_wait_limit)."""
        _check(lib().tgvdct_set_pipeline_wait_limit(self._ctx, int(limit_ns)), allow_stop=False)

    def check_device_error(self, stream=None):
        _check(lib().tgvdct_check_device_error(self._ctx, stream), allow_stop=False)

    def process_dev(self, f_ptr, u_ptr, l_ptr, r_ptr, mask_ptr=None,
                    set_negative_values_to_zero=True, add_background_back=False,
                    log_domain=False, stream=None, callback=None) -> int:
        return _check(lib().tgvdct_process_dev(self._ctx, f_ptr, mask_ptr,
                                               int(set_negative_values_to_zero),
                                               int(add_background_back), int(log_domain), u_ptr,
                                               l_ptr, r_ptr, callback or CALLBACK(), None,
                                               stream))
