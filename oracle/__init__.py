"""TEST INFRASTRUCTURE — Python bindings of the CPU oracle.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may use
this package, and only to check the CUDA path.  ``liboracle.so`` is the C++ restatement of
the reference's TGV-DCT kernel sequence (``tgv_oracle.hpp``); ``libref_cpu.so``
(optional, ``oracle/_ref``) is the reference's own CUDA source compiled for the CPU
by ``ref_cpu/build_ref_cpu.py`` where the reference tree is available.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "liboracle.so")
_REF_PATH = os.path.join(HERE, "_ref", "libref_cpu.so")

_lib = None
_ref = None

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u = ctypes.c_uint
_d = ctypes.c_double


def build() -> str:
    """Compile liboracle.so with the committed Makefile (g++, OpenMP)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_set_threads.restype = ctypes.c_int
        for suf, p in (("f32", _f32p), ("f64", _f64p)):
            fn = getattr(L, f"oracle_tgv2_deshade_{suf}")
            fn.argtypes = [p, _u, _u, _u, _d, _d, _d, _u, _d, _d, _d, ctypes.c_int, ctypes.c_int,
                           p, p, p, p]
            fn.restype = _u
            fn = getattr(L, f"oracle_divergence_{suf}")
            fn.argtypes = [p, p, p, _u, _u, _u, p]
            for name in ("cosine_transform", "inverse_cosine_transform", "solve_poisson"):
                fn = getattr(L, f"oracle_{name}_{suf}")
                fn.argtypes = [p, _u, _u, _u, p]
            fn = getattr(L, f"oracle_integrate_poisson_dct_{suf}")
            fn.argtypes = [p, p, p, _u, _u, _u, p]
            fn = getattr(L, f"oracle_deshade_epilogue_{suf}")
            fn.argtypes = [p, p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, p]
            fn = getattr(L, f"oracle_masked_deshade_epilogue_{suf}")
            fn.argtypes = [p, p, p, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, p]
            fn = getattr(L, f"oracle_convergence_test_{suf}")
            fn.argtypes = [p, ctypes.c_void_p, _u, _u, _u, _d, _d, _d, _u, _u, p, p, _u, p]
            fn.restype = _u
            fn = getattr(L, f"oracle_tgv2_deshade_masked_{suf}")
            fn.argtypes = [p, p, _u, _u, _u, _d, _d, _d, _u, _d, _d, _d, ctypes.c_int,
                           ctypes.c_int, p, p, p, p]
            fn.restype = _u
        for suf in ("f32", "f64"):
            fn = getattr(L, f"oracle_tgv2_step_{suf}")
            fn.argtypes = [ctypes.c_void_p, _u, _u, _u, _d, _d, _d, _u, _d, _d, _d, ctypes.c_int,
                           ctypes.c_int]
        L.oracle_resize_bspline3_f32.argtypes = [_f32p, _u, _u, _u, _f32p, _u, _u, _u]
        L.oracle_resize_factor_extent.argtypes = [_u, ctypes.c_float]
        L.oracle_resize_factor_extent.restype = _u
        vp = ctypes.c_void_p
        L.oracle_tgv2_gradient_f64.argtypes = [_f64p, _u, _u, _u, _d, _d, _d, _u, _d, _d, _d,
                                               ctypes.c_int, vp, vp, vp, vp, _f64p, _f64p, vp]
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    return lib().oracle_set_threads(int(n))


def _dt(dtype):
    dtype = np.dtype(dtype)
    if dtype == np.float32:
        return "f32"
    if dtype == np.float64:
        return "f64"
    raise TypeError(f"unsupported dtype {dtype}")


def _shape3(a: np.ndarray):
    """(depth, height, width) array -> (w, h, d); 2-D arrays are (height, width)."""
    if a.ndim == 2:
        return a.shape[1], a.shape[0], 1
    if a.ndim == 3:
        return a.shape[2], a.shape[1], a.shape[0]
    raise ValueError("expected a 2-D (H, W) or 3-D (D, H, W) array")


def tgv2_deshade(f, lambda_=1.0, alpha0=2.0, alpha1=1.0, iterations=100, *, tau=0.0, sigma=0.0,
                 theta=1.0, data_term="l1", two_d=False, dtype=np.float64):
    """Run the restated TGV2 loop.  Returns (u, v_x, v_y, v_z) shaped like f."""
    f = np.ascontiguousarray(f, dtype=dtype)
    w, h, d = _shape3(f)
    u = np.empty_like(f)
    vx, vy, vz = np.empty_like(f), np.empty_like(f), np.empty_like(f)
    dt = 0 if data_term in ("l1", 0) else 1
    getattr(lib(), f"oracle_tgv2_deshade_{_dt(dtype)}")(
        f, w, h, d, lambda_, alpha0, alpha1, iterations, tau, sigma, theta, dt, int(two_d),
        u, vx, vy, vz)
    return u, vx, vy, vz


# the persistent fields of one loop state, in the order oracle_tgv2_step_* takes them
STATE_FIELDS = ("f", "u", "u_bar", "p_x", "p_y", "p_z", "v_x", "v_y", "v_z", "vbar_x", "vbar_y",
                "vbar_z", "q_xx", "q_yy", "q_zz", "q_xy", "q_xz", "q_yz")


def tgv2_initial_state(f):
    """The loop's starting state: u = u_bar = f, every other field 0 (a dict of arrays
    keyed by STATE_FIELDS, shaped like f)."""
    f = np.ascontiguousarray(f)
    st = {k: np.zeros_like(f) for k in STATE_FIELDS}
    st["f"][...] = f
    st["u"][...] = f
    st["u_bar"][...] = f
    return st


def tgv2_step(state, iterations=1, lambda_=1.0, alpha0=2.0, alpha1=1.0, *, tau=0.0, sigma=0.0,
              theta=1.0, data_term="l1", two_d=False):
    """Advances a loop state (a dict from tgv2_initial_state, updated in place) by
    `iterations` iterations of the restated loop: the arithmetic of tgv2_deshade."""
    arrs = [state[k] for k in STATE_FIELDS]
    dtype = arrs[0].dtype
    for a in arrs:
        if a.dtype != dtype or not a.flags.c_contiguous or a.shape != arrs[0].shape:
            raise ValueError("state fields must be C-contiguous arrays of one shape and dtype")
    w, h, d = _shape3(arrs[0])
    ptrs = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    dt = 0 if data_term in ("l1", 0) else 1
    getattr(lib(), f"oracle_tgv2_step_{_dt(dtype)}")(
        ptrs, w, h, d, lambda_, alpha0, alpha1, iterations, tau, sigma, theta, dt, int(two_d))
    return state


def divergence(vx, vy, vz):
    vx = np.ascontiguousarray(vx)
    dtype = vx.dtype
    vy = np.ascontiguousarray(vy, dtype=dtype)
    vz = np.ascontiguousarray(vz if vz is not None else np.zeros_like(vx), dtype=dtype)
    w, h, d = _shape3(vx)
    out = np.empty_like(vx)
    getattr(lib(), f"oracle_divergence_{_dt(dtype)}")(vx, vy, vz, w, h, d, out)
    return out


def _unary(name, x):
    x = np.ascontiguousarray(x)
    w, h, d = _shape3(x)
    out = np.empty_like(x)
    getattr(lib(), f"oracle_{name}_{_dt(x.dtype)}")(x, w, h, d, out)
    return out


def cosine_transform(x):
    return _unary("cosine_transform", x)


def inverse_cosine_transform(x):
    return _unary("inverse_cosine_transform", x)


def solve_poisson(x):
    return _unary("solve_poisson", x)


def integrate_poisson_dct(vx, vy, vz):
    vx = np.ascontiguousarray(vx)
    dtype = vx.dtype
    vy = np.ascontiguousarray(vy, dtype=dtype)
    vz = np.ascontiguousarray(vz if vz is not None else np.zeros_like(vx), dtype=dtype)
    w, h, d = _shape3(vx)
    out = np.empty_like(vx)
    getattr(lib(), f"oracle_integrate_poisson_dct_{_dt(dtype)}")(vx, vy, vz, w, h, d, out)
    return out


def deshade_epilogue(u, l, mask=None, set_negative_values_to_zero=True, add_background_back=False):
    """r = u - l, optional mask (also applied to l, returned), clamp, add-back."""
    u = np.ascontiguousarray(u)
    l = np.array(l, dtype=u.dtype, copy=True, order="C")
    r = np.empty_like(u)
    mptr = None
    if mask is not None:
        mask = np.ascontiguousarray(mask, dtype=u.dtype)
        mptr = mask.ctypes.data_as(ctypes.c_void_p)
    getattr(lib(), f"oracle_deshade_epilogue_{_dt(u.dtype)}")(
        u, l, mptr, int(set_negative_values_to_zero), int(add_background_back), u.size, r)
    return r, l


def process_tgv2_l1(f, lambda_=1.0, alpha0=2.0, alpha1=1.0, iterations=100, *,
                    set_negative_values_to_zero=True, data_term="l1", two_d=False,
                    tau=0.0, sigma=0.0, dtype=np.float64):
    """The whole deshade: loop, Poisson-DCT integration of v, r = u - l (+clamp).

    Returns (denoised u, shading l, deshaded r) — the three images of
    TGVDeshadeProcessor::processTGV2L1GPUCuda (TGVDeshadeProcessor.cpp:122-166).
    """
    u, vx, vy, vz = tgv2_deshade(f, lambda_, alpha0, alpha1, iterations, tau=tau, sigma=sigma,
                                 data_term=data_term, two_d=two_d, dtype=dtype)
    l = integrate_poisson_dct(vx, vy, vz)
    r, _ = deshade_epilogue(u, l, None, set_negative_values_to_zero, False)
    return u, l, r


def tgv2_deshade_masked(f, mask, lambda_=1.0, alpha0=2.0, alpha1=1.0, iterations=100, *,
                        tau=0.0, sigma=0.0, theta=1.0, data_term="l1", two_d=None,
                        dtype=np.float64):
    """The masked loop: only voxels with mask >= 1 are updated.  two_d defaults to
    depth == 1, the choice TGVDeshadeMaskedProcessor makes.  Returns (u, v_x, v_y, v_z)."""
    f = np.ascontiguousarray(f, dtype=dtype)
    mask = np.ascontiguousarray(mask, dtype=dtype)
    w, h, d = _shape3(f)
    if two_d is None:
        two_d = d == 1
    u = np.empty_like(f)
    vx, vy, vz = np.empty_like(f), np.empty_like(f), np.empty_like(f)
    dt = 0 if data_term in ("l1", 0) else 1
    getattr(lib(), f"oracle_tgv2_deshade_masked_{_dt(dtype)}")(
        f, mask, w, h, d, lambda_, alpha0, alpha1, iterations, tau, sigma, theta, dt,
        int(two_d), u, vx, vy, vz)
    return u, vx, vy, vz


def masked_deshade_epilogue(u, l, mask, set_negative_values_to_zero=True,
                            add_background_back=False):
    """The masked processor's tail: returns (r, l * mask)."""
    u = np.ascontiguousarray(u)
    l = np.array(l, dtype=u.dtype, copy=True, order="C")
    mask = np.ascontiguousarray(mask, dtype=u.dtype)
    r = np.empty_like(u)
    getattr(lib(), f"oracle_masked_deshade_epilogue_{_dt(u.dtype)}")(
        u, l, mask, int(set_negative_values_to_zero), int(add_background_back), u.size, r)
    return r, l


def process_tgv2_l1_masked(f, mask, lambda_=1.0, alpha0=2.0, alpha1=1.0, iterations=100, *,
                           set_negative_values_to_zero=True, add_background_back=False,
                           tau=0.0, sigma=0.0, dtype=np.float64):
    """TGVDeshadeMaskedProcessor::processTGV2L1GPUCuda (TGVDeshadeMaskedProcessor.cpp:77-330):
    the masked loop (2-D operators when depth == 1), the Poisson-DCT integration of v,
    then the masked epilogue.  Returns (u, l, r)."""
    u, vx, vy, vz = tgv2_deshade_masked(f, mask, lambda_, alpha0, alpha1, iterations, tau=tau,
                                        sigma=sigma, dtype=dtype)
    l = integrate_poisson_dct(vx, vy, vz)
    r, l = masked_deshade_epilogue(u, l, mask, set_negative_values_to_zero, add_background_back)
    return u, l, r


def convergence_test(f, lambda_=1.0, alpha0=2.0, alpha1=1.0, iterations=20, interval=1,
                     mask=None, dtype=np.float64):
    """TGVDeshadeProcessor::processTGV2L1DeshadeCuda_convergenceTest(+Metric): returns
    (ncc history, time-TV history, (TV of the NCC series, TV of the time-TV series))."""
    f = np.ascontiguousarray(f, dtype=dtype)
    w, h, d = _shape3(f)
    cap = max(1, iterations // max(interval, 1))
    ncc, tv, mt = np.zeros(cap, dtype), np.zeros(cap, dtype), np.zeros(2, dtype)
    mptr = None
    if mask is not None:
        mask = np.ascontiguousarray(mask, dtype=dtype)
        mptr = mask.ctypes.data_as(ctypes.c_void_p)
    k = getattr(lib(), f"oracle_convergence_test_{_dt(dtype)}")(
        f, mptr, w, h, d, lambda_, alpha0, alpha1, iterations, interval, ncc, tv, cap, mt)
    return ncc[:k], tv[:k], mt


def tgv2_gradient(f, lambda_=1.0, alpha0=2.0, alpha1=1.0, iterations=10, *, grad_u=None,
                  grad_v=None, data_term="l1", tau=0.0, sigma=0.0, theta=1.0):
    """FP64 reverse mode of the 3-D loop: returns (u_K, dL/df, dL/d(lambda, alpha0, alpha1))
    for the loss gradient grad_u = dL/du_K (and grad_v = (dL/dv_x, dL/dv_y, dL/dv_z))."""
    f = np.ascontiguousarray(f, dtype=np.float64)
    w, h, d = _shape3(f)
    gf = np.empty_like(f)
    gp = np.zeros(3)
    u = np.empty_like(f)

    def ptr(a):
        return None if a is None else np.ascontiguousarray(a, np.float64).ctypes.data_as(
            ctypes.c_void_p)

    keep = [None if a is None else np.ascontiguousarray(a, np.float64)
            for a in ([grad_u] + list(grad_v or (None, None, None)))]
    dt = 0 if data_term in ("l1", 0) else 1
    lib().oracle_tgv2_gradient_f64(f, w, h, d, lambda_, alpha0, alpha1, iterations, tau, sigma,
                                   theta, dt, *[ptr(a) for a in keep], gf, gp,
                                   u.ctypes.data_as(ctypes.c_void_p))
    return u, gf, gp


# ---------------------------------------------------------------------------
# The reference's own kernels compiled for the CPU (available where they were built).

def resize_factor_shape(shape, factor):
    """Output (depth, height, width) of ResizeProcessor::process(image, factor)
    (ResizeProcessor.cpp:35-47)."""
    d, h, w = shape
    e = lib().oracle_resize_factor_extent
    return (e(d, factor), e(h, factor), e(w, factor))


def resize_bspline3(image, shape):
    """ResizeProcessor::process(image, width, height, depth, BSpline3) restated with
    ITK's cubic B-spline resample (resize_oracle.hpp).  shape is (depth, height,
    width); float32 in and out, FP64 inside."""
    x = np.ascontiguousarray(image, dtype=np.float32)
    w, h, d = _shape3(x)
    D, H, W = shape
    out = np.empty((D, H, W) if x.ndim == 3 else (H, W), dtype=np.float32)
    lib().oracle_resize_bspline3_f32(x, w, h, d, out, W, H, D)
    return out


def process_tgvk_l1_downsampled(f, downsampling_factor, lambda_, order, alpha, iterations, *,
                                mask=None, set_negative_values_to_zero=True,
                                add_background_back=False, not_masked=False,
                                calculate_div_v=False):
    """TGVKDeshadeDownsampledProcessor::processTGVKL1Cuda
    (tgvk_deshade_downsampled/TGVKDeshadeDownsampledProcessor.cpp:30-129), or with
    not_masked the NotMasked variant (TGVKDeshadeDownsampledNotMaskedProcessor.cpp:30-129),
    for order 2, the order the reference hands to its TGV2 processors
    (TGVKDeshadeMaskedProcessor.cpp:98-103, TGVKDeshadeProcessor.cpp:137-147: alpha0 =
    alpha[1], alpha1 = alpha[0]).  Float32 throughout, as the reference's images.
    Returns (denoised, shading, deshaded, div_v or None)."""
    if order != 2:
        raise ValueError("only order 2 (TGV2) is restated")
    f = np.ascontiguousarray(f, dtype=np.float32)
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
    one = np.float32(1)
    a0, a1 = float(alpha[1]), float(alpha[0])
    clamp, add_back = set_negative_values_to_zero, add_background_back
    background = None
    if not not_masked:
        if add_back and m is not None:
            background = f * (one - m)
        fin = f * m if m is not None else f
    else:
        fin = f

    def down(x):
        if downsampling_factor == 1:
            return x
        return resize_bspline3(x, resize_factor_shape(_dhw(x), downsampling_factor))

    ds = down(fin)
    dsm = None if m is None else down(m)
    two_d = _dhw(ds)[0] == 1
    if not not_masked:
        inner_mask = dsm if dsm is not None else np.ones_like(ds)
        u, vx, vy, vz = tgv2_deshade_masked(ds, inner_mask, lambda_, a0, a1, iterations,
                                            dtype=np.float32)
        l = integrate_poisson_dct(vx, vy, vz)
        _, l = masked_deshade_epilogue(u, l, inner_mask, clamp, add_back)
    else:
        u, vx, vy, vz = tgv2_deshade(ds, lambda_, a0, a1, iterations, two_d=two_d,
                                     dtype=np.float32)
        l = integrate_poisson_dct(vx, vy, vz)
        _, l = deshade_epilogue(u, l, dsm, clamp, add_back)
    div_v = divergence(vx, vy, vz) if calculate_div_v else None

    def up(x):
        if downsampling_factor == 1:
            return x
        return resize_bspline3(x, _dhw(f))

    denoised = up(u)
    shading = up(l)
    deshaded = fin - shading
    if not not_masked:
        if m is not None:
            shading = shading * m
            deshaded = deshaded * m
        if add_back and m is not None:
            deshaded = deshaded + background
    else:
        if m is not None:
            deshaded = deshaded * m
        if add_back and m is not None:
            deshaded = deshaded + fin * (one - m)
    if clamp:
        deshaded = np.where(deshaded < 0, np.float32(0), deshaded)
    if div_v is not None:
        div_v = up(div_v)
    return denoised, shading, deshaded, div_v


def _dhw(x):
    return (1,) + x.shape if x.ndim == 2 else x.shape


def ref_available() -> bool:
    return os.path.exists(_REF_PATH)


def ref() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        if not ref_available():
            raise FileNotFoundError(
                "oracle/_ref/libref_cpu.so is missing; run oracle/ref_cpu/build_ref_cpu.py "
                "where the reference sources are available")
        R = ctypes.CDLL(_REF_PATH)
        f = ctypes.c_float
        R.ref_tgv2_l1_deshade_f32.argtypes = [_f32p, _u, _u, _u, f, f, f, _u, _f32p, _f32p,
                                              _f32p, _f32p]
        R.ref_tgv2_l1_deshade_2d_f32.argtypes = [_f32p, _u, _u, f, f, f, _u, _f32p, _f32p, _f32p]
        R.ref_tgv2_denoise_f32.argtypes = [ctypes.c_int, _f32p, _u, _u, _u, f, f, f, _u, _f32p]
        R.ref_process_tgv2_l1_f32.argtypes = [_f32p, _u, _u, _u, f, f, f, _u, ctypes.c_int,
                                              _f32p, _f32p, _f32p]
        R.ref_convergence_test_f32.argtypes = [_f32p, ctypes.c_void_p, _u, _u, _u, f, f, f, _u,
                                               _u, _f32p, _f32p, _u, _f32p]
        R.ref_convergence_test_f32.restype = _u
        R.ref_tgv2_l1_deshade_masked_f32.argtypes = [_f32p, _f32p, _u, _u, _u, f, f, f, _u,
                                                     _f32p, _f32p, _f32p, _f32p]
        R.ref_process_tgv2_l1_masked_f32.argtypes = [_f32p, _f32p, _u, _u, _u, f, f, f, _u,
                                                     ctypes.c_int, ctypes.c_int, _f32p, _f32p,
                                                     _f32p]
        for suf, p in (("f32", _f32p), ("f64", _f64p)):
            getattr(R, f"ref_divergence_{suf}").argtypes = [p, p, p, _u, _u, _u, p]
            for name in ("cosine_transform", "inverse_cosine_transform", "solve_poisson"):
                getattr(R, f"ref_{name}_{suf}").argtypes = [p, _u, _u, _u, p]
            getattr(R, f"ref_integrate_poisson_dct_{suf}").argtypes = [p, p, p, _u, _u, _u, p]
        _ref = R
    return _ref
