"""The host-buffer one-shot calls keep their last context and device buffers between
calls (tgvdct_release_cached frees them).  A call served by the kept context gives
the bits of a call on a fresh one: for a repeated input, a new input, new
parameters, a switch between entry points, and a call re-entered from an iteration
callback, and for concurrent calls from several threads."""
import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d

pytestmark = pytest.mark.gpu

SHAPE = (14, 20, 32)
P = pkg.TGVDeshadeProcessor
MP = pkg.TGVDeshadeMaskedProcessor


def _deshade(f, lam=1.5, it=40, **kw):
    return P.processTGV2L1GPUCuda(f, lam, 2.0, 1.0, it, log_domain=True, **kw)


def _fresh(fn):
    pkg.release_cached()
    return fn()


def _same(a, b):
    for x, y in zip(a, b):
        assert np.array_equal(x, y, equal_nan=True)


def test_kept_context_gives_the_bits_of_a_fresh_one(gpu_lib):
    fa = tissue_phantom_3d(*SHAPE, seed=31)
    fb = tissue_phantom_3d(*SHAPE, seed=32)
    ref_a = _fresh(lambda: _deshade(fa))
    again = _deshade(fa)                       # kept context, same input
    _same(ref_a, again)
    got_b = _deshade(fb)                       # kept context, new input
    ref_b = _fresh(lambda: _deshade(fb))
    _same(got_b, ref_b)
    assert not np.array_equal(ref_a[1], ref_b[1])
    got_lam = _deshade(fa, lam=0.7)            # new parameters: a new entry
    ref_lam = _fresh(lambda: _deshade(fa, lam=0.7))
    _same(got_lam, ref_lam)
    pkg.release_cached()


def test_entry_points_do_not_share_state(gpu_lib):
    f = tissue_phantom_3d(*SHAPE, seed=33)
    mask = np.zeros(SHAPE, np.float32)
    mask[2:-2, 3:-3, 4:-4] = 1.0
    ref_plain = _fresh(lambda: _deshade(f, it=30))
    ref_masked = _fresh(lambda: MP.processTGV2L1GPUCuda(f, 1.5, 2.0, 1.0, 30, mask=mask,
                                                         log_domain=True))
    ref_loop = _fresh(lambda: pkg.tgv2_l1_deshade_launch(np.log(f), 1.5, 30))
    pkg.release_cached()
    # interleaved, every call after the first finds the entry keyed by another call
    for _ in range(2):
        _same(MP.processTGV2L1GPUCuda(f, 1.5, 2.0, 1.0, 30, mask=mask, log_domain=True),
              ref_masked)
        _same(_deshade(f, it=30), ref_plain)
        _same(pkg.tgv2_l1_deshade_launch(np.log(f), 1.5, 30), ref_loop)
    pkg.release_cached()


def test_reentrant_call_from_the_callback(gpu_lib):
    """An iteration callback that itself calls a one-shot entry point gets a private
    context; the outer call keeps using the entry it holds."""
    f = tissue_phantom_3d(*SHAPE, seed=34)
    g = np.log(tissue_phantom_3d(*SHAPE, seed=35))
    ref_outer = _fresh(lambda: pkg.tgv2_l1_deshade_launch(np.log(f), 1.5, 40))
    ref_inner = _fresh(lambda: pkg.tgv2_denoise_launch(g, 1.5, 20))
    inner = []

    def cb(it, n, u, vx, vy, vz):
        inner.append(pkg.tgv2_denoise_launch(g, 1.5, 20))
        return False

    pkg.release_cached()
    out = pkg.tgv2_l1_deshade_launch(np.log(f), 1.5, 40, paint_iteration_interval=10,
                                     iteration_finished_callback=cb)
    _same(out, ref_outer)
    assert len(inner) >= 3
    for u in inner:
        assert np.array_equal(u, ref_inner)
    pkg.release_cached()


def test_concurrent_calls_from_several_threads(gpu_lib):
    """Four threads in the host-buffer call at once (ctypes releases the GIL): one gets
    the kept context, the others private ones; all give the bits of a fresh call."""
    import threading
    fs = [tissue_phantom_3d(*SHAPE, seed=40 + k) for k in range(4)]
    refs = [_fresh(lambda f=f: _deshade(f, it=60)) for f in fs]
    pkg.release_cached()
    got = [None] * len(fs)
    errors = []

    def work(k):
        try:
            got[k] = _deshade(fs[k], it=60)
        except Exception as e:  # reported below, on the main thread
            errors.append(e)

    for _ in range(2):
        threads = [threading.Thread(target=work, args=(k,)) for k in range(len(fs))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        assert not errors, errors
        for k in range(len(fs)):
            _same(got[k], refs[k])
    pkg.release_cached()
