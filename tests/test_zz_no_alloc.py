"""foort_gpu_integrate_noalloc: integration without any device allocation by the library.

The entry point runs the same kernels as foort_gpu_integrate, with its launch counters
and image constants in a statically declared device array instead of cudaMalloc'd
memory. Each pixel's integration does not depend on where its constants live, so the
results must equal those of foort_gpu_integrate bit for bit. That is stricter than the
parity tolerances of the other GPU tests. Two different runs go through the entry point
back to back on one stream: the second overwrites the array the first one used.

This file is collected last and also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from foort_gb300 import abi, workloads


def _noalloc(lib, desc, d_px, n, d_out, stream, stats=None):
    return lib.foort_gpu_integrate_noalloc(C.byref(desc), C.c_void_p(d_px), n, C.c_void_p(d_out),
                                           C.c_void_p(stream), C.byref(stats) if stats is not None else None)


def _many_images(n_images, side):
    wl = workloads.c3(precision=abi.PREC_MIXED, n_images=n_images)
    px = np.concatenate([abi.square_pixels(side, image=i) for i in range(n_images)])
    return wl, px


def test_rejects_more_images_than_the_array_holds(engine_lib):
    """Checked before any CUDA call, so no GPU is needed."""
    wl, _ = _many_images(4, 2)
    images = [wl.images[i % 4] for i in range(abi.NOALLOC_MAX_IMAGES + 1)]
    keep = abi.attach_images(wl.desc, images)
    rc = _noalloc(engine_lib, wl.desc, 0, 0, 0, 0)
    msg = engine_lib.foort_gpu_last_error(None).decode()
    del keep
    assert rc == abi.FOORT_E_BADARG
    assert "exceeds" in msg and str(abi.NOALLOC_MAX_IMAGES) in msg


def test_rejects_null_buffers(engine_lib):
    wl = workloads.c1()
    assert _noalloc(engine_lib, wl.desc, 0, 10, 0, 0) == abi.FOORT_E_BADARG


@pytest.mark.gpu
def test_noalloc_equals_integrate_on_two_calls_in_a_row(engine_lib):
    import torch

    import foort_gb300
    foort_gb300.check_layout()
    runs = []
    # First call: mixed precision, 8 Kerr images (spins and inclinations differ).
    wl_a, px_a = _many_images(8, 24)
    runs.append((wl_a, px_a))
    # Second call: FP64, one Kerr image, a different pixel count.
    wl_b = workloads.c1(precision=abi.PREC_FP64)
    runs.append((wl_b, abi.square_pixels(50)))

    expected = []
    for wl, px in runs:
        with foort_gb300.Engine(wl.desc) as e:
            expected.append(e.integrate(px))

    # The test allocates the caller's buffers; the entry point allocates nothing.
    dev_bufs = []
    for wl, px in runs:
        d_px = torch.from_numpy(px.view(np.uint8).copy()).to("cuda")
        d_out = torch.zeros(len(px) * abi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        dev_bufs.append((d_px, d_out))
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    stats = abi.Stats()
    # Back to back on one stream; only the second call waits (stats given).
    for k, (wl, px) in enumerate(runs):
        d_px, d_out = dev_bufs[k]
        rc = _noalloc(engine_lib, wl.desc, d_px.data_ptr(), len(px), d_out.data_ptr(), stream.cuda_stream,
                      stats if k == 1 else None)
        assert rc == 0, engine_lib.foort_gpu_last_error(None).decode()
    torch.cuda.synchronize()
    assert stats.geodesics == len(runs[1][1]) and stats.status == 0 and stats.steps > 0

    for k, (wl, px) in enumerate(runs):
        got = dev_bufs[k][1].cpu().numpy().view(abi.RESULT_DTYPE)
        want = expected[k]
        assert len(got) == len(want)
        for name in abi.RESULT_DTYPE.names:
            np.testing.assert_array_equal(got[name], want[name], err_msg=f"call {k}, field {name}")
        print(f"call {k}: {len(px)} pixels, {np.bincount(got['term'], minlength=5)} terminations, identical")
