"""The autotuner on the GPU (foort_gpu_autotune, foort_gpu_set_autotune): the search
returns a measured shape and caches it, later launches use it, and -- since every
geodesic goes through the same arithmetic wherever it runs -- every shape gives the
default shape's results bit for bit."""
import numpy as np
import pytest

from foort_gb300 import abi, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import foort_gb300
    from foort_gb300 import build as engine_build
    engine_build.build()
    foort_gb300.check_layout()
    return foort_gb300


def c2_sample(n, seed=3):
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(509 * 509, n, replace=False))
    px = np.zeros(n, dtype=abi.PIXEL_DTYPE)
    px["row"], px["col"], px["grid"] = idx // 509, idx % 509, 509
    return px


def assert_same(a, b, what):
    for name in abi.RESULT_DTYPE.names:
        np.testing.assert_array_equal(a[name], b[name], err_msg=f"{what}: {name}")


def test_every_launch_shape_gives_the_same_results(eng):
    import torch
    wl = workloads.c2(abi.PREC_MIXED)
    px = c2_sample(1500)
    with eng.Engine(wl.desc) as e:
        ref = e.integrate(px)
        for bs in (32, 64, 128):
            for lanes in (1, 2):
                e.set_launch(bs, 0)
                e.set_lanes(lanes)
                got = e.integrate(px)
                st = e.stats()
                assert st["block_size"] == bs and st["lanes_per_geodesic"] == lanes
                assert_same(got, ref, f"block {bs} lanes {lanes}")
        # regrouping cadence and poll interval through a cached shape
        e.set_launch(0, 0)
        e.set_lanes(0)
        eng.tune_clear()
        key = eng.tune_key(wl.desc, torch.cuda.get_device_properties(0).multi_processor_count, len(px))
        for refill, poll in ((16, 128), (4, 2048)):
            eng.tune_put(key, block_size=64, lanes=1, refill_steps=refill, poll_steps=poll)
            got = e.integrate(px)
            st = e.stats()
            assert (st["refill_steps"], st["poll_steps"], st["block_size"]) == (refill, poll, 64)
            assert_same(got, ref, f"refill {refill} poll {poll}")
        eng.tune_clear()


def test_autotune_caches_the_fastest_shape_and_launches_use_it(eng, tmp_path):
    import torch
    wl = workloads.c2(abi.PREC_MIXED)
    px = c2_sample(3000, seed=5)
    eng.tune_clear()
    with eng.Engine(wl.desc) as e:
        ref = e.integrate(px)
        d_px = torch.from_numpy(px.view(np.uint8).copy()).to("cuda")
        d_out = torch.zeros(len(px) * abi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        stream = torch.cuda.Stream()
        best = e.autotune(d_px.data_ptr(), len(px), d_out.data_ptr(), stream.cuda_stream)
        print("best shape", best)
        assert best["ms"] > 0 and best["lanes"] in (1, 2) and best["block_size"] in (32, 64, 128)
        assert_same(d_out.cpu().numpy().view(abi.RESULT_DTYPE), ref, "autotune's own launch")
        assert eng.tune_count() == 1
        shape = e.launch_shape(len(px))
        assert {k: shape[k] for k in ("block_size", "lanes", "refill_steps", "poll_steps")} == \
            {k: best[k] for k in ("block_size", "lanes", "refill_steps", "poll_steps")}
        got = e.integrate(px)
        st = e.stats()
        assert (st["block_size"], st["lanes_per_geodesic"], st["refill_steps"], st["poll_steps"]) == \
            (best["block_size"], best["lanes"], best["refill_steps"], best["poll_steps"])
        assert_same(got, ref, "tuned launch")
    path = tmp_path / "shapes.txt"
    eng.tune_save(path)
    eng.tune_clear()
    eng.tune_load(path)
    assert eng.tune_count() == 1
    # automatic mode: a launch without an entry searches first, in another size bucket
    px2 = c2_sample(700, seed=9)
    with eng.Engine(wl.desc) as e:
        ref2 = e.integrate(px2)
        e.set_autotune(True)
        got2 = e.integrate(px2)
        assert eng.tune_count() == 2
        assert_same(got2, ref2, "automatic search")
    eng.tune_clear()
