"""The autotuner's launch-shape cache (include/foort_gpu.h foort_tune_*): keys, size
buckets, validation, and the text file it persists to. None of this needs a GPU; the
search itself is tested in test_gpu_tune.py."""
import pytest

import foort_gb300 as fg
from foort_gb300 import abi, workloads


@pytest.fixture(autouse=True)
def lib(engine_lib):
    fg.tune_clear()
    yield engine_lib
    fg.tune_clear()


def test_size_buckets_are_floor_log2(lib):
    for n, b in [(0, 0), (1, 0), (2, 1), (3, 1), (4, 2), (1023, 9), (1024, 10), (1025, 10), (26547, 14),
                 (1 << 40, 40), ((1 << 40) + 5, 40)]:
        assert lib.foort_tune_bucket(n) == b, n


def test_keys_name_the_kernel_variant_and_the_bucket():
    d = workloads.c2(abi.PREC_MIXED).desc
    k = fg.tune_key(d, 152, 3000)
    assert k == "sm152:m0:i0:p1:r0:d0:f0:b11"
    assert fg.tune_key(d, 152, 2048) == k and fg.tune_key(d, 152, 4096) != k
    assert fg.tune_key(d, 148, 3000) != k
    d.mixed_options = abi.MIXED_FP64_DECISIONS
    assert fg.tune_key(d, 152, 3000) == "sm152:m0:i0:p1:r0:d1:f0:b11"
    d.mixed_options = abi.MIXED_FP64_NEAR_HORIZON
    d.mixed_fp64_margin = 2.0
    assert fg.tune_key(d, 152, 3000).endswith(":f1:b11")
    d.mixed_options = abi.MIXED_FP64_TURNING_POINTS
    assert fg.tune_key(d, 152, 3000).endswith(":f2:b11")
    d4 = workloads.c4(abi.PREC_MIXED).desc
    assert fg.tune_key(d4, 152, 1 << 20) == "sm152:m3:i1:p1:r0:d0:f0:b20"


def test_put_get_and_validation():
    key = "sm152:m0:i0:p1:r0:d0:f0:b11"
    assert fg.tune_get(key) is None
    fg.tune_put(key, block_size=64, blocks_per_sm=0, lanes=2, refill_steps=4, poll_steps=512, ms=12.5)
    got = fg.tune_get(key)
    assert got == {"block_size": 64, "blocks_per_sm": 0, "lanes": 2, "refill_steps": 4, "poll_steps": 512, "ms": 12.5}
    assert fg.tune_count() == 1
    bad = [dict(block_size=48, lanes=1, refill_steps=1, poll_steps=1),
           dict(block_size=256, lanes=1, refill_steps=1, poll_steps=1),
           dict(block_size=64, lanes=3, refill_steps=1, poll_steps=1),
           dict(block_size=64, lanes=1, refill_steps=0, poll_steps=1),
           dict(block_size=64, lanes=1, refill_steps=1, poll_steps=0)]
    for s in bad:
        with pytest.raises(fg.FoortError):
            fg.tune_put("k", **s)
    with pytest.raises(fg.FoortError):
        fg.tune_put("has space", block_size=64, lanes=1, refill_steps=1, poll_steps=1)
    assert fg.tune_count() == 1


def test_cache_file_round_trip_and_merge(tmp_path):
    shapes = {"sm152:m0:i0:p1:r0:d0:f0:b14": dict(block_size=128, blocks_per_sm=0, lanes=2, refill_steps=1,
                                                  poll_steps=512, ms=101.25),
              "sm152:m3:i1:p1:r0:d0:f0:b20": dict(block_size=32, blocks_per_sm=3, lanes=1, refill_steps=16,
                                                  poll_steps=2048, ms=0.1 + 0.2)}
    for k, s in shapes.items():
        fg.tune_put(k, **s)
    path = tmp_path / "shapes.txt"
    fg.tune_save(path)
    fg.tune_clear()
    assert fg.tune_count() == 0
    fg.tune_put("sm152:m1:i0:p1:r0:d0:f0:b3", block_size=32, lanes=1, refill_steps=1, poll_steps=1)
    fg.tune_load(path)
    assert fg.tune_count() == 3
    for k, s in shapes.items():
        assert fg.tune_get(k) == s  # %.17g keeps the doubles exact


def test_malformed_cache_file_is_rejected_whole(tmp_path):
    fg.tune_put("keep", block_size=64, lanes=1, refill_steps=1, poll_steps=1)
    path = tmp_path / "bad.txt"
    path.write_text("# foort launch-shape cache v1\nsm152:a 64 0 1 1 512 1.0\nsm152:b 64 0 5 1 512 1.0\n")
    with pytest.raises(fg.FoortError):
        fg.tune_load(path)
    assert fg.tune_count() == 1 and fg.tune_get("sm152:a") is None
    with pytest.raises(fg.FoortError):
        fg.tune_load(tmp_path / "missing.txt")
