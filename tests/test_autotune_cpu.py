"""The batch-packing tuner: choice rule and on-disk cache (no GPU needed)."""
import json

from xlumina_gb300.autotune import BatchTuner


def test_smallest_batch_within_tolerance(tmp_path):
    t = BatchTuner(path=str(tmp_path / "a.json"), device_name="dev", tolerance=0.05)
    # throughput saturates at 8 requests per launch
    assert t.choose({1: 100.0, 2: 190.0, 4: 350.0, 8: 600.0, 16: 610.0, 32: 612.0}) == 8
    assert t.choose({1: 500.0, 2: 480.0}) == 1


def test_measures_once_then_caches(tmp_path):
    path = tmp_path / "tune.json"
    calls = []

    def measure(b):   # seconds per launch: fixed cost 1 ms + 0.1 ms per request -> favours big batches
        calls.append(b)
        return 1e-3 + 1e-4 * b

    t = BatchTuner(path=str(path), device_name="GB300", candidates=(1, 2, 4, 8), repeats=2)
    b = t.best_batch(("rs", 256, 256), measure)
    assert b == 8
    assert calls and set(calls) == {1, 2, 4, 8}
    n = len(calls)
    assert t.best_batch(("rs", 256, 256), measure) == 8
    assert len(calls) == n                      # cached: no new measurement
    assert t.best_batch(("rs", 256, 256), measure, max_batch=4) == 4
    data = json.loads(path.read_text())
    assert data["GB300"]["rs|256|256"]["batch"] == 8
    # a fresh tuner (another process) reads the cache; another device does not share it
    t2 = BatchTuner(path=str(path), device_name="GB300")
    assert t2.cached(("rs", 256, 256))["batch"] == 8
    assert BatchTuner(path=str(path), device_name="other").cached(("rs", 256, 256)) is None


def test_large_fields_pack_one(tmp_path):
    # the GPU is full with one request: time grows linearly with the batch
    t = BatchTuner(path=str(tmp_path / "t.json"), device_name="dev", candidates=(1, 2, 4), repeats=1)
    assert t.best_batch(("vrs", 2048, 2048), lambda b: 5e-4 * b) == 1


def test_variant_tuner_picks_fastest_and_caches(tmp_path):
    from xlumina_gb300.autotune import VariantTuner
    selected = {}
    times = {0: 2.0e-3, 1: 1.2e-3, 2: 1.5e-3}
    t = VariantTuner(path=str(tmp_path / "v.json"), device_name="GB300", repeats=2,
                     count=lambda p, l: 3, select=lambda p, l, v: selected.__setitem__((p, l), v))
    calls = []

    def measure():
        v = selected[(0, 12)]
        calls.append(v)
        return times[v]

    r = t.best_variant(0, 12, measure)
    assert r["variant"] == 1 and selected[(0, 12)] == 1 and not r["cached"]
    assert set(calls) == {0, 1, 2}
    n = len(calls)
    t2 = VariantTuner(path=str(tmp_path / "v.json"), device_name="GB300",
                      count=lambda p, l: 3, select=lambda p, l, v: selected.__setitem__((p, l), v))
    selected[(0, 12)] = 0
    r2 = t2.best_variant(0, 12, measure)
    assert r2 == {"variant": 1, "ms": {}, "cached": True} and selected[(0, 12)] == 1 and len(calls) == n
    # forced: measured again
    assert t2.best_variant(0, 12, measure, force=True)["variant"] == 1 and len(calls) > n


def test_latency_bound_limits_the_batch(tmp_path):
    """With a bound on the launch time the tuner gives up throughput for latency."""
    t = BatchTuner(path=str(tmp_path / "l.json"), device_name="dev", candidates=(1, 2, 4, 8, 16), repeats=1)
    measure = lambda b: 1e-3 + 1e-3 * b   # noqa: E731  (throughput keeps rising with the batch)
    assert t.best_batch(("vrs", 1024, 1024), measure) == 16
    assert t.best_batch(("vrs", 1024, 1024), measure, max_launch_s=5.5e-3) == 4
    assert t.best_batch(("vrs", 1024, 1024), measure, max_launch_s=1e-4) == 1   # none fits: the smallest
    # cached per bound
    assert t.best_batch(("vrs", 1024, 1024), lambda b: 1.0, max_launch_s=5.5e-3) == 4
