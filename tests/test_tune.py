"""The autotuner's host logic and the library's tunable-parameter registry (no GPU needed)."""
import pytest

from pymoresane_gb300 import _native, tune


@pytest.fixture(autouse=True)
def _reset_knobs():
    tune.reset()
    yield
    tune.reset()


def test_registry_defaults_ranges_and_epoch():
    assert tune.current() == {"fft_four_step": 1, "fft_sq_fwd_ctas": 0, "fft_sq_col_ctas": 0, "fft_sq_inv_ctas": 0,
                              "iuwt_threads": 256, "iuwt_threads_wide": 256}
    e0 = _native.query("msn_tune_epoch")
    tune.set_values({"iuwt_threads": 128})
    assert tune.get("iuwt_threads") == 128 and _native.query("msn_tune_epoch") != e0
    e1 = _native.query("msn_tune_epoch")
    tune.set_values({"iuwt_threads": 128})           # unchanged value: same epoch
    assert _native.query("msn_tune_epoch") == e1
    for name, bad in (("iuwt_threads", 96), ("iuwt_threads", 512), ("fft_four_step", 2), ("fft_sq_col_ctas", -1)):
        with pytest.raises(ValueError):
            tune.set_values({name: bad})
    with pytest.raises(ValueError):
        _native.call("msn_tune_set", b"no_such_knob", 1)


def test_choose_keeps_the_fastest_candidate():
    cost = {256: 3.0, 128: 1.0, 64: 2.0}
    best, times = tune.choose("iuwt_threads", (256, 128, 64), lambda: cost[tune.get("iuwt_threads")])
    assert best == 128 and times == cost and tune.get("iuwt_threads") == 128


def test_cache_round_trip_and_apply(tmp_path, monkeypatch):
    path = str(tmp_path / "sub" / "tune.json")
    entry = {"device": "dev-a", "values": {"fft_four_step": 0, "iuwt_threads": 64}, "times_s": {}}
    tune.save_cache({"dev-a": entry, "dev-b": {"values": {"iuwt_threads": 128}}}, path)
    assert tune.load_cache(path)["dev-a"] == entry
    monkeypatch.setattr(tune, "device_key", lambda: "dev-a")
    monkeypatch.setattr(tune, "_applied", False)
    assert tune.ensure_applied(path) == entry["values"]
    assert tune.get("fft_four_step") == 0 and tune.get("iuwt_threads") == 64
    assert tune.ensure_applied(path) is None          # once per process
    assert tune.load_cache(str(tmp_path / "missing.json")) == {}


def test_concurrent_values_nest_and_restore():
    # executors with several workers set the concurrency values while any of them runs; the
    # last to stop restores what was there before
    tune.set_values({"iuwt_threads": 256})
    tune.enter_concurrent()
    assert tune.get("iuwt_threads") == tune.CONCURRENT["iuwt_threads"]
    tune.enter_concurrent()
    tune.leave_concurrent()
    assert tune.get("iuwt_threads") == tune.CONCURRENT["iuwt_threads"]
    tune.leave_concurrent()
    assert tune.get("iuwt_threads") == 256
