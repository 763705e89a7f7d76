"""The batched form's autotuner search and its persistent cache, on the CPU
(cadr_autotune_with with a stand-in timer): a key that is in the cache is
answered without timing anything."""
import json

import pytest

from cadr_gb300 import lib


def _timer(calls):
    def t(tu):
        calls.append((tu.block_threads, tu.items_per_thread, tu.ctas_per_sm))
        # Fastest at (256, 8, 4).
        return 1.0 + abs(tu.block_threads - 256) / 100 + abs(tu.items_per_thread - 8) / 10 + abs(tu.ctas_per_sm - 4) / 10
    return t


def test_second_call_with_the_same_key_does_no_timing(cuda_lib, tmp_path):
    path = str(tmp_path / "tuning.json")
    calls = []
    best, ms, hit = lib.autotune_with(path, "GB300|sms=152|shape=1", _timer(calls))
    assert not hit and (best.block_threads, best.items_per_thread, best.ctas_per_sm) == (256, 8, 4)
    assert ms == pytest.approx(1.0)
    n_first = len(calls)
    # every supported tuning once: 24 persistent shapes and the three-launch form
    assert n_first == 25 and len(set(calls)) == 24
    d = json.load(open(path))
    assert d["version"] == 2
    assert d["entries"]["GB300|sms=152|shape=1"] == {"block_threads": 256, "items_per_thread": 8,
                                                      "ctas_per_sm": 4, "form": 0, "ms": 1.0}
    calls.clear()
    best2, ms2, hit2 = lib.autotune_with(path, "GB300|sms=152|shape=1", _timer(calls))
    assert hit2 and calls == [] and ms2 == pytest.approx(1.0)
    assert (best2.block_threads, best2.items_per_thread, best2.ctas_per_sm) == (256, 8, 4)


def test_other_keys_are_timed_and_kept_beside(cuda_lib, tmp_path):
    path = str(tmp_path / "tuning.json")
    lib.autotune_with(path, "A", _timer([]))
    calls = []
    _, _, hit = lib.autotune_with(path, "B", _timer(calls))
    assert not hit and len(calls) == 25
    assert set(json.load(open(path))["entries"]) == {"A", "B"}


def test_no_cache_times_every_call(cuda_lib):
    calls = []
    lib.autotune_with(None, "k", _timer(calls))
    lib.autotune_with(None, "k", _timer(calls))
    assert len(calls) == 50


def test_unreadable_cache_is_replaced(cuda_lib, tmp_path):
    path = tmp_path / "tuning.json"
    path.write_text("not json at all\n")
    calls = []
    _, _, hit = lib.autotune_with(str(path), "k", _timer(calls))
    assert not hit and len(calls) == 25
    assert "k" in json.load(open(path))["entries"]


def test_store_and_lookup(cuda_lib, tmp_path):
    import ctypes as C
    path = str(tmp_path / "t.json").encode()
    L = cuda_lib
    t = lib.Tuning(256, 8, 2, 1)
    lib.check(L.cadr_tuning_cache_store(path, b"GPU X|driver=13000", C.byref(t), 0.5))
    out, ms = lib.Tuning(), C.c_float()
    lib.check(L.cadr_tuning_cache_lookup(path, b"GPU X|driver=13000", C.byref(out), C.byref(ms)))
    assert (out.block_threads, out.items_per_thread, out.ctas_per_sm, out.form, ms.value) == (256, 8, 2, 1, 0.5)
    assert L.cadr_tuning_cache_lookup(path, b"other", C.byref(out), None) == lib.NOT_READY
    assert L.cadr_tuning_cache_store(path, b'bad"key', C.byref(t), 0.5) == lib.INVALID_ARG
