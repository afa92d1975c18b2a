"""The autotuner's cache (superintervals_gb300/autotune.py) on the host: a first call runs
the library's tuner and stores its choice; a second call with the same key applies it
without tuning; a choice that kept the automatic tile size restores it (-1)."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


class _FakeLib:
    def __init__(self, choice):
        self.choice = choice
        self.tuned = 0
        self.params = []

    def autotuneBatchedGpu(self, h, qs, qe, qc, nq, sample, flags, buf, n):
        self.tuned += 1
        buf.value = json.dumps(self.choice).encode()
        return 0

    def setBatchedParamsGpu(self, h, tile, cap, long_len, split):
        self.params.append((tile, cap, long_len, split))
        return 0


class _FakeIndex:
    def __init__(self, lib):
        self.h, self.lib, self.bits, self.ub = object(), lib, 32, None

    def size(self):
        return 1_000_000

    def n_contigs(self):
        return 24

    def set_upper_bound(self, mode):
        self.ub = mode


def _choice(tile_auto):
    return {"upper_bound": 2, "tile_queries": 128, "tile_auto": tile_auto, "tile_candidates": 2048,
            "split_len": 2048, "long_query_len": 16384, "sample_queries": 0, "sample_ms": 1.0, "trials": 9}


def test_tune_then_cached_apply(tmp_path):
    from superintervals_gb300 import autotune
    for tile_auto, want_tile in ((0, 128), (1, -1)):
        cache = str(tmp_path / f"tune{tile_auto}.json")
        lib = _FakeLib(_choice(tile_auto))
        idx = _FakeIndex(lib)
        first = autotune.tune(idx, None, None, None, 50_000, cache_path=cache)
        assert first["cached"] is False and lib.tuned == 1 and lib.params == []
        again = autotune.tune(idx, None, None, None, 50_000, cache_path=cache)
        assert again["cached"] is True and lib.tuned == 1
        assert lib.params == [(want_tile, 2048, 16384, 2048)] and idx.ub == 2
