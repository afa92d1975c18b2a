"""Cached autotuning of the batched path.

`tune()` runs the library's autotuner (`autotuneBatchedGpu`: coordinate descent over the
upper-bound provider, tile size, candidate capacity, length split, the emit's copy mode and the
Eytzinger tree's depth, timed on a sample of
the caller's own device-resident queries) once per (GPU model, index size, batch size,
coordinate width, contig count) and stores the choice in a JSON file; later calls with the
same key apply the stored choice without timing anything.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import subprocess

from . import _capi

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "superintervals_gb300", "autotune.json")


def gpu_name(device: int = 0) -> str:
    try:
        out = subprocess.run(["nvidia-smi", f"--id={device}", "--query-gpu=name", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=30)
        return out.stdout.strip() or "unknown"
    except Exception:
        return "unknown"


def _bucket(x: int) -> int:
    return int(2 ** round(math.log2(max(1, x))))


def cache_key(index, nq: int) -> str:
    return (f"{gpu_name()}|n~{_bucket(index.size())}|nq~{_bucket(nq)}|bits={index.bits}"
            f"|contigs={index.n_contigs()}")


def apply(index, choice: dict):
    lib = index.lib
    # a choice that kept the automatic tile size (per batch) restores it (-1)
    tile = -1 if int(choice.get("tile_auto", 0)) else int(choice["tile_queries"])
    _capi.check(lib.setBatchedParamsGpu(index.h, tile, int(choice["tile_candidates"]),
                                        int(choice["long_query_len"]), int(choice["split_len"])))
    if "emit_copy" in choice:
        _capi.check(lib.setBatchedOptionGpu(index.h, _capi.OPT_EMIT_COPY, int(choice["emit_copy"])))
    if "eytz_depth" in choice:
        _capi.check(lib.setBatchedOptionGpu(index.h, _capi.OPT_EYTZ_DEPTH, int(choice["eytz_depth"])))
    index.set_upper_bound(int(choice["upper_bound"]))


def tune(index, d_qs, d_qe, d_qc, nq: int, sample: int = 0, cache_path: str = DEFAULT_CACHE,
         use_cache: bool = True, keep_upper_bound: bool = False) -> dict:
    """Tune `index` (a GpuIndex) for a device-resident batch; returns the choice
    (plus "cached": True/False).  sample = 0 times the whole batch; keep_upper_bound fixes
    the current provider."""
    key = cache_key(index, nq) + ("|ub-fixed" if keep_upper_bound else "")
    cache = {}
    if use_cache and os.path.isfile(cache_path):
        try:
            with open(cache_path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        apply(index, cache[key])
        return dict(cache[key], cached=True)
    buf = C.create_string_buffer(1024)
    flags = _capi.TUNE_KEEP_UPPER_BOUND if keep_upper_bound else 0
    _capi.check(index.lib.autotuneBatchedGpu(index.h, d_qs, d_qe, d_qc, nq, sample, flags, buf, len(buf)))
    choice = json.loads(buf.value.decode())
    if use_cache:
        cache[key] = choice
        try:
            os.makedirs(os.path.dirname(cache_path), exist_ok=True)
            with open(cache_path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return dict(choice, cached=False)
