"""ctypes binding of libsi_gpu.so (the C-ABI declared in include/si_gpu/c_api.h).

This is the binding a Python host of the reference would add in place of the
Cython extension (src/superintervals/intervalmap.pyx).  The library is loaded
from the in-tree build directory; there is no fallback: if the CUDA library is
missing, importing the query API raises.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libsi_gpu.so")

SI_OK = 0
SI_ERR_INVALID = 1
SI_ERR_OOM = 2
SI_ERR_NOT_BUILT = 3
SI_ERR_CUDA = 4
SI_ERR_CAPACITY = 5
SI_ERR_UNSUPPORTED = 6
SI_ERR_TOO_LARGE = 7

ORDER_IDXS_CPP = 0
ORDER_DESC = 1

TUNE_KEEP_UPPER_BOUND = 1

OPT_EMIT_COPY = 1
OPT_EYTZ_DEPTH = 2

PATH_AUTO = 0
PATH_PLAIN = 1
PATH_BATCHED = 2

UB_BINARY = 0
UB_EYTZINGER = 1
UB_LEARNED = 2

_ERR_NAMES = {1: "INVALID", 2: "OOM", 3: "NOT_BUILT", 4: "CUDA", 5: "CAPACITY", 6: "UNSUPPORTED",
              7: "TOO_LARGE"}


class SIError(RuntimeError):
    """A non-zero status from the C-ABI, with the library's message."""

    def __init__(self, status, msg):
        super().__init__(f"SI_ERR_{_ERR_NAMES.get(status, status)}: {msg}")
        self.status = status


class cCsrResult(C.Structure):
    _fields_ = [("offsets", C.POINTER(C.c_int64)), ("values", C.POINTER(C.c_int32)),
                ("n_queries", C.c_size_t), ("size", C.c_size_t), ("capacity", C.c_size_t),
                ("offsets_capacity", C.c_size_t)]


class cBedStats(C.Structure):
    _fields_ = [(k, C.c_size_t) for k in ("lines", "intervals", "skipped_headers", "malformed", "filtered",
                                         "out_of_range", "unknown_contig")]


BED_HALF_OPEN = 1

_P = C.c_void_p
_H = C.c_void_p
_SZ = C.c_size_t
_I = C.c_int

# name -> (restype, argtypes); every function declared in include/si_gpu/c_api.h
SIGNATURES = {
    "createSuperIntervalsGpu": (_I, [C.POINTER(_H), _I, _I]),
    "destroySuperIntervalsGpu": (None, [_H]),
    "clearSuperIntervalsGpu": (_I, [_H]),
    "reserveSuperIntervalsGpu": (_I, [_H, _SZ]),
    "addIntervalGpu": (_I, [_H, C.c_int32, C.c_int32, C.c_int32]),
    "addIntervalGpu_i64": (_I, [_H, C.c_int64, C.c_int64, C.c_int32]),
    "addIntervalsGpu": (_I, [_H, _P, _P, _P, _SZ]),
    "addIntervalsGpu_i64": (_I, [_H, _P, _P, _P, _SZ]),
    "setContigsGpu": (_I, [_H, _SZ, _P]),
    "sizeSuperIntervalsGpu": (_SZ, [_H]),
    "numContigsGpu": (_SZ, [_H]),
    "indexSuperIntervalsGpu": (_I, [_H]),
    "getIndexArraysGpu": (_I, [_H, _P, _P, _P, _P]),
    "serializeIndexGpu": (_I, [_H, _P, _SZ, C.POINTER(_SZ)]),
    "ingestBedGpu": (_I, [_H, C.c_char_p, _SZ, _I, C.POINTER(cBedStats)]),
    "bedQueriesGpu": (_I, [_H, C.c_char_p, _SZ, _I, _P, _P, _P, _P, _SZ, C.POINTER(_SZ), C.POINTER(cBedStats)]),
    "contigNameGpu": (_I, [_H, _SZ, C.c_char_p, _SZ, C.POINTER(_SZ)]),
    "deserializeIndexGpu": (_I, [_H, _P, _SZ]),
    "saveIndexGpu": (_I, [_H, C.c_char_p]),
    "loadIndexGpu": (_I, [_H, C.c_char_p]),
    "setQueryPathGpu": (_I, [_H, _I]),
    "setUpperBoundModeGpu": (_I, [_H, _I]),
    "setOutputBudgetGpu": (_I, [_H, _SZ]),
    "setBatchedParamsGpu": (_I, [_H, _I, _I, C.c_int64, C.c_int64]),
    "getBatchedParamsGpu": (_I, [_H, _P, _P, _P, _P]),
    "setBatchedOptionGpu": (_I, [_H, _I, C.c_int64]),
    "getBatchedOptionGpu": (_I, [_H, _I, _P]),
    "autotuneBatchedGpu": (_I, [_H, _P, _P, _P, _SZ, _SZ, _I, C.c_char_p, _SZ]),
    "setProfilingGpu": (_I, [_H, _I]),
    "getPhaseTimesGpu": (_I, [_H, _P, _P]),
    "setDeviceBudgetGpu": (_I, [_SZ]),
    "deviceBytesInUseGpu": (_SZ, []),
    "deviceMemInfoGpu": (_I, [_I, C.POINTER(_SZ), C.POINTER(_SZ)]),
    "countOverlapsBatchGpu": (_I, [_H, _P, _P, _P, _SZ, _P]),
    "countOverlapsBatchGpu_i64": (_I, [_H, _P, _P, _P, _SZ, _P]),
    "anyOverlapsBatchGpu": (_I, [_H, _P, _P, _P, _SZ, _P]),
    "anyOverlapsBatchGpu_i64": (_I, [_H, _P, _P, _P, _SZ, _P]),
    "searchIdxsBatchGpu": (_I, [_H, _P, _P, _P, _SZ, _I, C.POINTER(cCsrResult)]),
    "searchIdxsBatchGpu_i64": (_I, [_H, _P, _P, _P, _SZ, _I, C.POINTER(cCsrResult)]),
    "searchValuesBatchGpu": (_I, [_H, _P, _P, _P, _SZ, C.POINTER(cCsrResult)]),
    "searchValuesBatchGpu_i64": (_I, [_H, _P, _P, _P, _SZ, C.POINTER(cCsrResult)]),
    "searchBatchIntoGpu": (_I, [_H, _P, _P, _P, _SZ, _I, _I, _P, _P, _SZ, C.POINTER(_SZ)]),
    "countOverlapsDeviceGpu": (_I, [_H, _P, _P, _P, _SZ, _P, _P]),
    "searchDeviceGpu": (_I, [_H, _P, _P, _P, _SZ, _I, _I, _P, _P, _SZ, C.POINTER(_SZ), _P]),
    "upperBoundDeviceGpu": (_I, [_H, _P, _P, _SZ, _I, _P, _P]),
    "searchDeviceGraphGpu": (_I, [_H, _P, _P, _P, _SZ, _I, _P, _P, _SZ, C.POINTER(_SZ), _P]),
    "searchIdxsNoAllocGpu": (_I, [_H, _P, _P, _P, _SZ, _I, _P, _P, _SZ, C.POINTER(_SZ), _P]),
    "intersectBatchGpu": (_I, [_H, _P, _P, _P, _SZ, _I, _P, _P, _P, _P, _SZ, C.POINTER(_SZ)]),
    "intersectDeviceGpu": (_I, [_H, _P, _P, _P, _SZ, _I, _P, _P, _P, _P, _SZ, C.POINTER(_SZ), _P]),
    "differenceBatchGpu": (_I, [_H, _P, _P, _P, _SZ, _P, _P, _P, _SZ, C.POINTER(_SZ)]),
    "differenceDeviceGpu": (_I, [_H, _P, _P, _P, _SZ, _P, _P, _P, _SZ, C.POINTER(_SZ), _P]),
    "searchKeysBatchGpu": (_I, [_H, _P, _P, _P, _SZ, _I, _P, _P, _P, _P, _SZ, C.POINTER(_SZ)]),
    "searchKeysDeviceGpu": (_I, [_H, _P, _P, _P, _SZ, _I, _P, _P, _P, _P, _SZ, C.POINTER(_SZ), _P]),
    "coverageBatchGpu": (_I, [_H, _P, _P, _P, _SZ, _P, _P]),
    "coverageDeviceGpu": (_I, [_H, _P, _P, _P, _SZ, _P, _P, _P]),
    "createCsrResult": (cCsrResult, []),
    "clearCsrResult": (None, [C.POINTER(cCsrResult)]),
    "destroyCsrResult": (None, [C.POINTER(cCsrResult)]),
    "lastErrorGpu": (C.c_char_p, []),
    "getStreamGpu": (_P, [_H]),
    "deviceCountGpu": (_I, [C.POINTER(_I)]),
    "deviceMallocGpu": (_I, [C.POINTER(_P), _SZ]),
    "deviceFreeGpu": (_I, [_P]),
    "hostMallocPinnedGpu": (_I, [C.POINTER(_P), _SZ]),
    "hostFreePinnedGpu": (_I, [_P]),
    "memcpyGpu": (_I, [_P, _P, _SZ, _P]),
    "streamSynchronizeGpu": (_I, [_P]),
    "eventCreateGpu": (_I, [C.POINTER(_P)]),
    "eventDestroyGpu": (_I, [_P]),
    "eventRecordGpu": (_I, [_P, _P]),
    "eventElapsedMsGpu": (_I, [_P, _P, C.POINTER(C.c_float)]),
    "flushL2Gpu": (_I, [_P]),
    "getLaunchCountGpu": (C.c_longlong, []),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libsi_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.isfile(path):
        raise ImportError(f"CUDA library {path} is missing: run "
                          "`python -c 'import __graft_entry__ as g; g.build()'` first")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status: int):
    if status != SI_OK:
        msg = _lib.lastErrorGpu() if _lib is not None else b""
        raise SIError(status, (msg or b"").decode(errors="replace"))
