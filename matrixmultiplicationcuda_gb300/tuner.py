"""Autotuner: the configuration table, the exhaustive sweep, the structure
features, and a persistent database of sweep results.

The sweep and the features run in the library (spmm_tune_sweep,
spmm_structure_features); this module keeps the results. The database is a
JSON file mapping a product's signature (shape, block shape, type, stored
blocks and a CRC of its index arrays) to the measured time of every
configuration on the named device, so a product is swept once per device.
"""
import ctypes
import json
import os
import zlib

import numpy as np

from ._lib import Config, check, lib, stream_handle

N_FEATURES = 18


def n_configs():
    return int(lib().spmm_tune_config_count())


def configs():
    """The table entries, in order (list of Config)."""
    out = []
    for i in range(n_configs()):
        c = Config()
        check(lib().spmm_tune_config(i, ctypes.byref(c)))
        out.append(c)
    return out


def config_key(c):
    return (c.kernel, c.n_tile, c.stages, c.ctas_per_sm, c.acc_buffers, c.schedule, max(c.split_k, 1))


def config_name(c):
    if c.kernel == 1:
        return "mma nt%d st%d" % (c.n_tile, c.stages)
    if c.kernel == 3:
        return "tc64 nt%d %s" % (c.n_tile, "queue" if c.schedule else "static")
    if c.schedule == 2:
        return "plan tc nt%d st%s acc%d" % (c.n_tile, c.stages or "d", c.acc_buffers)
    return "tc nt%d st%s acc%d %s split%d" % (c.n_tile, c.stages or "d", c.acc_buffers,
                                             "queue" if c.schedule else "static", max(c.split_k, 1))


def is_plan(c):
    """A table entry that runs as a per-matrix plan (schedule 2)."""
    return c.kernel == 2 and c.schedule == 2


def supported_mask(bR, dtype, N):
    """Boolean array over the table: which entries have a kernel."""
    cs = configs()
    return np.array([lib().spmm_config_supported(bR, int(dtype), N, ctypes.byref(c)) == 0 for c in cs])


def default_index(bR, dtype, N):
    """Table index of the configuration spmm_bcsr_mm runs when given none."""
    d = Config()
    check(lib().spmm_default_config(bR, int(dtype), N, ctypes.byref(d)))
    k = config_key(d)
    for i, c in enumerate(configs()):
        if config_key(c) == k:
            return i
    raise LookupError("default configuration is not a table entry")


def features_host(row_ptr, col_idx, M, K, bR, N, dtype=0):
    rp = np.ascontiguousarray(row_ptr, np.int32)
    ci = np.ascontiguousarray(col_idx, np.int32)
    if ci.size == 0:
        ci = np.zeros(1, np.int32)
    out = np.zeros(N_FEATURES, np.float32)
    if lib().spmm_structure_features_host(ctypes.c_void_p(rp.ctypes.data), ctypes.c_void_p(ci.ctypes.data),
                                          M, K, bR, N, int(dtype), ctypes.c_void_p(out.ctypes.data)) != 0:
        raise ValueError("bad BCSR structure")
    return out


def features(A, N, stream=None):
    """Features of a device BCSR (copies its index arrays to the host)."""
    out = np.zeros(N_FEATURES, np.float32)
    d = A.desc()
    check(lib().spmm_structure_features(ctypes.byref(d), int(N), ctypes.c_void_p(out.ctypes.data),
                                        stream_handle(stream)))
    return out


def sweep(A, B, N=None, C=None, warmup=2, reps=5, flush=None, stream=None, B_lo=None):
    """Mean time (ms) of every table entry on C = A @ B; +inf where unsupported."""
    import torch
    from .bcsr import _dense_desc
    N = int(B.shape[1]) if N is None else int(N)
    if C is None:
        C = torch.empty((A.M, N), dtype=torch.float32, device=B.device)
    ms = np.zeros(n_configs(), np.float32)
    a = A.desc()
    b = _dense_desc(B, B_lo, ldb=B.stride(0))
    fptr = ctypes.c_void_p(flush.data_ptr()) if flush is not None else None
    fbytes = flush.numel() * flush.element_size() if flush is not None else 0
    check(lib().spmm_tune_sweep(ctypes.byref(a), ctypes.byref(b), N, ctypes.c_void_p(C.data_ptr()),
                                int(C.stride(0)), warmup, reps, fptr, fbytes,
                                ctypes.c_void_p(ms.ctypes.data), stream_handle(stream)))
    return ms


def sweep_b2b(copies, launches=20, warmup=2, stream=None):
    """Mean time per launch (ms) of every table entry run back to back over
    `copies` -- a list of (A, B, C) or (A, B, C, B_lo, b_scale) of one problem
    -- replayed from a CUDA graph (spmm_tune_sweep_b2b); +inf where
    unsupported. Plan entries (schedule 2) chain their runs with the
    inputs-ready flag."""
    from ._lib import Problem
    from .bcsr import _dense_desc
    arr = (Problem * len(copies))()
    for i, cp in enumerate(copies):
        A, B, C = cp[:3]
        B_lo = cp[3] if len(cp) > 3 else None
        bs = cp[4] if len(cp) > 4 else 1.0
        arr[i].A = A.desc()
        arr[i].B = _dense_desc(B, B_lo, bs, ldb=B.stride(0))
        arr[i].N = int(B.shape[1])
        arr[i].C = C.data_ptr()
        arr[i].ldc = int(C.stride(0))
    ms = np.zeros(n_configs(), np.float32)
    check(lib().spmm_tune_sweep_b2b(arr, len(copies), int(launches), int(warmup), ctypes.c_void_p(ms.ctypes.data),
                                    stream_handle(stream)))
    return ms


def signature(A, N):
    """Key of a product in the database: shape, block shape, type, nnzb and a
    CRC-32 of row_ptr and col_idx."""
    rp = A.row_ptr.cpu().numpy().astype(np.int32)
    ci = A.col_idx.cpu().numpy().astype(np.int32)
    crc = zlib.crc32(ci.tobytes(), zlib.crc32(rp.tobytes()))
    return "%dx%dx%d/b%dx%d/t%d/nnzb%d/crc%08x" % (A.M, A.K, N, A.bR, A.bC, int(A.dtype), ci.size, crc)


class TuneDB:
    """Persistent sweep results: {device name: {signature: [ms per config]}}."""

    def __init__(self, path):
        self.path = path
        self.data = {}
        if path and os.path.exists(path):
            with open(path) as f:
                self.data = json.load(f)

    @staticmethod
    def device_name():
        import torch
        return torch.cuda.get_device_name() if torch.cuda.is_available() else "none"

    def get(self, sig, device=None):
        ms = self.data.get(device or self.device_name(), {}).get(sig)
        return None if ms is None else np.array([np.inf if v is None else v for v in ms], np.float32)

    def put(self, sig, ms, device=None):
        self.data.setdefault(device or self.device_name(), {})[sig] = [
            None if not np.isfinite(v) else float(v) for v in ms]

    def save(self):
        tmp = self.path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.data, f, indent=0, sort_keys=True)
        os.replace(tmp, self.path)


class Autotuner:
    """Picks a configuration per product: the database if the product was
    swept on this device, else the cost model if one is given, else a sweep
    (stored in the database)."""

    def __init__(self, db_path=None, model=None, warmup=2, reps=5):
        self.db = TuneDB(db_path) if db_path else None
        self.model = model
        self.warmup, self.reps = warmup, reps
        self._table = configs()

    def best(self, A, B, N=None, C=None, allow_sweep=True):
        N = int(B.shape[1]) if N is None else int(N)
        sig = signature(A, N)
        if self.db is not None:
            ms = self.db.get(sig)
            if ms is not None:
                return self._table[int(np.argmin(ms))]
        if self.model is not None:
            return self.model.select(A, N)
        if not allow_sweep:
            return None
        ms = sweep(A, B, N, C, self.warmup, self.reps)
        if self.db is not None:
            self.db.put(sig, ms)
            self.db.save()
        return self._table[int(np.argmin(ms))]
