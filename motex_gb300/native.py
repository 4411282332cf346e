"""ctypes binding of the C ABI in include/motex_gpu.h.

The library is loaded from ``motex_gb300/lib/libmotex_gpu.so`` (built
in-tree by ``motex_gb300.build``).  There is no fallback: if the library is
missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libmotex_gpu.so")
CLI_PATH = os.path.join(PKG, "lib", "motexGPU")

MOTEX_OK = 0
ERRORS = {-1: "EINVAL", -2: "ENOMEM", -3: "ECUDA", -4: "EUNSUPPORTED", -5: "ETIMEOUT",
          -6: "EBUSY", -7: "ENOTFOUND"}

# Every symbol the header declares (checked by the CPU tests).
EXPORTS = [
    "motex_ctx_create", "motex_ctx_destroy", "motex_gpu_run", "motex_result_free",
    "motex_gpu_load", "motex_gpu_execute", "motex_gpu_fetch", "motex_gpu_extract_pair",
    "motex_gpu_strerror", "motex_gpu_last_error", "motex_ctx_launches", "motex_probe_int_peak",
    "motex_gpu_extract_pair_static", "motex_gpu_run_batch", "motex_gpu_search",
    "motex_srv_create", "motex_srv_submit", "motex_srv_wait", "motex_srv_stats_get", "motex_srv_destroy",
    "motex_tune_lookup",
]


class MotexError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("d", C.c_uint32), ("l", C.c_uint32), ("e", C.c_uint32), ("q", C.c_uint32),
                ("Q", C.c_uint32), ("n", C.c_uint32), ("N", C.c_uint32), ("nb_gaps", C.c_uint32),
                ("gap_min", C.POINTER(C.c_uint32)), ("gap_max", C.POINTER(C.c_uint32)),
                ("blens", C.POINTER(C.c_uint32)), ("berrs", C.POINTER(C.c_uint32))]


class Job(C.Structure):
    _fields_ = [("prm", C.POINTER(Params)), ("seqs", C.POINTER(C.c_char_p)), ("lens", C.POINTER(C.c_uint32)),
                ("nseq", C.c_uint32)]


class Motif(C.Structure):
    _fields_ = [("seq", C.c_uint32), ("pos", C.c_uint32), ("strct", C.c_uint32),
                ("u", C.c_uint32), ("v", C.c_uint32)]


class Result(C.Structure):
    _fields_ = [("motifs", C.POINTER(Motif)), ("count", C.c_uint32), ("num_seqs", C.c_uint32),
                ("ref_cells", C.c_uint64), ("exec_cells", C.c_uint64), ("unique_words", C.c_uint32),
                ("launches", C.c_uint32), ("device_ms", C.c_double), ("dp_ms", C.c_double)]


class SrvTiming(C.Structure):
    _fields_ = [("queue_ms", C.c_double), ("run_ms", C.c_double), ("latency_ms", C.c_double),
                ("batch_size", C.c_uint32)]


class SrvStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("batches", C.c_uint64), ("cells", C.c_uint64), ("max_batch_seen", C.c_uint32),
                ("queued", C.c_uint32), ("in_use_bytes", C.c_uint64), ("budget_bytes", C.c_uint64)]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load (once) and declare the C ABI.  Raises if the library is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: build it with `python -m motex_gb300.build`")
    lib = C.CDLL(path)
    P = C.POINTER
    sig = {
        "motex_ctx_create": (C.c_int, [P(C.c_void_p), C.c_int]),
        "motex_ctx_destroy": (C.c_int, [C.c_void_p]),
        "motex_gpu_run": (C.c_int, [C.c_void_p, P(Params), P(C.c_char_p), P(C.c_uint32), C.c_uint32, P(Result)]),
        "motex_result_free": (None, [P(Result)]),
        "motex_gpu_load": (C.c_int, [C.c_void_p, P(Params), P(C.c_char_p), P(C.c_uint32), C.c_uint32]),
        "motex_gpu_execute": (C.c_int, [C.c_void_p]),
        "motex_gpu_fetch": (C.c_int, [C.c_void_p, P(Result)]),
        "motex_gpu_extract_pair": (C.c_int, [C.c_void_p, P(Params), C.c_char_p, C.c_uint32, C.c_char_p,
                                             C.c_uint32, P(C.c_uint32), P(C.c_uint32)]),
        "motex_gpu_search": (C.c_int, [C.c_void_p, P(Params), P(C.c_char_p), P(C.c_uint32), C.c_uint32,
                                       P(C.c_char_p), P(C.c_uint32), C.c_uint32, P(C.c_uint32), P(C.c_uint32)]),
        "motex_gpu_strerror": (C.c_char_p, [C.c_int]),
        "motex_gpu_last_error": (C.c_char_p, []),
        "motex_ctx_launches": (C.c_uint64, [C.c_void_p]),
        "motex_probe_int_peak": (C.c_int, [C.c_int, P(C.c_double), P(C.c_double), P(C.c_double)]),
        "motex_gpu_run_batch": (C.c_int, [C.c_void_p, P(Job), C.c_uint32, P(Result)]),
        "motex_srv_create": (C.c_int, [P(C.c_void_p), C.c_int, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]),
        "motex_srv_submit": (C.c_int, [C.c_void_p, P(Job), P(C.c_uint64)]),
        "motex_srv_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int, P(Result), P(SrvTiming)]),
        "motex_srv_stats_get": (C.c_int, [C.c_void_p, P(SrvStats)]),
        "motex_srv_destroy": (C.c_int, [C.c_void_p]),
        "motex_gpu_extract_pair_static": (C.c_int, [P(Params), C.c_char_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                                    C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
        "motex_tune_lookup": (C.c_int, [C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, P(C.c_int), P(C.c_int),
                                        P(C.c_int)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(rc: int):
    if rc != MOTEX_OK:
        lib = load_library()
        raise MotexError(rc, lib.motex_gpu_last_error().decode())


@dataclass
class Extraction:
    motifs: list          # (seq, pos, strct, u, v) in print order
    num_seqs: int
    ref_cells: int
    exec_cells: int
    unique_words: int
    launches: int
    device_ms: float
    dp_ms: float


def tune_lookup(B: int, l: int, e: int, d: int):
    """(W, NL, UR) the autotuner holds for the key, or None (host-only); a
    negative NL is the popc-free Hamming form with -NL guarded lanes."""
    lib = load_library()
    W, NL, UR = C.c_int(), C.c_int(), C.c_int()
    rc = lib.motex_tune_lookup(B, l, e, d, C.byref(W), C.byref(NL), C.byref(UR))
    if rc == -7:
        return None
    _check(rc)
    return W.value, NL.value, UR.value


def probe_int_peak(device: int = 0):
    """(lop3, iadd, popc) throughput in 10^12 ops/s, measured on the device."""
    lib = load_library()
    a, b, c = C.c_double(), C.c_double(), C.c_double()
    _check(lib.motex_probe_int_peak(device, C.byref(a), C.byref(b), C.byref(c)))
    return a.value, b.value, c.value


def make_params(d, l, e, q=0, Q=100, n=1, N=10000, boxes=()):
    p = Params(d, l, e, q, Q, n, N, len(boxes))
    keep = []
    if boxes:
        cols = list(zip(*boxes))
        for name, col in zip(("gap_min", "gap_max", "blens", "berrs"), cols):
            arr = (C.c_uint32 * len(col))(*col)
            keep.append(arr)
            setattr(p, name, C.cast(arr, C.POINTER(C.c_uint32)))
    p._keep = keep
    return p


class Context:
    """One CUDA device context of the engine (not thread-safe)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        self.h = C.c_void_p()
        _check(self.lib.motex_ctx_create(C.byref(self.h), device))

    def close(self):
        if self.h:
            self.lib.motex_ctx_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        return int(self.lib.motex_ctx_launches(self.h))

    @staticmethod
    def _seq_arrays(seqs):
        bs = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
        arr = (C.c_char_p * len(bs))(*bs)
        lens = (C.c_uint32 * len(bs))(*[len(b) for b in bs])
        return bs, arr, lens

    @staticmethod
    def _collect(res: Result) -> Extraction:
        motifs = [(res.motifs[i].seq, res.motifs[i].pos, res.motifs[i].strct, res.motifs[i].u, res.motifs[i].v)
                  for i in range(res.count)]
        return Extraction(motifs, res.num_seqs, res.ref_cells, res.exec_cells, res.unique_words,
                          res.launches, res.device_ms, res.dp_ms)

    def run(self, seqs, params: Params) -> Extraction:
        keep, arr, lens = self._seq_arrays(seqs)
        res = Result()
        _check(self.lib.motex_gpu_run(self.h, C.byref(params), arr, lens, len(keep), C.byref(res)))
        try:
            return self._collect(res)
        finally:
            self.lib.motex_result_free(C.byref(res))

    def run_batch(self, jobs):
        """jobs: list of (seqs, Params); returns one Extraction per job."""
        keep = []
        arr = (Job * len(jobs))()
        for i, (seqs, prm) in enumerate(jobs):
            bs, a, lens = self._seq_arrays(seqs)
            keep.append((bs, a, lens, prm))
            arr[i] = Job(C.pointer(prm), a, lens, len(bs))
        res = (Result * len(jobs))()
        _check(self.lib.motex_gpu_run_batch(self.h, arr, len(jobs), res))
        out = []
        for i in range(len(jobs)):
            out.append(self._collect(res[i]))
            self.lib.motex_result_free(C.byref(res[i]))
        return out

    def load(self, seqs, params: Params):
        keep, arr, lens = self._seq_arrays(seqs)
        _check(self.lib.motex_gpu_load(self.h, C.byref(params), arr, lens, len(keep)))

    def execute(self):
        _check(self.lib.motex_gpu_execute(self.h))

    def fetch(self) -> Extraction:
        res = Result()
        _check(self.lib.motex_gpu_fetch(self.h, C.byref(res)))
        try:
            return self._collect(res)
        finally:
            self.lib.motex_result_free(C.byref(res))

    def extract_pair(self, p: str, t: str, params: Params, u=None, v=None, nb_structs: int = 1):
        m = len(p)
        U = (C.c_uint32 * (m * nb_structs))(*(u or [0] * (m * nb_structs)))
        V = (C.c_uint32 * (m * nb_structs))(*(v or [0] * (m * nb_structs)))
        _check(self.lib.motex_gpu_extract_pair(self.h, C.byref(params), p.encode(), m, t.encode(), len(t), U, V))
        return list(U), list(V)

    def search(self, words, seqs, params: Params):
        """u, v of each word's last l symbols over the sequences (motex_gpu_search)."""
        wb, warr, wlens = self._seq_arrays(words)
        sb, sarr, slens = self._seq_arrays(seqs)
        U = (C.c_uint32 * max(1, len(wb)))()
        V = (C.c_uint32 * max(1, len(wb)))()
        _check(self.lib.motex_gpu_search(self.h, C.byref(params), warr, wlens, len(wb), sarr, slens, len(sb), U, V))
        return list(U)[:len(wb)], list(V)[:len(wb)]


class Server:
    """Continuous-batching extraction server (motex_srv_*)."""

    def __init__(self, device=0, hbm_budget=0, max_batch=32, workers=2, max_queue=0):
        self.lib = load_library()
        self.h = C.c_void_p()
        _check(self.lib.motex_srv_create(C.byref(self.h), device, hbm_budget, max_batch, workers, max_queue))

    def submit(self, seqs, params: Params) -> int:
        bs, arr, lens = Context._seq_arrays(seqs)
        job = Job(C.pointer(params), arr, lens, len(bs))
        rid = C.c_uint64()
        _check(self.lib.motex_srv_submit(self.h, C.byref(job), C.byref(rid)))
        return rid.value

    def wait(self, rid: int, timeout_ms: int = -1):
        """(Extraction, timing dict); raises MotexError (ETIMEOUT if still pending)."""
        res, tm = Result(), SrvTiming()
        rc = self.lib.motex_srv_wait(self.h, rid, timeout_ms, C.byref(res), C.byref(tm))
        try:
            _check(rc)
            return Context._collect(res), {"queue_ms": tm.queue_ms, "run_ms": tm.run_ms,
                                           "latency_ms": tm.latency_ms, "batch_size": tm.batch_size}
        finally:
            self.lib.motex_result_free(C.byref(res))

    def stats(self) -> dict:
        st = SrvStats()
        _check(self.lib.motex_srv_stats_get(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in SrvStats._fields_}

    def close(self):
        if self.h:
            self.lib.motex_srv_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
