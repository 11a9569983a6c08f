"""Python access to the CPU checkers -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this package, always as the checker and never as the thing
measured or shipped.

* :class:`Oracle` wraps ``liboracle.so`` (the C++ restatement in
  ``sdl_oracle.cc``; built by ``make -C oracle oracle``).
* :func:`run_reference` runs ``_ref/ref_driver`` (the unmodified reference,
  built by ``make -C oracle ref`` only where the reference sources exist).
* :func:`canon` / :func:`digest` put stage outputs (hit-index tuples) in a
  canonical multiset order so two implementations can be compared.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
STAGES = ("MD", "SG", "TL", "TP", "TC")
WIDTH = (2, 4, 8, 8, 16)

_i64, _i32, _u32, _f32 = ctypes.c_int64, ctypes.c_int32, ctypes.c_uint32, ctypes.c_float
_vp = ctypes.c_void_p


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def build(ref_dir: str | None = None) -> None:
    """Build liboracle.so; with ref_dir (the reference's source directory),
    also the unmodified reference and its driver (oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if ref_dir and os.path.isdir(ref_dir):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "-j8", "REFDIR=" + ref_dir], check=True)


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.sdlo_geometry_create.restype = _vp
        L.sdlo_geometry_create.argtypes = [_i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _vp]
        L.sdlo_geometry_free.argtypes = [_vp]
        L.sdlo_run.restype = _vp
        L.sdlo_run.argtypes = [_vp, _i64, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int]
        L.sdlo_count.restype = _i64
        L.sdlo_count.argtypes = [_vp, ctypes.c_int]
        L.sdlo_copy.argtypes = [_vp, ctypes.c_int, _vp]
        L.sdlo_counters.argtypes = [_vp, _vp]
        L.sdlo_vals.argtypes = [_vp, ctypes.c_int, _vp]
        L.sdlo_times.argtypes = [_vp, _vp]
        L.sdlo_free.argtypes = [_vp]
        L.sdlo_run_many.restype = _i64
        L.sdlo_run_many.argtypes = [_vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int]
        L.sdlo_run_many_digest.restype = _i64
        L.sdlo_run_many_digest.argtypes = [_vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                           _vp, _vp, _vp]
        L.sdlo_audit.restype = _i64
        L.sdlo_audit.argtypes = [_vp, _i64, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp, _i64, _vp]
        L.sdlo_audit_record_size.restype = ctypes.c_int
        L.sdlo_set_libm.argtypes = [ctypes.c_int]
        L.sdlo_libm_values.argtypes = [ctypes.c_int, ctypes.c_uint32, _i64, _vp, ctypes.c_int]
        L.sdlo_libm_counts.argtypes = [_vp, ctypes.c_int]
        _LIB = L
    return _LIB


LIBM_GLIBC, LIBM_ROUNDED, LIBM_COUNT = 0, 1, 2

# one near-cut audit record (sdlo_audit)
AUDIT_DTYPE = np.dtype([("stage", "<i4"), ("accept_glibc", "<i4"), ("primary", "<i4"), ("pad", "<i4"),
                        ("tuple", "<i4", (8,)), ("g_value", "<f4"), ("g_lo", "<f4"), ("g_hi", "<f4"),
                        ("r_value", "<f4"), ("r_lo", "<f4"), ("r_hi", "<f4"), ("where", "S24"), ("cut", "S88")])


def set_libm(mode: int) -> None:
    """Float libm of the restatement: LIBM_GLIBC (the reference's glibc float
    functions, default), LIBM_ROUNDED (correctly rounded floats, the GPU
    chain's arithmetic), LIBM_COUNT (glibc values, counting the calls whose
    correctly rounded value differs)."""
    lib().sdlo_set_libm(int(mode))


def libm_values(fn: int, start_bits: int, n: int, threads: int = 0) -> np.ndarray:
    """The host libm's float function fn (0 asin, 1 atan, 2 sin, 3 cos, 4 tan)
    on n consecutive float bit patterns."""
    out = np.empty(n, dtype=np.float32)
    lib().sdlo_libm_values(int(fn), int(start_bits), int(n), out.ctypes.data, int(threads or os.cpu_count() or 1))
    return out


def libm_counts(reset: bool = False):
    """(calls counted, calls whose glibc and correctly rounded values differ)"""
    out = np.zeros(2, dtype=np.uint64)
    lib().sdlo_libm_counts(out.ctypes.data, 1 if reset else 0)
    return int(out[0]), int(out[1])


class Oracle:
    """The restated chain bound to one detector geometry."""

    def __init__(self, det):
        L = lib()
        t_id, t_val, e_id, e_val, keys, off, dst = det.tables()
        self._keep = [np.ascontiguousarray(a) for a in (t_id, t_val, e_id, e_val, keys, off, dst)]
        t_id, t_val, e_id, e_val, keys, off, dst = self._keep
        self.h = L.sdlo_geometry_create(len(t_id), t_id.ctypes.data, t_val.ctypes.data, len(e_id),
                                        e_id.ctypes.data, e_val.ctypes.data, len(keys), keys.ctypes.data,
                                        off.ctypes.data, dst.ctypes.data)

    def __del__(self):
        if getattr(self, "h", None):
            lib().sdlo_geometry_free(self.h)
            self.h = None

    def run(self, ev, mode: int = 0, stop_after: int = 4, vals: bool = False):
        """Returns (tuples per stage, counters[110], seconds[5]); with vals,
        also the per-object floats of the mini-doublets (n x 4: dz,
        shiftedDz, dphi, dphichange) and segments (n x 6: dphi, dphimin,
        dphimax, dphichange, dphiminchange, dphimaxchange) in tuple order."""
        L = lib()
        arrs = [np.ascontiguousarray(a) for a in (ev.x, ev.y, ev.z, ev.idx, ev.detid)]
        r = L.sdlo_run(self.h, len(arrs[0]), *[a.ctypes.data for a in arrs], mode, stop_after)
        try:
            out = []
            for s in range(5):
                n = L.sdlo_count(r, s)
                a = np.empty((n, WIDTH[s]), dtype=np.int32)
                if n:
                    L.sdlo_copy(r, s, a.ctypes.data)
                out.append(a)
            cnt = np.empty(110, dtype=np.uint32)
            L.sdlo_counters(r, cnt.ctypes.data)
            sec = np.empty(5, dtype=np.float64)
            L.sdlo_times(r, sec.ctypes.data)
            vv = []
            for s, w in ((0, 4), (1, 6)):
                a = np.zeros((len(out[s]), w), dtype=np.float32)
                if len(a):
                    L.sdlo_vals(r, s, a.ctypes.data)
                vv.append(a)
        finally:
            L.sdlo_free(r)
        return (out, cnt, sec, vv) if vals else (out, cnt, sec)

    def audit(self, ev, mode: int = 0, cap: int = 4096):
        """Near-cut audit of one event: the chain with the reference's float
        libm and with correctly rounded floats.  Returns (records of the
        objects only one of them makes, AUDIT_DTYPE; summary 5 x 4 per stage:
        objects with glibc, with rounded floats, primary flips, secondary
        flips)."""
        L = lib()
        assert L.sdlo_audit_record_size() == AUDIT_DTYPE.itemsize
        arrs = [np.ascontiguousarray(a) for a in (ev.x, ev.y, ev.z, ev.idx, ev.detid)]
        out = np.zeros(cap, dtype=AUDIT_DTYPE)
        summ = np.zeros((5, 4), dtype=np.int64)
        n = L.sdlo_audit(self.h, len(arrs[0]), *[a.ctypes.data for a in arrs], mode, out.ctypes.data, cap,
                         summ.ctypes.data)
        return out[:min(n, cap)], summ

    def run_many(self, events, n_threads: int, mode: int = 0) -> int:
        """Runs whole chains on independent events in parallel threads;
        returns the total track-candidate count."""
        off = np.zeros(len(events) + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(e) for e in events])
        cat = [np.ascontiguousarray(np.concatenate([getattr(e, k) for e in events]))
               for k in ("x", "y", "z", "idx", "detid")]
        return int(lib().sdlo_run_many(self.h, len(events), off.ctypes.data, *[a.ctypes.data for a in cat],
                                       mode, n_threads))

    def run_many_digest(self, events, n_threads: int, mode: int = 0):
        """Whole chains on independent events in parallel threads; returns per
        event the object counts (n, 5), the order-independent digests of the
        object multisets (n, 5; sdl_gb300.tuples.multiset_digest) and the
        per-layer counters (n, 110)."""
        n = len(events)
        off = np.zeros(n + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(e) for e in events])
        cat = [np.ascontiguousarray(np.concatenate([getattr(e, k) for e in events]))
               for k in ("x", "y", "z", "idx", "detid")]
        counts = np.zeros((n, 5), dtype=np.int64)
        digests = np.zeros((n, 5), dtype=np.uint64)
        counters = np.zeros((n, 110), dtype=np.uint32)
        lib().sdlo_run_many_digest(self.h, n, off.ctypes.data, *[a.ctypes.data for a in cat], mode, n_threads,
                                   counts.ctypes.data, digests.ctypes.data, counters.ctypes.data)
        return counts, digests, counters


def read_dump(path):
    """Reads a dump written by ref_driver (same layout as Oracle.run)."""
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    out = []
    for s in range(5):
        n, w = np.frombuffer(data, dtype=np.int64, count=2, offset=pos)
        pos += 16
        a = np.frombuffer(data, dtype=np.int32, count=int(n * w), offset=pos).reshape(int(n), int(w))
        pos += int(n * w) * 4
        out.append(a.copy())
    cnt = np.frombuffer(data, dtype=np.uint32, count=110, offset=pos).copy()
    pos += 440
    sec = np.frombuffer(data, dtype=np.float64, count=5, offset=pos).copy()
    return out, cnt, sec


def run_reference(det, ev, mode: str = "map", workdir: str | None = None, tl_vars: bool = False):
    """Runs the compiled reference (oracle/_ref/ref_driver) on one event;
    with tl_vars, also returns the tracklets' final recovars (n_tl x 15, rows
    as the tracklet tuples)."""
    exe = os.path.join(HERE, "_ref", "ref_driver")
    if not os.path.exists(exe):
        raise FileNotFoundError("reference driver not built (make -C oracle ref)")
    with tempfile.TemporaryDirectory(dir=workdir) as d:
        paths = det.write_files(d)
        hb = os.path.join(d, "hits.bin")
        ob = os.path.join(d, "out.bin")
        vb = os.path.join(d, "vars.bin")
        ev.write_bin(hb)
        subprocess.run([exe, *paths, hb, ob, mode] + ([vb] if tl_vars else []), check=True, capture_output=True)
        res = read_dump(ob)
        if not tl_vars:
            return res
        v = np.fromfile(vb, dtype=np.float32).reshape(-1, 15)
        assert v.shape[0] == res[0][2].shape[0]
        return res + (v,)


def canon(t: np.ndarray) -> np.ndarray:
    """Rows sorted lexicographically: the canonical form of a tuple multiset."""
    t = np.ascontiguousarray(t, dtype=np.int32)
    if t.shape[0] == 0:
        return t
    order = np.lexsort(t.T[::-1])
    return t[order]


def canon_order(t: np.ndarray) -> np.ndarray:
    """The row order canon() applies (to carry per-row data along)."""
    t = np.ascontiguousarray(t, dtype=np.int32)
    return np.lexsort(t.T[::-1]) if t.shape[0] else np.zeros(0, dtype=np.int64)


def digest(t: np.ndarray) -> str:
    return hashlib.sha256(canon(t).tobytes()).hexdigest()[:24]


def multiset_diff(a: np.ndarray, b: np.ndarray):
    """(rows in a not in b, rows in b not in a), multiplicity-aware."""
    from collections import Counter
    ca = Counter(map(tuple, np.asarray(a).tolist()))
    cb = Counter(map(tuple, np.asarray(b).tolist()))
    return list((ca - cb).elements()), list((cb - ca).elements())
