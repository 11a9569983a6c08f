"""GB300 segment-linking chain: Python binding of libsdlgpu.so (C ABI in
include/sdl_gpu.h).

The classes mirror the reference's user-facing calls:

* :class:`Geometry`-loading methods replace ``SDL::tiltedGeometry.load``,
  ``SDL::endcapGeometry.load`` and ``SDL::moduleConnectionMap.load``;
* :meth:`Chain.set_events` replaces ``SDL::Event::addHitToModule`` for every
  hit of a batch of events;
* :meth:`Chain.run` replaces ``createMiniDoublets ->
  createSegmentsWithModuleMap -> createTrackletsWithModuleMap ->
  createTriplets -> createTrackCandidates``;
* :meth:`Chain.objects` / :meth:`Chain.counts` / :meth:`Chain.counters`
  replace the object lists and ``getNumberOf*`` counters.

There is no CPU fallback: a missing library or CUDA device raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsdlgpu.so")

STAGES = ("MD", "SG", "TL", "TP", "TC")
WIDTH = (2, 4, 8, 8, 16)
FLAG_SG_LAYERS = 1   # Event::createSegments (layer pairs) instead of createSegmentsWithModuleMap
FLAG_TL_LAYERS = 2   # Event::createTracklets (layer pairs) instead of createTrackletsWithModuleMap
FLAG_TL_NM1 = 4
FLAG_NO_GRAPH = 8
FLAG_MLP = 16        # learned pre-filter ahead of the tracklet cuts
FLAG_TL_NAV = 32     # Event::createTrackletsViaNavigation instead of createTrackletsWithModuleMap
FLAG_TC_FROM_TL = 64   # Event::createTrackCandidatesFromTracklets instead of createTrackCandidates
FLAG_TC_FROM_TP = 128  # Event::createTrackCandidatesFromTriplets instead of createTrackCandidates
FLAG_NO_B2_FILTER = 256  # without the single-precision phase-B2 filter (same tracklets)
FLAG_TEST_MLP_GIVE_UP = 4096  # self-test: the pre-filter's first tensor-core wait gives up at once
# the columns of Chain.tracklet_vars (the reference's Tracklet recovars keys)
TL_VAR_NAMES = ("betaIn", "betaInRHmin", "betaInRHmax", "betaOut", "betaOutRHmin", "betaOutRHmax", "betaAv", "pt_beta",
                "dBeta", "dBetaCut2", "dBetaLum2", "dBetaMuls", "dBetaRes", "dBetaRIn2", "dBetaROut2")
MLP_FEATURES = 12
MLP_PARAMS = 5057


class SDLError(RuntimeError):
    pass


_LIB = None


def lib():
    """Load libsdlgpu.so (raises if it is missing: there is no fallback)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise SDLError("libsdlgpu.so is not built (run __graft_entry__.build() or sdl_gb300/build.py)")
        L = ctypes.CDLL(LIB_PATH)
        vp, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
        L.sdlg_create.argtypes = [ctypes.POINTER(vp), i32]
        L.sdlg_destroy.argtypes = [vp]
        L.sdlg_last_error.argtypes = [vp]
        L.sdlg_last_error.restype = ctypes.c_char_p
        L.sdlg_geometry_load_files.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
        L.sdlg_geometry_upload.argtypes = [vp, i64, vp, vp, i64, vp, vp, i64, vp, vp, vp]
        L.sdlg_get_tracklet_vars.argtypes = [vp, i64, vp, i64, vp]
        L.sdlg_geometry_convert.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
        L.sdlg_geometry_load_binary.argtypes = [vp, ctypes.c_char_p]
        L.sdlg_num_modules.argtypes = [vp]
        L.sdlg_num_modules.restype = i64
        L.sdlg_set_events.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp]
        L.sdlg_stage_events.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp]
        L.sdlg_run.argtypes = [vp, i32, i32]
        L.sdlg_run_async.argtypes = [vp, i32, i32]
        L.sdlg_sync.argtypes = [vp]
        L.sdlg_get_counts.argtypes = [vp, i64, vp]
        L.sdlg_get_objects.argtypes = [vp, i32, i64, vp, i64, vp]
        L.sdlg_get_objects_async.argtypes = [vp, i32, i64, vp, i64, vp]
        L.sdlg_wait_objects.argtypes = [vp]
        L.sdlg_get_counters.argtypes = [vp, i64, vp]
        L.sdlg_last_times.argtypes = [vp, vp]
        L.sdlg_last_kernel_times.argtypes = [vp, vp]
        L.sdlg_last_tl_pass_times.argtypes = [vp, vp]
        L.sdlg_last_tl_pass_times4.argtypes = [vp, vp]
        L.sdlg_tl_b2_filter_check.argtypes = [vp, vp]
        L.sdlg_last_tl_list_counts.argtypes = [vp, vp]
        L.sdlg_math_check.argtypes = [vp, i32, i32, ctypes.c_uint64, i64, ctypes.c_uint64, vp]
        L.sdlg_tl_phase_a_check.argtypes = [vp, vp]
        L.sdlg_autotune.argtypes = [vp, i32, i32, vp]
        L.sdlg_last_launches.argtypes = [vp]
        L.sdlg_last_launches.restype = i64
        L.sdlg_mini_doublets_static.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, i64, vp, vp, vp]
        L.sdlg_run_stages.argtypes = [vp, i32, i32, i32]
        L.sdlg_set_capacities.argtypes = [vp, vp]
        L.sdlg_build_line_map.argtypes = [i32, vp, i64, vp, vp, vp, i64, i64, vp, vp, vp, vp, vp]
        L.sdlg_get_capacities.argtypes = [vp, vp]
        L.sdlg_get_object_links.argtypes = [vp, i32, i64, vp, vp, vp, i64, vp]
        L.sdlg_get_module_detids.argtypes = [vp, vp, i64, vp]
        L.sdlg_module_info.argtypes = [ctypes.c_uint32, vp]
        L.sdlg_hit_derived.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp]
        L.sdlg_libm_eval.argtypes = [vp, i32, ctypes.c_uint32, i64, vp]
        L.sdlg_libm_stats.argtypes = [i32, vp]
        L.sdlg_host_alloc.argtypes = [vp, i64, ctypes.POINTER(vp)]
        L.sdlg_host_free.argtypes = [vp, vp]
        u64, f32 = ctypes.c_uint64, ctypes.c_float
        L.sdlg_mlp_set_params.argtypes = [vp, vp, f32]
        L.sdlg_mlp_get_params.argtypes = [vp, vp, vp]
        L.sdlg_mlp_set_threshold.argtypes = [vp, f32]
        L.sdlg_mlp_init.argtypes = [vp, u64]
        L.sdlg_mlp_collect.argtypes = [vp, f32, u64, vp]
        L.sdlg_mlp_add_samples.argtypes = [vp, i64, vp, vp]
        L.sdlg_mlp_num_samples.argtypes = [vp, vp]
        L.sdlg_mlp_get_samples.argtypes = [vp, vp, vp, i64, vp]
        L.sdlg_mlp_clear_samples.argtypes = [vp]
        L.sdlg_mlp_train.argtypes = [vp, i32, i32, f32, f32, u64, vp]
        L.sdlg_mlp_gradient.argtypes = [vp, i64, vp, vp, vp, vp, vp]
        L.sdlg_mlp_score.argtypes = [vp, i64, vp, vp]
        L.sdlg_mlp_stats.argtypes = [vp, vp]
        _LIB = L
    return _LIB


def module_info(detid: int) -> dict:
    """SDL::Module's detId decoding (no device needed)."""
    out = np.zeros(11, dtype=np.uint32)
    rc = lib().sdlg_module_info(int(detid), out.ctypes.data)
    keys = ("subdet", "side", "layer", "rod", "ring", "module", "isLower", "isInverted", "partnerDetId",
            "moduleType", "moduleLayerType")
    d = {k: int(v) for k, v in zip(keys, out)}
    d["valid"] = rc == 0
    return d


def hit_derived(x, y, z):
    """SDL::Hit's derived quantities (rt, phi, eta, r3) of float32 points (no device needed)."""
    x, y, z = (np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z))
    out = [np.empty(len(x), dtype=np.float32) for _ in range(4)]
    rc = lib().sdlg_hit_derived(len(x), x.ctypes.data, y.ctypes.data, z.ctypes.data, *[o.ctypes.data for o in out])
    if rc != 0:
        raise SDLError("%d: sdlg_hit_derived" % rc)
    return tuple(out)


class LineMapLayout(ctypes.Structure):
    """sdlg_line_map_layout of include/sdl_gpu.h"""
    _fields_ = [("barrel_r", ctypes.c_double * 6), ("barrel_nphi", ctypes.c_int32 * 6), ("zmax", ctypes.c_double),
                ("module_dz", ctypes.c_double), ("flat_zmax_tilted", ctypes.c_double), ("lum_z", ctypes.c_double),
                ("radius_1gev", ctypes.c_double), ("n_tilt_rings", ctypes.c_int32), ("has_tilt", ctypes.c_int32),
                ("has_endcap", ctypes.c_int32), ("disk_z", ctypes.c_double * 5), ("disk_nrings", ctypes.c_int32 * 5),
                ("ec_rmin", ctypes.c_double), ("ec_rmax", ctypes.c_double)]


def line_map(det, device: int = 0) -> dict:
    """The straight-line module connection map of a synthetic detector
    (sdl_gb300.synth), built on the GPU (sdlg_build_line_map): lower detId ->
    sorted list of the connected lower detIds."""
    from . import synth
    lay = LineMapLayout()
    for i in range(6):
        lay.barrel_r[i] = synth.BARREL_R[i]
        lay.barrel_nphi[i] = det.n_phi(i + 1)
    lay.zmax, lay.module_dz, lay.flat_zmax_tilted = synth.ZMAX, synth.MOD_DZ, synth.FLAT_ZMAX_TILTED
    lay.lum_z, lay.radius_1gev = synth.LUM_Z, 1.0 / synth.KR
    lay.n_tilt_rings, lay.has_tilt, lay.has_endcap = synth.N_TILT_RINGS, int(det.has_tilt), int(det.has_endcap)
    for i in range(5):
        lay.disk_z[i] = synth.DISK_Z[i]
        lay.disk_nrings[i] = synth.DISK_NRINGS[i]
    lay.ec_rmin, lay.ec_rmax = synth.EC_RMIN, synth.EC_RMAX
    idx = np.nonzero(det.is_inner)[0]
    detid = np.ascontiguousarray(det.detid[idx], dtype=np.uint32)
    kind = np.ascontiguousarray(det.kind[idx], dtype=np.int8)
    geom = np.ascontiguousarray(np.concatenate(
        [det.center[idx], det.taxis[idx], det.uaxis[idx]] +
        [getattr(det, k)[idx][:, None] for k in ("half_t", "half_z", "r0", "r1", "phic", "dphi", "tilt")], axis=1),
        dtype=np.float64)
    nk, nd = ctypes.c_int64(), ctypes.c_int64()
    L = lib()
    args = (device, ctypes.byref(lay), len(idx), detid.ctypes.data, kind.ctypes.data, geom.ctypes.data)
    rc = L.sdlg_build_line_map(*args, 0, 0, None, None, None, ctypes.byref(nk), ctypes.byref(nd))
    if rc != 0:
        raise SDLError("%d: sdlg_build_line_map" % rc)
    keys = np.empty(nk.value, np.uint32)
    off = np.empty(nk.value + 1, np.int64)
    dst = np.empty(nd.value, np.uint32)
    rc = L.sdlg_build_line_map(*args, nk.value, nd.value, keys.ctypes.data, off.ctypes.data, dst.ctypes.data,
                               ctypes.byref(nk), ctypes.byref(nd))
    if rc != 0:
        raise SDLError("%d: sdlg_build_line_map" % rc)
    return {int(k): [int(v) for v in dst[off[i]:off[i + 1]]] for i, k in enumerate(keys)}


def geometry_convert(tilted, endcap, cmap, out_path):
    """Parse the three geometry text files (any may be None) into one binary
    file for Chain.load_binary (no device needed)."""
    enc = lambda p: p.encode() if p else None
    rc = lib().sdlg_geometry_convert(enc(tilted), enc(endcap), enc(cmap), out_path.encode())
    if rc != 0:
        raise SDLError("%d: cannot convert the geometry files" % rc)


class Chain:
    """One device context: geometry, a batch of events and their results."""

    def __init__(self, device: int = 0):
        L = lib()
        h = ctypes.c_void_p()
        rc = L.sdlg_create(ctypes.byref(h), device)
        if rc != 0:
            raise SDLError("sdlg_create failed (%d): no usable CUDA device %d" % (rc, device))
        self.h = h
        self._pinned = []

    def close(self):
        if getattr(self, "h", None):
            lib().sdlg_wait_objects(self.h)  # no readback may still be writing pinned memory
            for p in self._pinned:
                lib().sdlg_host_free(self.h, p)
            self._pinned = []
            lib().sdlg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc != 0:
            raise SDLError("%d: %s" % (rc, lib().sdlg_last_error(self.h).decode()))

    # geometry -------------------------------------------------------------
    def load_files(self, tilted=None, endcap=None, cmap=None):
        enc = lambda p: p.encode() if p else None
        self._ck(lib().sdlg_geometry_load_files(self.h, enc(tilted), enc(endcap), enc(cmap)))

    def load_binary(self, path):
        """Geometry from a binary file written by :func:`geometry_convert`."""
        self._ck(lib().sdlg_geometry_load_binary(self.h, path.encode()))

    def upload_tables(self, t_id, t_val, e_id, e_val, keys, off, dst):
        arrs = [np.ascontiguousarray(a, dtype=d) for a, d in
                ((t_id, np.uint32), (t_val, np.float32), (e_id, np.uint32), (e_val, np.float32),
                 (keys, np.uint32), (off, np.int64), (dst, np.uint32))]
        t_id, t_val, e_id, e_val, keys, off, dst = arrs
        self._ck(lib().sdlg_geometry_upload(self.h, len(t_id), t_id.ctypes.data, t_val.ctypes.data, len(e_id),
                                            e_id.ctypes.data, e_val.ctypes.data, len(keys), keys.ctypes.data,
                                            off.ctypes.data, dst.ctypes.data))

    def upload_detector(self, det):
        """Geometry tables of a :class:`sdl_gb300.synth.Detector`."""
        self.upload_tables(*det.tables())

    @property
    def num_modules(self) -> int:
        return int(lib().sdlg_num_modules(self.h))

    # events -----------------------------------------------------------------
    def pinned(self, nbytes: int) -> np.ndarray:
        """A pinned host byte buffer owned by this context."""
        p = ctypes.c_void_p()
        self._ck(lib().sdlg_host_alloc(self.h, nbytes, ctypes.byref(p)))
        self._pinned.append(p)
        return np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(p.value))

    @staticmethod
    def _event_arrays(events, ev_off, x, y, z, idx, detid):
        if events is not None:
            ev_off = np.zeros(len(events) + 1, dtype=np.int64)
            ev_off[1:] = np.cumsum([len(e.x) for e in events])
            x = np.concatenate([e.x for e in events])
            y = np.concatenate([e.y for e in events])
            z = np.concatenate([e.z for e in events])
            idx = np.concatenate([e.idx for e in events])
            detid = np.concatenate([e.detid for e in events])
        ev_off = np.ascontiguousarray(ev_off, dtype=np.int64)
        arrs = [np.ascontiguousarray(a, dtype=d) for a, d in
                ((x, np.float32), (y, np.float32), (z, np.float32), (idx, np.int32), (detid, np.uint32))]
        return ev_off, arrs

    def set_events(self, events=None, *, ev_off=None, x=None, y=None, z=None, idx=None, detid=None):
        """Either a list of objects with x/y/z/idx/detid arrays, or the
        concatenated arrays with ev_off (int64, n_events + 1)."""
        ev_off, arrs = self._event_arrays(events, ev_off, x, y, z, idx, detid)
        self._ck(lib().sdlg_set_events(self.h, len(ev_off) - 1, ev_off.ctypes.data, *[a.ctypes.data for a in arrs]))
        self.n_events = len(ev_off) - 1
        self._staged = None

    def set_events_raw(self, n_events, ev_off_ptr, x_ptr, y_ptr, z_ptr, idx_ptr, det_ptr):
        self._ck(lib().sdlg_set_events(self.h, n_events, ev_off_ptr, x_ptr, y_ptr, z_ptr, idx_ptr, det_ptr))
        self.n_events = n_events
        self._staged = None

    def stage_events(self, events=None, *, ev_off=None, x=None, y=None, z=None, idx=None, detid=None):
        """The next batch (arguments as set_events), copied to the device
        while a run may still be going; the next run from the hits
        (run, run_async, autotune) takes it as its events."""
        ev_off, arrs = self._event_arrays(events, ev_off, x, y, z, idx, detid)
        self._ck(lib().sdlg_stage_events(self.h, len(ev_off) - 1, ev_off.ctypes.data, *[a.ctypes.data for a in arrs]))
        self._staged = len(ev_off) - 1

    def stage_events_raw(self, n_events, ev_off_ptr, x_ptr, y_ptr, z_ptr, idx_ptr, det_ptr):
        self._ck(lib().sdlg_stage_events(self.h, n_events, ev_off_ptr, x_ptr, y_ptr, z_ptr, idx_ptr, det_ptr))
        self._staged = n_events

    def _take_staged(self):
        if getattr(self, "_staged", None) is not None:
            self.n_events = self._staged
            self._staged = None

    # running ----------------------------------------------------------------
    def run(self, stop_after: int = 4, flags: int = 0):
        self._take_staged()
        self._ck(lib().sdlg_run(self.h, stop_after, flags))

    def set_capacities(self, caps):
        """Starting capacities (MD, SG, TL, TP, TC, pre-filter list; 0 = default);
        frees the batch: call set_events next."""
        c = np.ascontiguousarray(caps, dtype=np.int64)
        if c.size != 6:
            raise ValueError("six capacities")
        self._ck(lib().sdlg_set_capacities(self.h, c.ctypes.data))

    def capacities(self) -> np.ndarray:
        out = np.zeros(6, dtype=np.int64)
        self._ck(lib().sdlg_get_capacities(self.h, out.ctypes.data))
        return out

    def run_stages(self, first: int, last: int, flags: int = 0):
        """Stages first..last (one create* call at a time): continues the last
        run when `first` follows its final stage, else runs from the hits."""
        if int(first) == 0:
            self._take_staged()
        self._ck(lib().sdlg_run_stages(self.h, int(first), int(last), int(flags)))

    def run_async(self, stop_after: int = 4, flags: int = 0):
        self._take_staged()
        self._ck(lib().sdlg_run_async(self.h, stop_after, flags))

    def sync(self):
        self._ck(lib().sdlg_sync(self.h))

    # results ----------------------------------------------------------------
    def counts(self, event: int = -1) -> np.ndarray:
        out = np.zeros(5, dtype=np.int64)
        self._ck(lib().sdlg_get_counts(self.h, event, out.ctypes.data))
        return out

    def objects(self, stage: int, event: int = -1, out: np.ndarray | None = None) -> np.ndarray:
        """Hit-index tuples of a stage's objects (all events: event = -1).
        `out` (int32, C-contiguous, at least as many rows as objects and the
        stage's width), e.g. a view of pinned() memory, is filled and its
        first rows returned; otherwise a new array is."""
        n = ctypes.c_int64()
        self._ck(lib().sdlg_get_objects(self.h, stage, event, None, 0, ctypes.byref(n)))
        if out is None:
            out = np.empty((n.value, WIDTH[stage]), dtype=np.int32)
        elif (out.dtype != np.int32 or out.ndim != 2 or out.shape[1] != WIDTH[stage] or out.shape[0] < n.value
              or not out.flags.c_contiguous):
            raise ValueError("out must be a C-contiguous int32 array of shape (>= %d, %d)" % (n.value, WIDTH[stage]))
        if n.value:
            self._ck(lib().sdlg_get_objects(self.h, stage, event, out.ctypes.data, n.value, ctypes.byref(n)))
        return out[:n.value]

    def objects_async(self, stage: int, event: int, out: np.ndarray) -> int:
        """Start reading a stage's tuples into `out` (int32, C-contiguous,
        shape (>= n, width); pinned() memory for the copy to overlap the next
        run) and return n without waiting: `out` holds them once
        wait_objects() returns.  The tuples are gathered and copied on a
        second stream; the next set_events may follow at once, and the next
        run starts once they are gathered."""
        n = ctypes.c_int64()
        self._ck(lib().sdlg_get_objects(self.h, stage, event, None, 0, ctypes.byref(n)))
        if (out.dtype != np.int32 or out.ndim != 2 or out.shape[1] != WIDTH[stage] or out.shape[0] < n.value
                or not out.flags.c_contiguous):
            raise ValueError("out must be a C-contiguous int32 array of shape (>= %d, %d)" % (n.value, WIDTH[stage]))
        self._ck(lib().sdlg_get_objects_async(self.h, stage, event, out.ctypes.data, out.shape[0], ctypes.byref(n)))
        return n.value

    def wait_objects(self):
        """Wait for the readback objects_async() started."""
        self._ck(lib().sdlg_wait_objects(self.h))

    def links(self, stage: int, event: int = 0):
        """The object graph of one event's stage: (constituents n x 2 as
        indices into the stage below -- hits in input order for
        mini-doublets --, inner lower module index n, per-object floats
        n x nv with nv 4 for mini-doublets, 6 for segments, 0 otherwise)."""
        n = ctypes.c_int64()
        self._ck(lib().sdlg_get_object_links(self.h, stage, event, None, None, None, 0, ctypes.byref(n)))
        nv = {0: 4, 1: 6}.get(stage, 0)
        lk = np.empty((n.value, 2), dtype=np.int32)
        md = np.empty(n.value, dtype=np.int32)
        vals = np.empty((n.value, nv), dtype=np.float32)
        if n.value:
            self._ck(lib().sdlg_get_object_links(self.h, stage, event, lk.ctypes.data, md.ctypes.data,
                                                 vals.ctypes.data if nv else None, n.value, ctypes.byref(n)))
        return lk, md, vals

    def module_detids(self) -> np.ndarray:
        n = ctypes.c_int64()
        self._ck(lib().sdlg_get_module_detids(self.h, None, 0, ctypes.byref(n)))
        out = np.empty(n.value, dtype=np.uint32)
        self._ck(lib().sdlg_get_module_detids(self.h, out.ctypes.data, n.value, ctypes.byref(n)))
        return out

    def libm_eval(self, fn: int, start_bits: int, n: int) -> np.ndarray:
        """The chain's value of the host libm's float function fn (0 asin,
        1 atan, 2 sin, 3 cos, 4 tan) on n consecutive float bit patterns."""
        out = np.empty(n, dtype=np.float32)
        self._ck(lib().sdlg_libm_eval(self.h, int(fn), int(start_bits), int(n), out.ctypes.data))
        return out

    @staticmethod
    def libm_stats(fn: int) -> dict:
        out = np.zeros(3, dtype=np.uint64)
        rc = lib().sdlg_libm_stats(int(fn), out.ctypes.data)
        if rc != 0:
            raise SDLError("%d: sdlg_libm_stats" % rc)
        return {"tabulated": int(out[0]), "moved": int(out[1]), "exceptions": int(out[2])}

    def tracklet_vars(self, event: int = -1) -> np.ndarray:
        """The tracklets' final cut variables (rows as objects(2, event), columns
        TL_VAR_NAMES), as the reference's Tracklet recovars."""
        n = ctypes.c_int64()
        self._ck(lib().sdlg_get_tracklet_vars(self.h, event, None, 0, ctypes.byref(n)))
        out = np.empty((n.value, len(TL_VAR_NAMES)), dtype=np.float32)
        if n.value:
            self._ck(lib().sdlg_get_tracklet_vars(self.h, event, out.ctypes.data, n.value, ctypes.byref(n)))
        return out

    def counters(self, event: int = 0) -> np.ndarray:
        out = np.zeros(110, dtype=np.uint32)
        self._ck(lib().sdlg_get_counters(self.h, event, out.ctypes.data))
        return out

    def kernel_times(self) -> np.ndarray:
        """Device ms of each stage's candidate-evaluation kernel in the last run."""
        out = np.zeros(5, dtype=np.float32)
        self._ck(lib().sdlg_last_kernel_times(self.h, out.ctypes.data))
        return out

    @property
    def launches(self) -> int:
        """Kernels one run of the chain launches."""
        return int(lib().sdlg_last_launches(self.h))

    def mini_doublets_static(self, n_hits, d_x, d_y, d_z, d_idx, d_detid, d_pairs, pair_cap, d_count, d_status,
                             stream=None):
        """Allocation-free mini-doublets of one event (device pointers in and
        out, working memory in the library's fixed array); see
        sdlg_mini_doublets_static in include/sdl_gpu.h."""
        self._ck(lib().sdlg_mini_doublets_static(self.h, n_hits, d_x, d_y, d_z, d_idx, d_detid, d_pairs, pair_cap,
                                                 d_count, d_status, stream))

    def times(self) -> np.ndarray:
        """Device ms of the last run: ingest, MD, SG, TL, TP, TC, total."""
        out = np.zeros(7, dtype=np.float32)
        self._ck(lib().sdlg_last_times(self.h, out.ctypes.data))
        return out

    # ---------------------------------------------------------------- pre-filter
    def mlp_set_params(self, params, threshold: float = 0.0):
        """Load the pre-filter's FP32 parameter vector (MLP_PARAMS floats) and
        logit threshold."""
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != MLP_PARAMS:
            raise SDLError("expected %d parameters, got %d" % (MLP_PARAMS, p.size))
        self._ck(lib().sdlg_mlp_set_params(self.h, p.ctypes.data, float(threshold)))

    def mlp_params(self):
        """(parameters, threshold)"""
        p = np.empty(MLP_PARAMS, dtype=np.float32)
        t = ctypes.c_float()
        self._ck(lib().sdlg_mlp_get_params(self.h, p.ctypes.data, ctypes.addressof(t)))
        return p, float(t.value)

    def mlp_set_threshold(self, threshold: float):
        self._ck(lib().sdlg_mlp_set_threshold(self.h, float(threshold)))

    def mlp_init(self, seed: int = 0):
        self._ck(lib().sdlg_mlp_init(self.h, int(seed)))

    def mlp_collect(self, neg_keep: float = 1.0, seed: int = 0) -> int:
        """Append training samples from the last run's tracklet candidates;
        returns the number of samples held."""
        n = ctypes.c_int64()
        self._ck(lib().sdlg_mlp_collect(self.h, float(neg_keep), int(seed), ctypes.addressof(n)))
        return int(n.value)

    def mlp_add_samples(self, x, y):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, MLP_FEATURES)
        y = np.ascontiguousarray(y, dtype=np.float32).reshape(-1)
        self._ck(lib().sdlg_mlp_add_samples(self.h, len(y), x.ctypes.data, y.ctypes.data))

    def mlp_num_samples(self) -> int:
        n = ctypes.c_int64()
        self._ck(lib().sdlg_mlp_num_samples(self.h, ctypes.addressof(n)))
        return int(n.value)

    def mlp_samples(self):
        """(features n x 12, labels n) of the training set"""
        n = self.mlp_num_samples()
        x = np.empty((n, MLP_FEATURES), dtype=np.float32)
        y = np.empty(n, dtype=np.float32)
        m = ctypes.c_int64()
        self._ck(lib().sdlg_mlp_get_samples(self.h, x.ctypes.data, y.ctypes.data, n, ctypes.addressof(m)))
        return x, y

    def mlp_labels(self) -> np.ndarray:
        """labels of the training set (1: accepted by the tracklet cuts)"""
        n = self.mlp_num_samples()
        y = np.empty(n, dtype=np.float32)
        m = ctypes.c_int64()
        self._ck(lib().sdlg_mlp_get_samples(self.h, None, y.ctypes.data, n, ctypes.addressof(m)))
        return y

    def mlp_clear_samples(self):
        self._ck(lib().sdlg_mlp_clear_samples(self.h))

    def mlp_train(self, epochs: int, batch: int = 4096, lr: float = 2e-3, pos_weight: float = 4.0, seed: int = 0):
        """Train on the GPU (the library's forward / backward / Adam kernels);
        returns the mean loss of each epoch."""
        out = np.zeros(max(epochs, 1), dtype=np.float32)
        self._ck(lib().sdlg_mlp_train(self.h, int(epochs), int(batch), float(lr), float(pos_weight), int(seed),
                                      out.ctypes.data))
        return out[:epochs]

    def mlp_gradient(self, x, y, w):
        """(gradient, loss) of mean_i w_i * logistic loss at the current parameters"""
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, MLP_FEATURES)
        y = np.ascontiguousarray(y, dtype=np.float32).reshape(-1)
        w = np.ascontiguousarray(w, dtype=np.float32).reshape(-1)
        g = np.empty(MLP_PARAMS, dtype=np.float32)
        loss = ctypes.c_double()
        self._ck(lib().sdlg_mlp_gradient(self.h, len(y), x.ctypes.data, y.ctypes.data, w.ctypes.data, g.ctypes.data,
                                         ctypes.addressof(loss)))
        return g, float(loss.value)

    def mlp_score(self, x) -> np.ndarray:
        """Logits of feature rows through the tensor-core kernel."""
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, MLP_FEATURES)
        z = np.empty(len(x), dtype=np.float32)
        self._ck(lib().sdlg_mlp_score(self.h, len(x), x.ctypes.data, z.ctypes.data))
        return z

    def tl_pass_times(self) -> np.ndarray:
        """Device ms of the last run's tracklet passes: enumeration + float cuts,
        the pre-filter (0 without FLAG_MLP), the single-precision phase-B2
        filter, the double-precision cuts."""
        out = np.zeros(4, dtype=np.float32)
        self._ck(lib().sdlg_last_tl_pass_times4(self.h, out.ctypes.data))
        return out

    def tl_list_counts(self) -> dict:
        """Entries of the last run's tracklet candidate lists: phase-A survivors,
        those the pre-filter kept (0 without FLAG_MLP), and what the phase-B2
        filter left of the list before it (the exact phases' input)."""
        out = np.zeros(3, dtype=np.int64)
        self._ck(lib().sdlg_last_tl_list_counts(self.h, out.ctypes.data))
        return {"listed": int(out[0]), "kept": int(out[1]), "filtered": int(out[2])}

    def tl_b2_filter_check(self) -> dict:
        """Self-check of the single-precision phase-B2 filter over the last
        run's phase-A survivors against the exact phases B1 and B2."""
        out = np.zeros(12, dtype=np.uint64)
        self._ck(lib().sdlg_tl_b2_filter_check(self.h, out.ctypes.data))
        r = out[6:9].astype(np.uint32).view(np.float32)
        return {"entries": int(out[0]), "b1_pass": int(out[1]), "b2_pass": int(out[2]), "rejected": int(out[3]),
                "violations": int(out[4]), "rejected_of_b1_pass": int(out[5]),
                "bound_ratio": {"dbeta": float(r[0]), "cut2": float(r[1]), "betaout": float(r[2])},
                "undecided_early": int(out[9]), "accepted": int(out[10]), "accept_violations": int(out[11])}

    def autotune(self, stop_after: int = 4, flags: int = 0) -> dict:
        """Pick the fastest launch shape per stage on the current batch (kept for later runs)."""
        out = np.zeros(10, dtype=np.int32)
        self._take_staged()
        self._ck(lib().sdlg_autotune(self.h, int(stop_after), int(flags), out.ctypes.data))
        return {"task": [int(v) for v in out[:5]], "ctas_per_sm": [int(v) for v in out[5:]]}

    def math_check(self, fn: int, n: int, *, start: int = 0, exhaustive: bool = False, seed: int = 0) -> dict:
        """Self-check of a float-float fast path against the double evaluation."""
        out = np.zeros(8, dtype=np.uint64)
        self._ck(lib().sdlg_math_check(self.h, int(fn), 1 if exhaustive else 0, int(start), int(n), int(seed),
                                       out.ctypes.data))
        return {"answered": int(out[0]), "mismatches": int(out[1]),
                "first": [int(v) for v in out[3:8]] if out[2] else None}

    def tl_phase_a_check(self) -> dict:
        """Self-check of the tracklet enumeration's single-precision decisions
        (phase A, then phase B1) over the last run's candidates: how many they
        settled alone, how many needed an exact evaluation, and how many they
        settled differently from the exact cuts (0)."""
        out = np.zeros(4, dtype=np.uint64)
        self._ck(lib().sdlg_tl_phase_a_check(self.h, out.ctypes.data))
        return {"candidates": int(out[0]), "settled": int(out[1]), "exact": int(out[2]), "mismatches": int(out[3])}

    def mlp_stats(self) -> dict:
        """Pre-filter counts of the last run with FLAG_MLP: tracklet candidates,
        those through the float cuts and the enumeration's phase-B1 decision
        (scored by the network), those kept."""
        out = np.zeros(4, dtype=np.int64)
        self._ck(lib().sdlg_mlp_stats(self.h, out.ctypes.data))
        return {"candidates": int(out[0]), "scored": int(out[1]), "kept": int(out[2]), "timeouts": int(out[3])}
