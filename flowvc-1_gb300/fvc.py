"""ctypes binding of libfvc.so (include/fvc.h) for Python callers and tests.

The engine's public interface is the C ABI; this module is a thin wrapper
that passes numpy arrays as plain pointers.  It never computes anything on
the CPU: if the shared library cannot be loaded, or no GPU is present, every
call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libfvc.so")

PREC_FP64, PREC_BF16, PREC_FP16 = 0, 1, 2
PRECISIONS = {"fp64": PREC_FP64, "bf16": PREC_BF16, "fp16": PREC_FP16}
FVC_OK, FVC_ERR_IO, FVC_ERR_ARG, FVC_ERR_OOM, FVC_ERR_WALK, FVC_ERR_TIMEOUT, FVC_ERR_CUDA, FVC_ERR_STATE, FVC_ERR_TLOC = range(9)
STATUS_NAMES = {0: "FVC_OK", 1: "FVC_ERR_IO", 2: "FVC_ERR_ARG", 3: "FVC_ERR_OOM", 4: "FVC_ERR_WALK",
                5: "FVC_ERR_TIMEOUT", 6: "FVC_ERR_CUDA", 7: "FVC_ERR_STATE", 8: "FVC_ERR_TLOC"}

# every entry point include/fvc.h declares, with its C signature
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_llp = C.POINTER(C.c_longlong)
_vp = C.c_void_p


class Opts(C.Structure):
    _fields_ = [("device", C.c_int), ("dims", C.c_int), ("mesh_type", C.c_int), ("max_hops", C.c_int)]


class FtleSpec(C.Structure):
    _fields_ = [("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double), ("ymax", C.c_double),
                ("zmin", C.c_double), ("zmax", C.c_double), ("xres", C.c_int), ("yres", C.c_int),
                ("zres", C.c_int), ("local_search_checking", C.c_int), ("start_time", C.c_double),
                ("stop_time", C.c_double), ("generate", C.c_int)]


class TracerSpec(C.Structure):
    _fields_ = [("local_search_checking", C.c_int), ("seed_chain", C.c_int), ("center", C.c_double * 3)]


class JobStats(C.Structure):
    _fields_ = [("intervals", C.c_longlong), ("steps_main", C.c_longlong), ("steps_early", C.c_longlong),
                ("ms_main", C.c_double), ("ms_early", C.c_double), ("ms_reduce", C.c_double),
                ("ms_setup", C.c_double), ("launches", C.c_longlong), ("steps_early_recorded", C.c_longlong)]


class BatchOpts(C.Structure):
    _fields_ = [("tmin", C.c_double), ("tdelta", C.c_double), ("tres", C.c_int), ("periodic", C.c_int),
                ("hbm_budget", C.c_longlong), ("max_jobs", C.c_int), ("resort_every", C.c_int),
                ("tick_intervals", C.c_int)]


class BatchJobSpec(C.Structure):
    _fields_ = [("kind", C.c_int), ("t_start", C.c_double), ("t_stop", C.c_double), ("n", C.c_int),
                ("seeds", C.POINTER(C.c_double)), ("local_search_checking", C.c_int), ("grid", FtleSpec)]


class BatchResult(C.Structure):
    _fields_ = [("kind", C.c_int), ("n", C.c_longlong), ("X", _dp), ("eid", _ip), ("left", _ip), ("ldt", _dp),
                ("rt", _dp), ("ftle_wT", _dp), ("ftle_woT", _dp)]


class BatchStats(C.Structure):
    _fields_ = [("ticks", C.c_longlong), ("graphs", C.c_longlong), ("launches", C.c_longlong),
                ("steps", C.c_longlong), ("jobs_submitted", C.c_longlong), ("jobs_done", C.c_longlong),
                ("ms_run", C.c_double), ("tuned_threads", C.c_int), ("tuned_blocks", C.c_int),
                ("tuned_resort", C.c_int), ("hbm_used", C.c_longlong)]


JOB_TRACERS, JOB_RESIDENCE, JOB_FTLE = 0, 1, 2
BATCH_QUEUED, BATCH_RUNNING, BATCH_DONE, BATCH_FAILED, BATCH_RELEASED = range(5)

SIGNATURES = {
    "fvc_abi_version": (C.c_int, []),
    "fvc_create": (C.c_int, [C.POINTER(_vp), C.POINTER(Opts)]),
    "fvc_destroy": (None, [_vp]),
    "fvc_last_error": (C.c_char_p, [_vp]),
    "fvc_set_cart_mesh": (C.c_int, [_vp, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double, C.c_int,
                                    C.c_double, C.c_double, C.c_int]),
    "fvc_set_unstruct_mesh": (C.c_int, [_vp, C.c_int, _dp, C.c_int, _ip, _ip]),
    "fvc_set_bounds": (C.c_int, [_vp, _dp]),
    "fvc_set_integrator": (C.c_int, [_vp, C.c_int, C.c_double, C.c_int]),
    "fvc_upload_frame": (C.c_int, [_vp, C.c_int, _dp]),
    "fvc_set_window": (C.c_int, [_vp, C.c_int, C.c_int, C.c_double, C.c_double]),
    "fvc_set_precision": (C.c_int, [_vp, C.c_int]),
    "fvc_set_rkf": (C.c_int, [_vp, C.c_double, C.c_double, C.c_double]),
    "fvc_advect": (C.c_int, [_vp, C.c_int, _dp, _dp, _ip, _ip, _dp, C.c_double, C.c_double, _llp]),
    "fvc_advect_device": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp, C.c_double, C.c_double, _llp]),
    "fvc_advect_noalloc": (C.c_int, [_vp, C.c_int, _dp, _dp, _ip, _ip, _dp, C.c_double, C.c_double, _llp]),
    "fvc_velocity": (C.c_int, [_vp, C.c_int, _dp, _ip, _ip, C.c_double, _dp]),
    "fvc_local_search": (C.c_int, [_vp, C.c_int, _dp, _ip, _ip]),
    "fvc_global_search": (C.c_int, [_vp, C.c_int, _dp, _ip]),
    "fvc_ftle_create": (C.c_int, [_vp, C.POINTER(FtleSpec), C.POINTER(_vp)]),
    "fvc_ftle_set_state": (C.c_int, [_vp, _dp, _ip, _ip, _dp, _ip, _dp, _dp]),
    "fvc_ftle_get_state": (C.c_int, [_vp, _dp, _ip, _ip, _dp, _ip, _dp, _dp]),
    "fvc_ftle_interval": (C.c_int, [_vp, C.c_int, C.c_double, C.c_double, _llp]),
    "fvc_ftle_reduce": (C.c_int, [_vp, C.c_double, _dp, _dp]),
    "fvc_tracer_create": (C.c_int, [_vp, C.POINTER(TracerSpec), C.c_int, _dp, C.POINTER(_vp)]),
    "fvc_tracer_launch": (C.c_int, [_vp, C.c_double]),
    "fvc_tracer_advance": (C.c_int, [_vp, C.c_double, C.c_double, _llp]),
    "fvc_tracer_snapshot": (C.c_int, [_vp, C.c_int, _dp, _llp]),
    "fvc_tracer_get_state": (C.c_int, [_vp, _dp, _ip, _ip, _dp]),
    "fvc_tracer_output_begin": (C.c_int, [_vp, C.c_int, _llp]),
    "fvc_tracer_output_wait": (C.c_int, [_vp, C.c_longlong, C.POINTER(_dp), _llp]),
    "fvc_tracer_output_release": (C.c_int, [_vp, C.c_longlong]),
    "fvc_job_get_stats": (C.c_int, [_vp, C.POINTER(JobStats)]),
    "fvc_stream": (_vp, [_vp]),
    "fvc_job_destroy": (None, [_vp]),
    "fvc_cet_enable": (C.c_int, [_vp, C.c_int]),
    "fvc_cet_results": (C.c_int, [_vp, C.c_int, _dp, _dp, _ip]),
    "fvc_tracer_residence": (C.c_int, [_vp, C.c_double, C.c_double, _dp]),
    "fvc_upload_frame_async": (C.c_int, [_vp, C.c_int, _dp]),
    "fvc_frame_ready": (C.c_int, [_vp, C.c_int, _ip]),
    "fvc_frame_wait": (C.c_int, [_vp, C.c_int]),
    "fvc_host_alloc": (C.c_int, [C.POINTER(_vp), C.c_size_t]),
    "fvc_host_free": (None, [_vp]),
    "fvc_batch_create": (C.c_int, [_vp, C.POINTER(BatchOpts), C.POINTER(_vp)]),
    "fvc_batch_destroy": (None, [_vp]),
    "fvc_batch_submit": (C.c_int, [_vp, C.POINTER(BatchJobSpec), _ip]),
    "fvc_batch_tick": (C.c_int, [_vp, _ip]),
    "fvc_batch_run": (C.c_int, [_vp, C.c_int]),
    "fvc_batch_autotune": (C.c_int, [_vp]),
    "fvc_batch_poll": (C.c_int, [_vp, C.c_int, _ip]),
    "fvc_batch_tracer_result": (C.c_int, [_vp, C.c_int, _dp, _ip, _ip, _dp]),
    "fvc_batch_residence_result": (C.c_int, [_vp, C.c_int, _dp]),
    "fvc_batch_ftle_result": (C.c_int, [_vp, C.c_int, _dp, _dp]),
    "fvc_batch_job_stats": (C.c_int, [_vp, C.c_int, C.POINTER(JobStats)]),
    "fvc_batch_result_begin": (C.c_int, [_vp, C.c_int, _llp]),
    "fvc_batch_result_ready": (C.c_int, [_vp, C.c_longlong, _ip]),
    "fvc_batch_result_get": (C.c_int, [_vp, C.c_longlong, C.POINTER(BatchResult)]),
    "fvc_batch_result_release": (C.c_int, [_vp, C.c_longlong]),
    "fvc_batch_release": (C.c_int, [_vp, C.c_int]),
    "fvc_batch_get_stats": (C.c_int, [_vp, C.POINTER(BatchStats)]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libfvc.so and declare every entry point; raises if it is missing."""
    global _lib
    if _lib is not None and path == LIB_PATH:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libfvc.so not built ({path}); run __graft_entry__.build()")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _lib = lib
    return lib


class PinnedArray:
    """A float64 numpy array in page-locked host memory (fvc_host_alloc),
    freed with the object."""

    def __init__(self, shape):
        lib = load()
        self.lib = lib
        n = int(np.prod(shape))
        self.p = _vp()
        st = lib.fvc_host_alloc(C.byref(self.p), max(n, 1) * 8)
        if st:
            raise FvcError(st, "fvc_host_alloc failed")
        buf = (C.c_double * max(n, 1)).from_address(self.p.value)
        self.a = np.frombuffer(buf, dtype=np.float64, count=n).reshape(shape)

    def __del__(self):
        try:
            if self.p:
                self.lib.fvc_host_free(self.p)
                self.p = _vp()
        except Exception:
            pass


TRACER_OUTPUT_SLOTS = 4  # FVC_TRACER_OUTPUT_SLOTS of fvc.h
BATCH_RESULT_SLOTS = 8  # FVC_BATCH_RESULT_SLOTS of fvc.h


class FvcError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.reshape(shape) if shape is not None else a


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Context:
    """One fvc_ctx: a mesh, resident frames, a window and integrator settings."""

    def __init__(self, dims, mesh_type, device=0, max_hops=0):
        self.lib = load()
        self.h = _vp()
        o = Opts(device, dims, mesh_type, max_hops)
        st = self.lib.fvc_create(C.byref(self.h), C.byref(o))
        if st:
            raise FvcError(st, "fvc_create failed (no usable GPU?)")
        self.dims, self.mesh_type = dims, mesh_type

    def _chk(self, st):
        if st:
            raise FvcError(st, self.lib.fvc_last_error(self.h).decode())

    def stream(self):
        """The context's cudaStream_t as an integer handle."""
        return self.lib.fvc_stream(self.h) or 0

    def close(self):
        if self.h:
            self.lib.fvc_destroy(self.h)
            self.h = _vp()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- mesh and settings
    def set_cart_mesh(self, xmin, xmax, xres, ymin, ymax, yres, zmin, zmax, zres):
        self._chk(self.lib.fvc_set_cart_mesh(self.h, xmin, xmax, xres, ymin, ymax, yres, zmin, zmax, zres))

    def set_unstruct_mesh(self, xyz, conn, adj):
        xyz, conn, adj = f64(xyz), i32(conn), i32(adj)
        self._chk(self.lib.fvc_set_unstruct_mesh(self.h, xyz.shape[0], _d(xyz), conn.shape[0], _i(conn), _i(adj)))

    def set_bounds(self, b):
        b = f64(b)
        self._chk(self.lib.fvc_set_bounds(self.h, _d(b)))

    def set_integrator(self, int_type, h, extrapolate=0):
        self._chk(self.lib.fvc_set_integrator(self.h, int_type, h, extrapolate))

    def set_rkf(self, accuracy, min_step, max_step):
        """Int_Accuracy, Int_MinTimeStep, Int_MaxTimeStep for Int_Type 2."""
        self._chk(self.lib.fvc_set_rkf(self.h, accuracy, min_step, max_step))

    def upload_frame(self, frame_id, uvw):
        uvw = f64(uvw)
        self._chk(self.lib.fvc_upload_frame(self.h, frame_id, _d(uvw)))

    def upload_frame_async(self, frame_id, uvw):
        """Starts the upload; uvw (a C-contiguous float64 array, pinned for
        overlap) must stay alive and unchanged until frame_wait / frame_ready."""
        assert uvw.dtype == np.float64 and uvw.flags.c_contiguous
        self._chk(self.lib.fvc_upload_frame_async(self.h, frame_id, _d(uvw)))

    def frame_ready(self, frame_id):
        r = C.c_int(0)
        self._chk(self.lib.fvc_frame_ready(self.h, frame_id, C.byref(r)))
        return bool(r.value)

    def frame_wait(self, frame_id):
        self._chk(self.lib.fvc_frame_wait(self.h, frame_id))

    def set_window(self, lo, hi, tmin, tmax):
        self._chk(self.lib.fvc_set_window(self.h, lo, hi, tmin, tmax))

    def set_precision(self, precision):
        """PREC_FP64 (ompVC's arithmetic), PREC_BF16 or PREC_FP16 (mixed form);
        also accepts the names "fp64", "bf16", "fp16"."""
        if isinstance(precision, str):
            precision = PRECISIONS[precision]
        self._chk(self.lib.fvc_set_precision(self.h, precision))

    # ---- step level
    def advect(self, X, V, eid, left, ldt, t0, t1):
        """In-place Advect over arrays; returns the accepted step count."""
        steps = C.c_longlong(0)
        self._chk(self.lib.fvc_advect(self.h, X.shape[0], _d(X), _d(V), _i(eid), _i(left), _d(ldt), t0, t1,
                                      C.byref(steps)))
        return steps.value

    def output_wait(self, ticket):
        """The positions of a queued tracer output as a read-only view of the
        library's page-locked slot (count x 3), valid until output_release.
        Safe to call from another thread than the context's."""
        p, cnt = _dp(), C.c_longlong(0)
        st = self.lib.fvc_tracer_output_wait(self.h, ticket, C.byref(p), C.byref(cnt))
        if st:
            raise FvcError(st, f"fvc_tracer_output_wait: status {st}")
        if cnt.value == 0:
            return np.empty((0, 3))
        a = np.ctypeslib.as_array(p, shape=(cnt.value, 3))
        a.flags.writeable = False
        return a

    def output_release(self, ticket):
        st = self.lib.fvc_tracer_output_release(self.h, ticket)
        if st:
            raise FvcError(st, f"fvc_tracer_output_release: status {st}")

    def advect_noalloc(self, X, V, eid, left, ldt, t0, t1):
        """advect() through fvc_advect_noalloc: same results, no device
        allocation (at most NOALLOC_MAX_POINTS points a call)."""
        steps = C.c_longlong(0)
        self._chk(self.lib.fvc_advect_noalloc(self.h, X.shape[0], _d(X), _d(V), _i(eid), _i(left), _d(ldt), t0,
                                              t1, C.byref(steps)))
        return steps.value

    def velocity(self, X, eid, left, tq):
        out = np.zeros_like(X)
        self._chk(self.lib.fvc_velocity(self.h, X.shape[0], _d(X), _i(eid), _i(left), tq, _d(out)))
        return out

    def local_search(self, X, guess):
        out = np.empty(X.shape[0], np.int32)
        self._chk(self.lib.fvc_local_search(self.h, X.shape[0], _d(f64(X)), _i(i32(guess)), _i(out)))
        return out

    def cet_enable(self, substeps):
        self._chk(self.lib.fvc_cet_enable(self.h, substeps))

    def cet_results(self, ntracers, nelem):
        cet, met, enc = np.empty(nelem), np.empty(nelem), np.empty(nelem, np.int32)
        self._chk(self.lib.fvc_cet_results(self.h, ntracers, _d(cet), _d(met), _i(enc)))
        return cet, met, enc

    def global_search(self, X):
        out = np.empty(X.shape[0], np.int32)
        self._chk(self.lib.fvc_global_search(self.h, X.shape[0], _d(f64(X)), _i(out)))
        return out


class FtleJob:
    def __init__(self, ctx: Context, spec: FtleSpec):
        self.ctx, self.lib = ctx, ctx.lib
        self.h = _vp()
        ctx._chk(self.lib.fvc_ftle_create(ctx.h, C.byref(spec), C.byref(self.h)))
        d = ctx.dims
        self.shape = (spec.xres, spec.yres, spec.zres if d == 3 else 1)
        self.n = int(np.prod(self.shape))

    def interval(self, launch, t1, t2, wait=True):
        """One frame interval; wait=False only queues it (steps: None; faults
        surface at the next call that waits: reduce, get_state, stats)."""
        if not wait:
            self.ctx._chk(self.lib.fvc_ftle_interval(self.h, int(launch), t1, t2, None))
            return None
        steps = C.c_longlong(0)
        self.ctx._chk(self.lib.fvc_ftle_interval(self.h, int(launch), t1, t2, C.byref(steps)))
        return steps.value

    def reduce(self, int_t, out=None, fetch=True):
        """The FTLE fields (fvc_ftle_reduce).  out: (wT, wN) float64 arrays of
        n values to fill (page-locked ones copy fastest); fetch=False leaves
        the fields on the device and returns (None, None)."""
        if not fetch:
            self.ctx._chk(self.lib.fvc_ftle_reduce(self.h, int_t, None, None))
            return None, None
        wT, wN = out if out is not None else (np.empty(self.n), np.empty(self.n))
        assert wT.size == wN.size == self.n and wT.dtype == wN.dtype == np.float64
        self.ctx._chk(self.lib.fvc_ftle_reduce(self.h, int_t, _d(wT), _d(wN)))
        return wT, wN

    def stats(self):
        st = JobStats()
        self.ctx._chk(self.lib.fvc_job_get_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in JobStats._fields_}

    def get_state(self):
        n = self.n
        X, ldt, wT, wN = np.empty((n, 3)), np.empty(n), np.empty(n), np.empty(n)
        eid, left, have = np.empty(n, np.int32), np.empty(n, np.int32), np.empty(n, np.int32)
        self.ctx._chk(self.lib.fvc_ftle_get_state(self.h, _d(X), _i(eid), _i(left), _d(ldt), _i(have), _d(wT), _d(wN)))
        return dict(X=X, eid=eid, left=left, ldt=ldt, have=have, ftT=wT, ftN=wN)

    def set_state(self, s):
        self.ctx._chk(self.lib.fvc_ftle_set_state(
            self.h, _d(f64(s["X"])), _i(i32(s["eid"])), _i(i32(s["left"])), _d(f64(s["ldt"])),
            _i(i32(s["have"])), _d(f64(s["ftT"])), _d(f64(s["ftN"]))))

    def close(self):
        if self.h:
            self.lib.fvc_job_destroy(self.h)
            self.h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TracerJob:
    def __init__(self, ctx: Context, seeds, lsc=1, chain=0, center=(0.0, 0.0, 0.0)):
        self.ctx, self.lib = ctx, ctx.lib
        self.h = _vp()
        seeds = f64(seeds)
        self.n = seeds.shape[0]
        sp = TracerSpec(lsc, chain, (C.c_double * 3)(*center))
        ctx._chk(self.lib.fvc_tracer_create(ctx.h, C.byref(sp), self.n, _d(seeds), C.byref(self.h)))

    def launch(self, t):
        self.ctx._chk(self.lib.fvc_tracer_launch(self.h, t))

    def advance(self, t1, t2, wait=True):
        """Accepted steps of the advance; wait=False queues it and returns
        None (its steps appear in stats())."""
        if not wait:
            self.ctx._chk(self.lib.fvc_tracer_advance(self.h, t1, t2, None))
            return None
        steps = C.c_longlong(0)
        self.ctx._chk(self.lib.fvc_tracer_advance(self.h, t1, t2, C.byref(steps)))
        return steps.value

    def output_begin(self, always=0):
        """Queues an asynchronous output (fvc_tracer_output_begin); returns its ticket."""
        t = C.c_longlong(0)
        self.ctx._chk(self.lib.fvc_tracer_output_begin(self.h, always, C.byref(t)))
        return t.value

    def snapshot(self, always=0):
        out = np.empty((max(self.n, 1), 3))
        cnt = C.c_longlong(0)
        self.ctx._chk(self.lib.fvc_tracer_snapshot(self.h, always, _d(out), C.byref(cnt)))
        return out[: cnt.value].copy()

    def stats(self):
        st = JobStats()
        self.ctx._chk(self.lib.fvc_job_get_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in JobStats._fields_}

    def get_state(self):
        n = self.n
        X, ldt = np.empty((n, 3)), np.empty(n)
        eid, left = np.empty(n, np.int32), np.empty(n, np.int32)
        self.ctx._chk(self.lib.fvc_tracer_get_state(self.h, _d(X), _i(eid), _i(left), _d(ldt)))
        return dict(X=X, eid=eid, left=left, ldt=ldt)

    def residence(self, launch_time, stop_time):
        rt = np.empty(max(self.n, 1))
        self.ctx._chk(self.lib.fvc_tracer_residence(self.h, launch_time, stop_time, _d(rt)))
        return rt[: self.n].copy()

    def close(self):
        if self.h:
            self.lib.fvc_job_destroy(self.h)
            self.h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Batched / served jobs on one context (fvc_batch_*): submit jobs, then
    run them all (run) or advance tick by tick (tick) while submitting more."""

    def __init__(self, ctx: Context, tmin, tdelta, tres, periodic=0, hbm_budget=0, max_jobs=0, resort_every=0,
                 tick_intervals=0):
        self.ctx, self.lib = ctx, ctx.lib
        self.h = _vp()
        self.sizes = {}
        o = BatchOpts(tmin, tdelta, tres, periodic, int(hbm_budget), max_jobs, resort_every, tick_intervals)
        ctx._chk(self.lib.fvc_batch_create(ctx.h, C.byref(o), C.byref(self.h)))

    def _submit(self, spec, keep=None):
        jid = C.c_int(0)
        self.ctx._chk(self.lib.fvc_batch_submit(self.h, C.byref(spec), C.byref(jid)))
        return jid.value

    def submit_tracers(self, seeds, t_start, t_stop, residence=False, lsc=1):
        seeds = f64(seeds)
        spec = BatchJobSpec(JOB_RESIDENCE if residence else JOB_TRACERS, t_start, t_stop, seeds.shape[0],
                            _d(seeds), lsc, FtleSpec())
        jid = self._submit(spec)
        self.sizes[jid] = seeds.shape[0]
        return jid

    def submit_ftle(self, grid, t_start, t_stop, lsc=1):
        g = FtleSpec(*grid[:6], *grid[6:9], lsc, t_start, t_stop, 1)
        spec = BatchJobSpec(JOB_FTLE, t_start, t_stop, 0, C.POINTER(C.c_double)(), lsc, g)
        jid = self._submit(spec)
        self.sizes[jid] = int(grid[6]) * int(grid[7]) * int(grid[8])
        return jid

    def tick(self):
        pend = C.c_int(0)
        self.ctx._chk(self.lib.fvc_batch_tick(self.h, C.byref(pend)))
        return pend.value

    def run(self, graph=False):
        self.ctx._chk(self.lib.fvc_batch_run(self.h, 1 if graph else 0))

    def autotune(self):
        self.ctx._chk(self.lib.fvc_batch_autotune(self.h))

    def poll(self, jid):
        st = C.c_int(0)
        self.ctx._chk(self.lib.fvc_batch_poll(self.h, jid, C.byref(st)))
        return st.value

    def tracer_result(self, jid):
        n = self.sizes[jid]
        X, ldt = np.empty((max(n, 1), 3)), np.empty(max(n, 1))
        eid, left = np.empty(max(n, 1), np.int32), np.empty(max(n, 1), np.int32)
        self.ctx._chk(self.lib.fvc_batch_tracer_result(self.h, jid, _d(X), _i(eid), _i(left), _d(ldt)))
        return dict(X=X[:n], eid=eid[:n], left=left[:n], ldt=ldt[:n])

    def residence_result(self, jid):
        n = self.sizes[jid]
        rt = np.empty(max(n, 1))
        self.ctx._chk(self.lib.fvc_batch_residence_result(self.h, jid, _d(rt)))
        return rt[:n]

    def ftle_result(self, jid):
        n = self.sizes[jid]
        wT, wN = np.empty(n), np.empty(n)
        self.ctx._chk(self.lib.fvc_batch_ftle_result(self.h, jid, _d(wT), _d(wN)))
        return wT, wN

    def result_begin(self, jid):
        """Queues a finished job's results into a page-locked block
        (fvc_batch_result_begin); returns the ticket."""
        t = C.c_longlong(0)
        self.ctx._chk(self.lib.fvc_batch_result_begin(self.h, jid, C.byref(t)))
        return t.value

    def result_ready(self, ticket):
        r = C.c_int(0)
        self.ctx._chk(self.lib.fvc_batch_result_ready(self.h, ticket, C.byref(r)))
        return bool(r.value)

    def result_get(self, ticket):
        """Waits for the ticket's results and returns them as numpy views of
        the library's block (valid until result_release): for tracer kinds
        X, eid, left, ldt, rt; for FTLE wT, wN."""
        r = BatchResult()
        self.ctx._chk(self.lib.fvc_batch_result_get(self.h, ticket, C.byref(r)))
        n = int(r.n)

        def view(p, shape, dt):
            return np.ctypeslib.as_array(p, shape=shape) if n else np.empty(shape, dt)
        if r.kind == JOB_FTLE:
            return {"wT": view(r.ftle_wT, (n,), np.float64), "wN": view(r.ftle_woT, (n,), np.float64)}
        return {"X": view(r.X, (n, 3), np.float64), "eid": view(r.eid, (n,), np.int32),
                "left": view(r.left, (n,), np.int32), "ldt": view(r.ldt, (n,), np.float64),
                "rt": view(r.rt, (n,), np.float64)}

    def result_release(self, ticket):
        self.ctx._chk(self.lib.fvc_batch_result_release(self.h, ticket))

    def job_stats(self, jid):
        st = JobStats()
        self.ctx._chk(self.lib.fvc_batch_job_stats(self.h, jid, C.byref(st)))
        return {k: getattr(st, k) for k, _ in JobStats._fields_}

    def release(self, jid):
        self.ctx._chk(self.lib.fvc_batch_release(self.h, jid))

    def stats(self):
        st = BatchStats()
        self.ctx._chk(self.lib.fvc_batch_get_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in BatchStats._fields_}

    def close(self):
        if self.h:
            self.lib.fvc_batch_destroy(self.h)
            self.h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
