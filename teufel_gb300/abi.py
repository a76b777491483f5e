"""ctypes binding of the C-ABI in include/teufel_cuda.h (libteufel_gb300.so).

The library is built in-tree (teufel_gb300/_lib) on first use.  There is no
CPU fallback: without the CUDA library or an sm_103 device the calls return
TEUFEL_ERR_NODEVICE and the Python wrappers raise.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import _build

TEUFEL_OK = 0
TEUFEL_ERR_ARG = 1
TEUFEL_ERR_NOMEM = 2
TEUFEL_ERR_CUDA = 3
TEUFEL_ERR_RANGE = 4
TEUFEL_ERR_TIMEOUT = 5
TEUFEL_ERR_NODEVICE = 6

E_CHARGE = 1.6021766208e-19  # src/global.h:36

PREC_FP32_SPLIT = 0
PREC_FP64 = 1
PREC_FP32_FP64TIME = 2

# The functions include/teufel_cuda.h declares (checked by the tests).
EXPORTED = [
    "teufel_cuda_default_options", "teufel_cuda_status_string", "teufel_cuda_traj_upload",
    "teufel_cuda_traj_free", "teufel_cuda_traj_points", "teufel_cuda_integrate_screen",
    "teufel_cuda_integrate_point", "teufel_cuda_integrate_screen_ex",
    "teufel_cuda_point_decisions", "teufel_cuda_deposit_injected", "teufel_cuda_last_inwindow",
    "teufel_cuda_probe_peaks", "teufel_cuda_last_timing", "teufel_cuda_integrate_screen_noalloc",
    "teufel_cuda_batch_create", "teufel_cuda_batch_run", "teufel_cuda_batch_status",
    "teufel_cuda_batch_free", "teufel_cuda_autotune", "teufel_cuda_retarded_field",
    "teufel_cuda_traj_track", "teufel_cuda_traj_download", "teufel_cuda_record_decisions",
    "teufel_cuda_batch_record_decisions", "teufel_cuda_check_fixed_division",
]

# bytes of the fixed device array used by teufel_cuda_integrate_screen_noalloc
NOALLOC_SCRATCH_BYTES = 64 * 1024 * 1024


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("device_pointers", ctypes.c_int),
                ("n_slots", ctypes.c_int), ("kernel_variant", ctypes.c_int),
                ("timing", ctypes.c_int), ("max_device_mib", ctypes.c_int),
                ("overwrite_out", ctypes.c_int)]


class ObserverDesc(ctypes.Structure):
    """teufel_observer: one observer of a batch (device pointers)."""
    _fields_ = [("traj", ctypes.c_void_p), ("pix_pos", ctypes.c_void_p),
                ("pix_t0", ctypes.c_void_p), ("dt", ctypes.c_double), ("Nt", ctypes.c_int),
                ("Np", ctypes.c_int), ("out", ctypes.c_void_p)]


class Lattice(ctypes.Structure):
    """teufel_lattice: a planar undulator and/or a homogeneous field."""
    _fields_ = [("has_undulator", ctypes.c_int), ("b_peak", ctypes.c_double),
                ("lambda_u", ctypes.c_double), ("n_periods", ctypes.c_int),
                ("origin", ctypes.c_double * 3), ("has_homogeneous", ctypes.c_int),
                ("E", ctypes.c_double * 3), ("B", ctypes.c_double * 3)]


def lattice(b_peak=0.0, lambda_u=1.0, n_periods=0, origin=(0.0, 0.0, 0.0), E=None, B=None):
    L = Lattice()
    L.has_undulator = 1 if n_periods > 0 else 0
    L.b_peak, L.lambda_u, L.n_periods = b_peak, lambda_u, n_periods
    L.origin[:] = list(origin)
    L.has_homogeneous = 1 if (E is not None or B is not None) else 0
    L.E[:] = list(E or (0.0, 0.0, 0.0))
    L.B[:] = list(B or (0.0, 0.0, 0.0))
    return L


class TeufelError(RuntimeError):
    """A non-zero status of the C-ABI.  TEUFEL_ERR_RANGE corresponds to the
    IOexception that FieldTrace::add throws (src/fieldtrace.cpp:185-190)."""

    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = status_string(status)
        super().__init__(f"{what}: {msg} (status {status})" if what else msg)


_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = _build.build_cuda()
        if not os.path.exists(path):
            raise RuntimeError(f"CUDA library missing: {path}")
        L = ctypes.CDLL(str(path))
        L.teufel_cuda_default_options.restype = None
        L.teufel_cuda_default_options.argtypes = [ctypes.POINTER(Options)]
        L.teufel_cuda_status_string.restype = ctypes.c_char_p
        L.teufel_cuda_status_string.argtypes = [ctypes.c_int]
        L.teufel_cuda_traj_upload.restype = ctypes.c_int
        L.teufel_cuda_traj_upload.argtypes = [ctypes.c_int, _ip, _dp, _dp, _dp, _dp, _dp,
                                              ctypes.POINTER(_vp)]
        L.teufel_cuda_traj_free.restype = ctypes.c_int
        L.teufel_cuda_traj_free.argtypes = [_vp]
        L.teufel_cuda_traj_points.restype = ctypes.c_int64
        L.teufel_cuda_traj_points.argtypes = [_vp]
        L.teufel_cuda_integrate_screen.restype = ctypes.c_int
        L.teufel_cuda_integrate_screen.argtypes = [_vp, _vp, _vp, ctypes.c_double, ctypes.c_int,
                                                   ctypes.c_int, _vp, _vp]
        L.teufel_cuda_integrate_point.restype = ctypes.c_int
        L.teufel_cuda_integrate_point.argtypes = [_vp, _dp, ctypes.c_double, ctypes.c_double,
                                                  ctypes.c_int, _dp, _vp]
        L.teufel_cuda_integrate_screen_ex.restype = ctypes.c_int
        L.teufel_cuda_integrate_screen_ex.argtypes = [_vp, _vp, _vp, ctypes.c_double,
                                                      ctypes.c_int, ctypes.c_int, _vp,
                                                      ctypes.POINTER(Options), _vp]
        L.teufel_cuda_point_decisions.restype = ctypes.c_int
        L.teufel_cuda_point_decisions.argtypes = [_vp, ctypes.c_int, _dp, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_int, _lp, _ip, _dp,
                                                  ctypes.POINTER(ctypes.c_float)]
        L.teufel_cuda_deposit_injected.restype = ctypes.c_int
        L.teufel_cuda_deposit_injected.argtypes = [ctypes.c_int, _ip, _dp, _dp, ctypes.c_double,
                                                   ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                                   _dp]
        L.teufel_cuda_last_inwindow.restype = ctypes.c_int
        L.teufel_cuda_last_inwindow.argtypes = [_vp, _lp, _lp]
        L.teufel_cuda_last_timing.restype = ctypes.c_int
        L.teufel_cuda_last_timing.argtypes = [_vp, _lp, _lp, _ip, _dp, _dp]
        L.teufel_cuda_integrate_screen_noalloc.restype = ctypes.c_int
        L.teufel_cuda_integrate_screen_noalloc.argtypes = [_vp, _vp, _vp, ctypes.c_double,
                                                           ctypes.c_int, ctypes.c_int, _vp, _vp]
        L.teufel_cuda_probe_peaks.restype = ctypes.c_int
        L.teufel_cuda_probe_peaks.argtypes = [_dp, _dp, _dp]
        L.teufel_cuda_check_fixed_division.restype = ctypes.c_int
        L.teufel_cuda_check_fixed_division.argtypes = [
            ctypes.c_int, _dp, ctypes.c_double, _dp, ctypes.c_double, ctypes.c_double,
            ctypes.c_int, _dp, ctypes.POINTER(ctypes.c_int32)]
        L.teufel_cuda_batch_create.restype = ctypes.c_int
        L.teufel_cuda_batch_create.argtypes = [ctypes.c_int, ctypes.POINTER(ObserverDesc),
                                               ctypes.POINTER(Options),
                                               ctypes.POINTER(ctypes.c_void_p)]
        L.teufel_cuda_batch_run.restype = ctypes.c_int
        L.teufel_cuda_batch_run.argtypes = [_vp, _vp]
        L.teufel_cuda_batch_status.restype = ctypes.c_int
        L.teufel_cuda_batch_status.argtypes = [_vp, _lp, _lp, _dp]
        L.teufel_cuda_traj_track.restype = ctypes.c_int
        L.teufel_cuda_traj_track.argtypes = [ctypes.c_int, _dp, _dp, _dp,
                                             ctypes.POINTER(Lattice), ctypes.c_double,
                                             ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        L.teufel_cuda_traj_download.restype = ctypes.c_int
        L.teufel_cuda_traj_download.argtypes = [_vp, _dp, _dp, _dp, _dp]
        L.teufel_cuda_retarded_field.restype = ctypes.c_int
        L.teufel_cuda_retarded_field.argtypes = [_vp, ctypes.c_double, ctypes.c_int, _dp, _dp,
                                                 _vp]
        L.teufel_cuda_autotune.restype = ctypes.c_int
        L.teufel_cuda_autotune.argtypes = [_vp, _vp, _vp, ctypes.c_double, ctypes.c_int,
                                           ctypes.c_int, ctypes.POINTER(Options),
                                           ctypes.POINTER(Options), _dp]
        L.teufel_cuda_batch_free.restype = ctypes.c_int
        L.teufel_cuda_batch_free.argtypes = [_vp]
        _i32p = ctypes.POINTER(ctypes.c_int32)
        L.teufel_cuda_record_decisions.restype = ctypes.c_int
        L.teufel_cuda_record_decisions.argtypes = [_vp, _dp, _dp, ctypes.c_double, ctypes.c_int,
                                                   ctypes.c_int, ctypes.POINTER(Options), _i32p,
                                                   _dp]
        L.teufel_cuda_batch_record_decisions.restype = ctypes.c_int
        L.teufel_cuda_batch_record_decisions.argtypes = [_vp, ctypes.c_int, _i32p]
        _lib = L
    return _lib


def status_string(status: int) -> str:
    return lib().teufel_cuda_status_string(status).decode()


def check(status: int, what: str = "") -> None:
    if status != TEUFEL_OK:
        raise TeufelError(status, what)


def _c(a, dtype=np.float64):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


def options(precision: int = PREC_FP32_SPLIT, device_pointers: bool = False,
            n_slots: int = 0, timing: bool = False, variant: int = 0,
            max_device_mib: int = 0, overwrite_out: bool = False) -> Options:
    o = Options()
    lib().teufel_cuda_default_options(ctypes.byref(o))
    o.precision = precision
    o.device_pointers = 1 if device_pointers else 0
    o.n_slots = n_slots
    o.timing = 1 if timing else 0
    o.kernel_variant = variant
    o.max_device_mib = max_device_mib
    o.overwrite_out = 1 if overwrite_out else 0
    return o


class TrajSet:
    """A device-resident particle set (teufel_cuda_traj_upload)."""

    def __init__(self, traj):
        L = lib()
        n = traj.n_particles
        npnt = _c(traj.n_points, np.int32)
        # charge in Coulomb, formed as the reference forms Charge*ElementaryCharge
        ch = _c(np.asarray(traj.charge, dtype=np.float64) * E_CHARGE)
        t, x, p, a = _c(traj.t), _c(traj.x), _c(traj.p), _c(traj.a)
        h = _vp()
        check(L.teufel_cuda_traj_upload(n, _ptr(npnt, _ip), _ptr(ch), _ptr(t), _ptr(x), _ptr(p),
                                        _ptr(a), ctypes.byref(h)), "teufel_cuda_traj_upload")
        self.handle = h
        self.n_particles = n
        self.n_points = npnt.copy()

    @classmethod
    def from_arrays(cls, n_points, charge, t, x, p, a):
        """Upload from host arrays (possibly pinned); charge in units of e."""
        class _T:
            pass
        tr = _T()
        tr.n_particles = len(n_points)
        tr.n_points, tr.charge, tr.t, tr.x, tr.p, tr.a = n_points, charge, t, x, p, a
        return cls(tr)

    @classmethod
    def track(cls, init, charge_e, mass, lat, tstep, n_steps):
        """teufel_cuda_traj_track: particles tracked on the device by the Vay
        pusher through `lat` (abi.lattice(...)); init[n][7] = t, x, y, z,
        beta*gamma; charge in units of e, mass in electron masses (arrays or
        scalars)."""
        init = _c(init).reshape(-1, 7)
        n = init.shape[0]
        ch = _c(np.broadcast_to(np.asarray(charge_e, dtype=np.float64), (n,)))
        ms = _c(np.broadcast_to(np.asarray(mass, dtype=np.float64), (n,)))
        h = _vp()
        check(lib().teufel_cuda_traj_track(n, _ptr(init), _ptr(ch), _ptr(ms), ctypes.byref(lat),
                                           tstep, n_steps, ctypes.byref(h)),
              "teufel_cuda_traj_track")
        obj = cls.__new__(cls)
        obj.handle = h
        obj.n_particles = n
        obj.n_points = np.full(n, n_steps + 1, dtype=np.int32)
        return obj

    def download(self):
        """(t, x, bg, a) of the set's trajectories (teufel_cuda_traj_download)."""
        N = int(np.sum(self.n_points))
        t, x, p, a = np.empty(N), np.empty((N, 3)), np.empty((N, 3)), np.empty((N, 3))
        check(lib().teufel_cuda_traj_download(self.handle, _ptr(t), _ptr(x), _ptr(p), _ptr(a)),
              "teufel_cuda_traj_download")
        return t, x, p, a

    def free(self):
        if self.handle:
            lib().teufel_cuda_traj_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()

    def points(self) -> int:
        return int(lib().teufel_cuda_traj_points(self.handle))

    # -- integration ----------------------------------------------------
    def integrate_screen(self, pix_pos, pix_t0, dt, nots, out=None,
                         precision: int = PREC_FP32_SPLIT, n_slots: int = 0,
                         stream: int = 0, variant: int = 0,
                         max_device_mib: int = 0, overwrite_out: bool = False) -> np.ndarray:
        """Traces of all particles on the pixels, added into ``out``
        ([Np][nots][6] doubles, zeros if None) -- host buffers.  With
        ``overwrite_out`` they are stored into ``out`` instead (its contents
        neither read nor uploaded)."""
        pix_pos = _c(pix_pos).reshape(-1, 3)
        pix_t0 = _c(pix_t0).reshape(-1)
        n_pix = pix_pos.shape[0]
        if out is None:
            # zeros, not an unwritten buffer: copying the traces back into
            # pages the process has never touched runs at a few GB/s
            out = np.zeros((n_pix, nots, 6))
        if not (out.dtype == np.float64 and out.flags.c_contiguous):
            raise ValueError("out must be a C-contiguous float64 array")
        opt = options(precision, False, n_slots, variant=variant, max_device_mib=max_device_mib,
                      overwrite_out=overwrite_out)
        check(lib().teufel_cuda_integrate_screen_ex(self.handle, pix_pos.ctypes.data,
                                                    pix_t0.ctypes.data, dt, nots, n_pix,
                                                    out.ctypes.data, ctypes.byref(opt),
                                                    _vp(stream)),
              "teufel_cuda_integrate_screen")
        return out

    def integrate_screen_device(self, pos_ptr: int, t0_ptr: int, dt: float, nots: int,
                                n_pix: int, out_ptr: int, precision: int = PREC_FP32_SPLIT,
                                n_slots: int = 0, stream: int = 0, timing: bool = False,
                                variant: int = 0, overwrite_out: bool = False) -> None:
        """Device-pointer variant; returns once the work is enqueued."""
        opt = options(precision, True, n_slots, timing, variant, overwrite_out=overwrite_out)
        check(lib().teufel_cuda_integrate_screen_ex(self.handle, _vp(pos_ptr), _vp(t0_ptr), dt,
                                                    nots, n_pix, _vp(out_ptr),
                                                    ctypes.byref(opt), _vp(stream)),
              "teufel_cuda_integrate_screen_ex")

    def integrate_point(self, pos, t0, dt, nots, out=None) -> np.ndarray:
        pos = _c(pos).reshape(3)
        if out is None:
            out = np.zeros((nots, 6))
        check(lib().teufel_cuda_integrate_point(self.handle, _ptr(pos), t0, dt, nots, _ptr(out),
                                                None), "teufel_cuda_integrate_point")
        return out

    def last_inwindow(self):
        iw = ctypes.c_int64(0)
        fb = ctypes.c_int64(0)
        st = lib().teufel_cuda_last_inwindow(self.handle, ctypes.byref(iw), ctypes.byref(fb))
        return int(iw.value), int(fb.value), st

    def last_timing(self):
        """(deposits, point evaluations, kernel launches, integration-kernel
        ms, reduction ms) of the last call; the times need timing=True on
        that call."""
        dep = ctypes.c_int64(0)
        nev = ctypes.c_int64(0)
        nl = ctypes.c_int(0)
        k = ctypes.c_double(0)
        r = ctypes.c_double(0)
        check(lib().teufel_cuda_last_timing(self.handle, ctypes.byref(dep), ctypes.byref(nev),
                                            ctypes.byref(nl), ctypes.byref(k), ctypes.byref(r)),
              "teufel_cuda_last_timing")
        return int(dep.value), int(nev.value), int(nl.value), float(k.value), float(r.value)

    def retarded_field(self, obs_time, pos):
        """teufel_cuda_retarded_field: the summed field [n, 6] at obs_time on
        the points pos[n, 3] (the SnapshotObserver computation)."""
        pos = _c(pos).reshape(-1, 3)
        out = np.empty((pos.shape[0], 6))
        check(lib().teufel_cuda_retarded_field(self.handle, obs_time, pos.shape[0], _ptr(pos),
                                               _ptr(out), None), "teufel_cuda_retarded_field")
        return out

    def autotune(self, pix_pos, pix_t0, dt, nots, n_pix=None, device=False):
        """teufel_cuda_autotune: (kernel_variant, n_slots, ms) of the fastest
        FP32 configuration for this observer; later automatic calls on a
        similar shape use it.  With device=True pix_pos/pix_t0 are device
        pointers (ints) and n_pix must be given."""
        opt = options(PREC_FP32_SPLIT, device)
        best = Options()
        ms = ctypes.c_double(0)
        if device:
            args = (ctypes.c_void_p(pix_pos), ctypes.c_void_p(pix_t0), dt, nots, int(n_pix))
        else:
            pos = _c(pix_pos).reshape(-1, 3)
            t0 = _c(pix_t0).reshape(-1)
            args = (pos.ctypes.data_as(ctypes.c_void_p), t0.ctypes.data_as(ctypes.c_void_p), dt,
                    nots, pos.shape[0])
        check(lib().teufel_cuda_autotune(self.handle, *args, ctypes.byref(opt), ctypes.byref(best),
                                         ctypes.byref(ms)), "teufel_cuda_autotune")
        return int(best.kernel_variant), int(best.n_slots), float(ms.value)

    def record_decisions(self, pix_pos, pix_t0, dt, nots, variant: int = 4, n_slots: int = 0):
        """teufel_cuda_record_decisions: (traces [Np][nots][6], decision record
        [Np][n_particles][max points] int32) of the recording instantiation
        of the shipping pair kernel (variant 4 or 8)."""
        pix_pos = _c(pix_pos).reshape(-1, 3)
        pix_t0 = _c(pix_t0).reshape(-1)
        n_pix = pix_pos.shape[0]
        out = np.zeros((n_pix, nots, 6))
        stride = int(np.max(self.n_points)) if self.n_particles else 0
        rec = np.zeros((n_pix, self.n_particles, stride), dtype=np.int32)
        opt = options(PREC_FP32_SPLIT, False, n_slots, variant=variant)
        check(lib().teufel_cuda_record_decisions(self.handle, _ptr(pix_pos), _ptr(pix_t0), dt,
                                                 nots, n_pix, ctypes.byref(opt),
                                                 _ptr(rec, ctypes.POINTER(ctypes.c_int32)),
                                                 _ptr(out)),
              "teufel_cuda_record_decisions")
        return out, rec

    def point_decisions(self, m, pos, t0, dt, nots):
        n = int(self.n_points[m])
        idx = np.zeros(n, dtype=np.int64)
        flags = np.zeros(n, dtype=np.int32)
        u = np.zeros(n)
        band = np.zeros(n, dtype=np.float32)
        pos = _c(pos).reshape(3)
        check(lib().teufel_cuda_point_decisions(self.handle, m, _ptr(pos), t0, dt, nots,
                                                _ptr(idx, _lp), _ptr(flags, _ip), _ptr(u),
                                                _ptr(band, ctypes.POINTER(ctypes.c_float))),
              "teufel_cuda_point_decisions")
        self.last_band = band
        return idx, flags, u


def deposit_injected(ts_list, f_list, t0, dt, nots, precision=PREC_FP64, trace=None):
    """Device deposit of injected (arrival time, field) sequences."""
    n_points = np.array([len(v) for v in ts_list], dtype=np.int32)
    ts = _c(np.concatenate([np.asarray(v, dtype=np.float64) for v in ts_list]) if ts_list
            else np.zeros(0))
    f = _c(np.concatenate([np.asarray(v, dtype=np.float64).reshape(-1, 6) for v in f_list])
           if f_list else np.zeros((0, 6)))
    if trace is None:
        trace = np.zeros((nots, 6))
    st = lib().teufel_cuda_deposit_injected(len(ts_list), _ptr(n_points, _ip), _ptr(ts), _ptr(f),
                                            t0, dt, nots, precision, _ptr(trace))
    return trace, st


def check_fixed_division(a, b, ts, t0, dt, nt):
    """teufel_cuda_check_fixed_division: (quotients [n][2], bins [n][2]) --
    the FP64-time mode's a/b and bin of ts, and the IEEE ones."""
    a = _c(a).reshape(-1)
    ts = _c(ts).reshape(-1)
    assert a.shape == ts.shape
    n = a.shape[0]
    q = np.zeros((n, 2))
    k = np.zeros((n, 2), dtype=np.int32)
    check(lib().teufel_cuda_check_fixed_division(n, _ptr(a), b, _ptr(ts), t0, dt, nt, _ptr(q),
                                                 _ptr(k, ctypes.POINTER(ctypes.c_int32))),
          "teufel_cuda_check_fixed_division")
    return q, k


def probe_peaks():
    """(FFMA, packed FFMA2, DFMA) throughput of the current device in TFLOP/s."""
    a = ctypes.c_double(0)
    b = ctypes.c_double(0)
    c = ctypes.c_double(0)
    check(lib().teufel_cuda_probe_peaks(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
          "probe_peaks")
    return a.value, b.value, c.value


class Batch:
    """A planned batch of observers (teufel_cuda_batch_create): one persistent
    launch over a device work queue plus one reduction, replayed as a CUDA
    graph.  observers: (TrajSet, pix_pos, pix_t0, dt, Nt, Np, out) with device
    pointers (ints) for pix_pos, pix_t0 and out."""

    def __init__(self, observers, n_slots: int = 0):
        self._keep = [o[0] for o in observers]
        arr = (ObserverDesc * max(1, len(observers)))()
        for k, (ts, pos, t0, dt, nt, npix, out) in enumerate(observers):
            arr[k] = ObserverDesc(ts.handle, pos, t0, dt, nt, npix, out)
        opt = options(PREC_FP32_SPLIT, True, n_slots)
        h = ctypes.c_void_p()
        check(lib().teufel_cuda_batch_create(len(observers), arr, ctypes.byref(opt),
                                             ctypes.byref(h)), "teufel_cuda_batch_create")
        self.handle = h

    def run(self, stream: int = 0) -> None:
        check(lib().teufel_cuda_batch_run(self.handle, stream), "teufel_cuda_batch_run")

    def status(self):
        """(status, work items, in-window steps, integration-kernel ms) of the
        last run; synchronizes with it."""
        items = ctypes.c_int64(0)
        inw = ctypes.c_int64(0)
        ms = ctypes.c_double(0)
        st = lib().teufel_cuda_batch_status(self.handle, ctypes.byref(items), ctypes.byref(inw),
                                            ctypes.byref(ms))
        return st, int(items.value), int(inw.value), float(ms.value)

    def record_decisions(self, obs: int, n_pix: int, traj_set) -> np.ndarray:
        """teufel_cuda_batch_record_decisions: one run of the batch in which
        observer `obs` (n_pix pixels, trajectory set traj_set) records its
        decisions, [n_pix][n_particles][max points] int32."""
        stride = int(np.max(traj_set.n_points)) if traj_set.n_particles else 0
        rec = np.zeros((n_pix, traj_set.n_particles, stride), dtype=np.int32)
        check(lib().teufel_cuda_batch_record_decisions(self.handle, obs,
                                                       _ptr(rec, ctypes.POINTER(ctypes.c_int32))),
              "teufel_cuda_batch_record_decisions")
        return rec

    def close(self) -> None:
        if self.handle:
            lib().teufel_cuda_batch_free(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
