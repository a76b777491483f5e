"""ctypes bindings of the CPU oracle (oracle/liblw_oracle.so) and of the
reference's own compiled code (oracle/_ref/libteufel_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.  See the header of
oracle/lw_oracle.c for what the restatement follows, file by line.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "liblw_oracle.so"
REF_SO = HERE / "_ref" / "libteufel_ref.so"

_dp = ctypes.POINTER(ctypes.c_double)
_lp = ctypes.POINTER(ctypes.c_int64)
_bp = ctypes.POINTER(ctypes.c_int8)
_i64 = ctypes.c_int64

_oracle = None
_ref = None


_ref_src_cache: list = []


def reference_src():
    """The reference's source directory, as oracle/Makefile finds it
    (TEUFEL_REFERENCE_SRC, else the recipe's default location), or None when
    the tree is absent (on the GPU machine it always is)."""
    if not _ref_src_cache:
        r = subprocess.run(["make", "-s", "-C", str(HERE), "refdir"], stdout=subprocess.PIPE,
                           stderr=subprocess.DEVNULL, text=True)
        d = r.stdout.strip() if r.returncode == 0 else ""
        _ref_src_cache.append(Path(d) if d else None)
    return _ref_src_cache[0]


def build(with_reference: bool = True) -> None:
    """make -C oracle (and the reference build where its sources exist)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    src = reference_src() if with_reference else None
    if src is not None:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={src}"], check=True)


def reference_available() -> bool:
    return REF_SO.exists()


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def oracle():
    global _oracle
    if _oracle is None:
        if not ORACLE_SO.exists():
            build(with_reference=False)
        L = ctypes.CDLL(str(ORACLE_SO))
        L.lwo_retarded_time.restype = ctypes.c_double
        L.lwo_retarded_time.argtypes = [ctypes.c_double, _dp, _dp]
        L.lwo_retarded_field.restype = None
        L.lwo_retarded_field.argtypes = [_dp, _dp, _dp, ctypes.c_double, _dp, _dp]
        L.lwo_integrate_screen.restype = ctypes.c_int
        L.lwo_integrate_screen.argtypes = [_i64, _lp, _dp, _dp, _dp, _dp, _dp, _i64, _dp, _dp,
                                           ctypes.c_double, _i64, _dp, ctypes.c_int, _lp]
        L.lwo_integrate_screen_ext.restype = ctypes.c_int
        L.lwo_integrate_screen_ext.argtypes = [_i64, _lp, _dp, _dp, _dp, _dp, _dp, _i64, _dp,
                                               _dp, ctypes.c_double, _i64, _dp, ctypes.c_int]
        L.lwo_deposit_injected.restype = ctypes.c_int
        L.lwo_deposit_injected.argtypes = [_i64, _lp, _dp, _dp, ctypes.c_double,
                                           ctypes.c_double, _i64, _dp]
        L.lwo_point_decisions.restype = None
        L.lwo_point_decisions.argtypes = [_i64, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double,
                                          _i64, _lp, ctypes.POINTER(ctypes.c_int32)]
        L.lwo_retarded_field_at.restype = ctypes.c_int
        L.lwo_retarded_field_at.argtypes = [_i64, _lp, _dp, _dp, _dp, _dp, _dp, ctypes.c_double,
                                            _i64, _dp, _dp, ctypes.c_int]
        L.lwo_screen_decisions.restype = None
        L.lwo_screen_decisions.argtypes = [_i64, _lp, _dp, _dp, _i64, _dp, _dp, ctypes.c_double,
                                           _i64, _i64, ctypes.POINTER(ctypes.c_int32)]
        L.lwo_step_decisions.restype = None
        L.lwo_step_decisions.argtypes = [_i64, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double,
                                         _i64, _lp, _lp, _bp]
        _oracle = L
    return _oracle


def reference():
    global _ref
    if _ref is None:
        if not REF_SO.exists():
            raise FileNotFoundError("the reference build oracle/_ref is absent")
        L = ctypes.CDLL(str(REF_SO))
        L.ref_track.restype = ctypes.c_int
        L.ref_track.argtypes = [_i64, _dp, ctypes.c_double, ctypes.c_double, _dp,
                                ctypes.c_double, _i64, _dp, _dp, _dp, _dp]
        L.ref_integrate_screen.restype = ctypes.c_int
        L.ref_integrate_screen.argtypes = [_i64, _lp, _dp, _dp, _dp, _dp, _dp, _dp, _i64, _dp,
                                           _dp, ctypes.c_double, _i64, _dp, ctypes.c_int]
        L.ref_retarded_field_at.restype = ctypes.c_int
        L.ref_retarded_field_at.argtypes = [_i64, _lp, _dp, _dp, _dp, _dp, _dp, _dp,
                                            ctypes.c_double, _i64, _dp, _dp]
        L.ref_deposit_injected.restype = ctypes.c_int
        L.ref_deposit_injected.argtypes = [_i64, _lp, _dp, _dp, ctypes.c_double,
                                           ctypes.c_double, _i64, _dp]
        L.ref_coordinates_at_time.restype = ctypes.c_int
        L.ref_coordinates_at_time.argtypes = [_i64, _lp, _dp, _dp, _dp, ctypes.c_double, _dp]
        _ref = L
    return _ref


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def integrate_screen(traj, pix_pos, pix_t0, dt, nots, out=None, nthreads=0, impl="oracle"):
    """Traces [n_pix, nots, 6] of a particle set (harness.Trajectories) on the
    given pixels, added into ``out`` (zeros if None).  impl: "oracle" (the C
    restatement) or "reference" (the reference's compiled particle.cpp)."""
    pix_pos = _c(pix_pos)
    pix_t0 = _c(pix_t0)
    n_pix = pix_pos.shape[0]
    if out is None:
        out = np.zeros((n_pix, nots, 6))
    assert out.dtype == np.float64 and out.flags.c_contiguous and out.shape == (n_pix, nots, 6)
    offs = _c(traj.offsets, np.int64)
    t, x, p, a = _c(traj.t), _c(traj.x), _c(traj.p), _c(traj.a)
    ch = _c(traj.charge)
    if impl == "extended":
        rc = oracle().lwo_integrate_screen_ext(traj.n_particles, _p(offs, _lp), _p(ch), _p(t),
                                               _p(x), _p(p), _p(a), n_pix, _p(pix_pos),
                                               _p(pix_t0), dt, nots, _p(out), nthreads)
    elif impl == "oracle":
        touched = ctypes.c_int64(0)
        rc = oracle().lwo_integrate_screen(traj.n_particles, _p(offs, _lp), _p(ch), _p(t), _p(x),
                                           _p(p), _p(a), n_pix, _p(pix_pos), _p(pix_t0), dt,
                                           nots, _p(out), nthreads, ctypes.byref(touched))
    else:
        ms = _c(traj.mass)
        rc = reference().ref_integrate_screen(traj.n_particles, _p(offs, _lp), _p(ch), _p(ms),
                                              _p(t), _p(x), _p(p), _p(a), n_pix, _p(pix_pos),
                                              _p(pix_t0), dt, nots, _p(out), nthreads)
    return out, rc


def deposit_injected(ts_list, f_list, t0, dt, nots, impl="oracle"):
    """Deposit injected (arrival time, field) sequences, one per particle."""
    n_points = np.array([len(ts) for ts in ts_list], dtype=np.int64)
    offs = np.zeros(len(ts_list) + 1, dtype=np.int64)
    np.cumsum(n_points, out=offs[1:])
    ts = _c(np.concatenate([np.asarray(v, dtype=np.float64) for v in ts_list]))
    f = _c(np.concatenate([np.asarray(v, dtype=np.float64).reshape(-1, 6) for v in f_list]))
    trace = np.zeros((nots, 6))
    fn = oracle().lwo_deposit_injected if impl == "oracle" else reference().ref_deposit_injected
    rc = fn(len(ts_list), _p(offs, _lp), _p(ts), _p(f), t0, dt, nots, _p(trace))
    return trace, rc


def retarded_field_at(traj, obs_time, pos, nthreads=0, impl="oracle"):
    """The summed field [n_obs, 6] of a particle set at time obs_time on the
    observation points pos[n_obs, 3] (ChargedParticle::RetardedField(double,
    Vector) per particle, summed as Bunch::RetardedField).  impl: "oracle" or
    "reference"."""
    pos = _c(pos).reshape(-1, 3)
    n = pos.shape[0]
    out = np.zeros((n, 6))
    offs = _c(traj.offsets, np.int64)
    t, x, p, a = _c(traj.t), _c(traj.x), _c(traj.p), _c(traj.a)
    ch = _c(traj.charge)
    if impl == "oracle":
        rc = oracle().lwo_retarded_field_at(traj.n_particles, _p(offs, _lp), _p(ch), _p(t), _p(x),
                                            _p(p), _p(a), ctypes.c_double(obs_time), n, _p(pos),
                                            _p(out), nthreads)
    else:
        ms = _c(traj.mass)
        rc = reference().ref_retarded_field_at(traj.n_particles, _p(offs, _lp), _p(ch), _p(ms),
                                               _p(t), _p(x), _p(p), _p(a),
                                               ctypes.c_double(obs_time), n, _p(pos), _p(out))
    return out, rc


def point_decisions(traj, m, obs, t0, dt, nots):
    """Per point of particle m: (bin index clamped to [-2, nots+1], flags with
    bit0 = ts <= tmin, bit1 = ts < tmax) in the reference's arithmetic."""
    o = traj.offsets
    t = _c(traj.t[o[m]:o[m + 1]])
    x = _c(traj.x[o[m]:o[m + 1]])
    n = t.shape[0]
    idx = np.zeros(n, dtype=np.int64)
    fl = np.zeros(n, dtype=np.int32)
    oracle().lwo_point_decisions(n, _p(t), _p(x), _p(_c(obs)), t0, dt, nots, _p(idx, _lp),
                                 _p(fl, ctypes.POINTER(ctypes.c_int32)))
    return idx, fl


def screen_decisions(traj, pix_pos, pix_t0, dt, nots):
    """The reference's decision of every (pixel, particle, point) of a screen,
    [n_pix, n_particles, max_points] int32 encoded as the device's decision
    record: (bin index + 4) | (flags << 27), flags bit0 = ts <= tmin,
    bit1 = ts < tmax; 0 beyond a particle's last point."""
    pix_pos = _c(pix_pos)
    pix_t0 = _c(pix_t0)
    n_pix = pix_pos.shape[0]
    stride = int(np.max(traj.n_points)) if traj.n_particles else 0
    rec = np.zeros((n_pix, traj.n_particles, stride), dtype=np.int32)
    offs = _c(traj.offsets, np.int64)
    oracle().lwo_screen_decisions(traj.n_particles, _p(offs, _lp), _p(_c(traj.t)),
                                  _p(_c(traj.x)), n_pix, _p(pix_pos), _p(pix_t0), dt, nots,
                                  stride, _p(rec, ctypes.POINTER(ctypes.c_int32)))
    return rec


def step_decisions(traj, m, obs, t0, dt, nots):
    """Per step of particle m: (round((ts1-t0)/dt), round((ts2-t0)/dt), case)
    with case 0 = outside the window, 1 = starts before it, 2 = inside."""
    o = traj.offsets
    t = _c(traj.t[o[m]:o[m + 1]])
    x = _c(traj.x[o[m]:o[m + 1]])
    n = t.shape[0]
    i1 = np.zeros(max(n - 1, 0), dtype=np.int64)
    i2 = np.zeros_like(i1)
    k = np.zeros(max(n - 1, 0), dtype=np.int8)
    ob = _c(obs)
    oracle().lwo_step_decisions(n, _p(t), _p(x), _p(ob), t0, dt, nots, _p(i1, _lp), _p(i2, _lp),
                                _p(k, _bp))
    return i1, i2, k


def track_reference(init, lattice_packed, tstep, n_steps, charge, mass):
    init = _c(init)
    n = init.shape[0]
    npnt = n_steps + 1
    t = np.empty(n * npnt)
    x = np.empty((n * npnt, 3))
    p = np.empty((n * npnt, 3))
    a = np.empty((n * npnt, 3))
    rc = reference().ref_track(n, _p(init), charge, mass, _p(_c(lattice_packed)), tstep,
                               n_steps, _p(t), _p(x), _p(p), _p(a))
    if rc != 0:
        raise RuntimeError(f"ref_track failed: {rc}")
    return t, x, p, a


def reference_file(rel: str):
    """Path of a file of the reference tree (rel to its root), or None where
    the tree is absent.  The tree is found beside its src/ directory."""
    src = reference_src()
    if src is None:
        return None
    f = src.parent / rel
    return f if f.exists() else None


MU_NULL = 4.0 * np.pi * 1e-7  # src/global.h:43


def mesh_cells(corner, tri):
    """Cell areas and unit normals of a triangle mesh, as MeshedScreen::init
    computes them (src/mesh.cpp:227-247): n = (p3-p1) x (p2-p1)."""
    p1, p2, p3 = corner[tri[:, 0]], corner[tri[:, 1]], corner[tri[:, 2]]
    n = np.cross(p3 - p1, p2 - p1)
    norm = np.linalg.norm(n, axis=1)
    return 0.5 * norm, n / norm[:, None]


def mesh_energy(corner, tri, traces, dt):
    """(total, per-cell) energy through a meshed screen [J]: minus the cell
    area times the time-integrated Poynting vector along the normal
    (MeshedScreen::totalEnergy, src/mesh.cpp:744-754, with
    FieldTrace::Poynting, src/fieldtrace.cpp:192-198)."""
    area, normal = mesh_cells(corner, tri)
    s = np.cross(traces[:, :, 0:3], traces[:, :, 3:6]).sum(axis=1) / MU_NULL * dt
    flux = -area * np.einsum("ij,ij->i", s, normal)
    return float(flux.sum()), flux


def coordinates_at_time(traj, time):
    """[n_particles][6] position and beta*gamma of every particle at ``time``
    from the reference's ChargedParticle::CoordinatesAtTime."""
    out = np.zeros((traj.n_particles, 6))
    reference().ref_coordinates_at_time(traj.n_particles, _p(_c(traj.offsets, np.int64), _lp),
                                        _p(_c(traj.t)), _p(_c(traj.x)), _p(_c(traj.p)), time,
                                        _p(out))
    return out
