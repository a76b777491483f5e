"""Synthetic, seeded workloads for the field integration.

The reference's field integration consumes tracked trajectories and an
observer geometry.  This module builds both for the five benchmark workloads
(single electron, 1e4-particle bunch, batched uneven screens, 1e5-particle
coherent-emission screen, gamma=2000 precision stress) through the native
trajectory source in ``csrc/trajgen.cpp`` (a restatement of the reference's
Vay pusher and planar undulator, src/particle.cpp:407-512 and
src/undulator.cpp:107-125).

Screen geometry follows ScreenObserver (src/screen.cpp:97-110): the pixel
(ix, iy) sits at ``Origin + dX*(ix - Nx//2) + dY*(iy - Ny//2)`` and its trace
starts at ``t0 + dtx*(ix - Nx//2) + dty*(iy - Ny//2)``; pixels are ordered ix
major, iy minor, which is the order of ScreenObserver::getBuffer
(src/screen.cpp:249-272).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _build

E_CHARGE = 1.6021766208e-19  # src/global.h:36
C_LIGHT = 2.99792458e8       # src/global.h:38

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_harness()
        L = ctypes.CDLL(str(path))
        dp = ctypes.POINTER(ctypes.c_double)
        L.tg_undulator_b0.restype = ctypes.c_double
        L.tg_undulator_b0.argtypes = [ctypes.c_double, ctypes.c_double]
        L.tg_track.restype = ctypes.c_int
        L.tg_track.argtypes = [ctypes.c_int64, dp, ctypes.c_double, ctypes.c_double, dp,
                               ctypes.c_double, ctypes.c_int64, dp, dp, dp, dp, ctypes.c_int]
        L.tg_gaussian_bunch.restype = None
        L.tg_gaussian_bunch.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_uint64,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, dp]
        L.tg_uniform.restype = None
        L.tg_uniform.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_double,
                                 ctypes.c_double, dp]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


# --------------------------------------------------------------------------
# trajectories
# --------------------------------------------------------------------------
@dataclass
class Lattice:
    """A planar undulator centred on ``origin`` and/or a homogeneous field."""
    b_peak: float = 0.0
    lambda_u: float = 1.0
    n_periods: int = 0
    origin: tuple = (0.0, 0.0, 0.0)
    hom_e: Optional[tuple] = None
    hom_b: Optional[tuple] = None

    def packed(self) -> np.ndarray:
        v = np.zeros(16)
        if self.n_periods > 0:
            v[0] = 1.0
            v[1], v[2], v[3] = self.b_peak, self.lambda_u, self.n_periods
            v[4:7] = self.origin
        if self.hom_e is not None or self.hom_b is not None:
            v[7] = 1.0
            v[8:11] = self.hom_e or (0.0, 0.0, 0.0)
            v[11:14] = self.hom_b or (0.0, 0.0, 0.0)
        return v

    @property
    def z1(self) -> float:
        """Upstream end of the undulator's field region (src/undulator.cpp:112)."""
        return -(self.n_periods + 1) * self.lambda_u / 2.0 + self.origin[2]

    @property
    def z2(self) -> float:
        return (self.n_periods + 1) * self.lambda_u / 2.0 + self.origin[2]


def undulator(K: float, lambda_u: float, n_periods: int) -> Lattice:
    return Lattice(b_peak=lib().tg_undulator_b0(K, lambda_u), lambda_u=lambda_u,
                   n_periods=n_periods)


@dataclass
class Trajectories:
    """Concatenated trajectories of a particle set (the reference's
    ChargedParticle::Time/X/P/A arrays, src/particle.h:417-427)."""
    t: np.ndarray        # [Npts]
    x: np.ndarray        # [Npts, 3]
    p: np.ndarray        # [Npts, 3] beta*gamma
    a: np.ndarray        # [Npts, 3] d(beta*gamma)/dt
    n_points: np.ndarray  # [Npart] int32
    charge: np.ndarray   # [Npart] units of e
    mass: np.ndarray     # [Npart] electron masses

    @property
    def n_particles(self) -> int:
        return int(self.n_points.shape[0])

    @property
    def offsets(self) -> np.ndarray:
        o = np.zeros(self.n_particles + 1, dtype=np.int64)
        np.cumsum(self.n_points, out=o[1:])
        return o

    def subset(self, idx) -> "Trajectories":
        o = self.offsets
        sel = np.concatenate([np.arange(o[i], o[i + 1]) for i in idx]) if len(idx) else \
            np.zeros(0, dtype=np.int64)
        return Trajectories(self.t[sel].copy(), self.x[sel].copy(), self.p[sel].copy(),
                            self.a[sel].copy(), self.n_points[list(idx)].copy(),
                            self.charge[list(idx)].copy(), self.mass[list(idx)].copy())


def track(init: np.ndarray, lattice: Lattice, tstep: float, n_steps: int,
          charge: float, mass: float, nthreads: int = 0) -> Trajectories:
    """Track every particle of ``init`` ([n,7]: t,x,y,z,px,py,pz) for n_steps
    Vay steps; each trajectory holds n_steps+1 points."""
    init = np.ascontiguousarray(init, dtype=np.float64)
    n = init.shape[0]
    npnt = n_steps + 1
    t = np.empty(n * npnt)
    x = np.empty((n * npnt, 3))
    p = np.empty((n * npnt, 3))
    a = np.empty((n * npnt, 3))
    rc = lib().tg_track(n, _dp(init), charge, mass, _dp(lattice.packed()), tstep, n_steps,
                        _dp(t), _dp(x), _dp(p), _dp(a), nthreads)
    if rc != 0:
        raise ValueError("tg_track rejected its arguments")
    return Trajectories(t, x, p, a, np.full(n, npnt, dtype=np.int32),
                        np.full(n, charge, dtype=np.float64), np.full(n, mass, dtype=np.float64))


def gaussian_bunch(n: int, seed: int, sx: float, sy: float, sz: float, spx: float, spy: float,
                   gamma0: float, sgamma: float, z0: float, first: int = 0) -> np.ndarray:
    out = np.empty((n, 7))
    lib().tg_gaussian_bunch(first, n, seed, sx, sy, sz, spx, spy, gamma0, sgamma, z0, _dp(out))
    return out


def uniform(seed: int, n: int, lo: float, hi: float) -> np.ndarray:
    out = np.empty(n)
    lib().tg_uniform(seed, n, lo, hi, _dp(out))
    return out


# --------------------------------------------------------------------------
# observers
# --------------------------------------------------------------------------
@dataclass
class Screen:
    """ScreenObserver geometry (src/screen.cpp:34-86)."""
    origin: tuple
    dx: tuple
    dy: tuple
    nx: int
    ny: int
    t0: float
    dt: float
    nots: int
    dtx: float = 0.0
    dty: float = 0.0

    @property
    def n_pix(self) -> int:
        return self.nx * self.ny

    def pixel_positions(self) -> np.ndarray:
        """CellPosition(ix, iy) = Origin + dX*(ix-Nx/2) + dY*(iy-Ny/2)
        (src/screen.cpp:97-103); evaluated in the same order."""
        o = np.array(self.origin, dtype=np.float64)
        dX = np.array(self.dx, dtype=np.float64)
        dY = np.array(self.dy, dtype=np.float64)
        ix = (np.arange(self.nx) - self.nx // 2).astype(np.float64)
        iy = (np.arange(self.ny) - self.ny // 2).astype(np.float64)
        a = o[None, None, :] + dX[None, None, :] * ix[:, None, None]
        pos = a + dY[None, None, :] * iy[None, :, None]
        return np.ascontiguousarray(pos.reshape(-1, 3))

    def pixel_t0(self) -> np.ndarray:
        """CellTimeZero(ix, iy) (src/screen.cpp:105-110)."""
        ix = (np.arange(self.nx) - self.nx // 2).astype(np.float64)
        iy = (np.arange(self.ny) - self.ny // 2).astype(np.float64)
        t = self.t0 + self.dtx * ix[:, None]
        t = t + self.dty * iy[None, :]
        return np.ascontiguousarray(t.reshape(-1))


@dataclass
class Workload:
    name: str
    traj: Trajectories
    pix_pos: np.ndarray
    pix_t0: np.ndarray
    dt: float
    nots: int
    info: dict = field(default_factory=dict)

    @property
    def n_pix(self) -> int:
        return int(self.pix_pos.shape[0])

    @property
    def triples(self) -> int:
        """particle x step x pixel evaluations (every step, in window or not)."""
        return int(np.sum(np.maximum(self.traj.n_points.astype(np.int64) - 1, 0))) * self.n_pix

    def pixel_subset(self, idx) -> "Workload":
        idx = np.asarray(idx)
        return Workload(self.name + f"[{len(idx)} px]", self.traj,
                        np.ascontiguousarray(self.pix_pos[idx]),
                        np.ascontiguousarray(self.pix_t0[idx]), self.dt, self.nots,
                        dict(self.info))


# --------------------------------------------------------------------------
# the five workloads
# --------------------------------------------------------------------------
def _undulator_run(gamma0, K, lambda_u, n_periods, steps_per_period, drift):
    lat = undulator(K, lambda_u, n_periods)
    beta0 = math.sqrt(1.0 - 1.0 / (gamma0 * gamma0))
    tstep = lambda_u / (steps_per_period * beta0 * C_LIGHT)
    z_start = lat.z1 - drift
    length = (lat.z2 + drift) - z_start
    n_steps = int(math.ceil(length / (beta0 * C_LIGHT * tstep)))
    return lat, beta0, tstep, z_start, n_steps


def _entrance_signal_time(z_start, z1, beta0, z_screen):
    """Arrival time on the screen axis of the signal a particle moving
    straight at beta0 emits when it passes the undulator entrance z1."""
    t_enter = (z1 - z_start) / (beta0 * C_LIGHT)
    return t_enter + (z_screen - z1) / C_LIGHT


def config1(nthreads: int = 0) -> Workload:
    """One electron, gamma=50, 8-period K=1 undulator (lambda_u=0.1 m),
    200 steps/period and 0.5 m drifts; 21x21 screen at z=10 m, pitch 0.01 m;
    2048 x 5 fs traces starting 1 ps before the on-axis straight-line arrival."""
    gamma0, K, lu, nper = 50.0, 1.0, 0.1, 8
    lat, beta0, tstep, z_start, n_steps = _undulator_run(gamma0, K, lu, nper, 200, 0.5)
    init = np.array([[0.0, 0.0, 0.0, z_start, 0.0, 0.0, gamma0 * beta0]])
    traj = track(init, lat, tstep, n_steps, -1.0, 1.0, nthreads)
    t_arr = _entrance_signal_time(z_start, lat.z1, beta0, 10.0)
    scr = Screen((0.0, 0.0, 10.0), (0.01, 0.0, 0.0), (0.0, 0.01, 0.0), 21, 21,
                 t_arr - 1.0e-12, 5.0e-15, 2048)
    return Workload("config1", traj, scr.pixel_positions(), scr.pixel_t0(), scr.dt, scr.nots,
                    dict(screen=scr, n_steps=n_steps, tstep=tstep, lattice=lat))


def _bunch_config(name, *, n_particles, total_charge, sx, sy, sz, eps_n, gamma0, rel_spread,
                  K, lu, nper, spp, drift, z_screen, width, npix, dt, nots, seed, t0_mode,
                  first=0, count=None, nthreads=0):
    lat, beta0, tstep, z_start, n_steps = _undulator_run(gamma0, K, lu, nper, spp, drift)
    count = n_particles if count is None else count
    init = gaussian_bunch(count, seed, sx, sy, sz, eps_n / sx, eps_n / sy, gamma0,
                          gamma0 * rel_spread, z_start, first=first)
    ne = total_charge / E_CHARGE / n_particles
    traj = track(init, lat, tstep, n_steps, -ne, ne, nthreads)
    t_arr = _entrance_signal_time(z_start, lat.z1, beta0, z_screen)
    pitch = width / (npix - 1)
    if t0_mode == "entrance":
        t0 = t_arr - 1.0e-12
    else:  # centred on the on-axis signal from the undulator centre
        t_c = (0.0 - z_start) / (beta0 * C_LIGHT) + z_screen / C_LIGHT
        t_c += _slippage_to_centre(lat, gamma0, K, z_start)
        t0 = t_c - 0.5 * nots * dt
    scr = Screen((0.0, 0.0, z_screen), (pitch, 0.0, 0.0), (0.0, pitch, 0.0), npix, npix,
                 t0, dt, nots)
    return Workload(name, traj, scr.pixel_positions(), scr.pixel_t0(), dt, nots,
                    dict(screen=scr, n_steps=n_steps, tstep=tstep, n_particles=n_particles,
                         first=first, seed=seed))


def _slippage_to_centre(lat, gamma0, K, z_start):
    """Extra on-axis delay of the wiggling particle relative to the straight
    line at beta0 when it reaches the undulator centre: half the undulator
    length times K^2/(4 gamma^2)/c (average longitudinal slow-down)."""
    half = 0.0 - lat.z1
    return half * K * K / (4.0 * gamma0 * gamma0) / C_LIGHT


def config2(n_particles: int = 10000, first: int = 0, count: Optional[int] = None,
            nthreads: int = 0) -> Workload:
    """1e4 macro-particles, 100 pC, sigma_x=y=0.5 mm, eps_n=10 mm mrad,
    sigma_z=300 um, gamma=50 +- 0.1%; config-1 undulator; 64x64 pixels over
    the same 0.2 m screen; 2048 x 5 fs."""
    return _bunch_config("config2", n_particles=n_particles, total_charge=100e-12, sx=0.5e-3,
                         sy=0.5e-3, sz=300e-6, eps_n=10e-6, gamma0=50.0, rel_spread=1e-3, K=1.0,
                         lu=0.1, nper=8, spp=200, drift=0.5, z_screen=10.0, width=0.2, npix=64,
                         dt=5e-15, nots=2048, seed=20240602, t0_mode="entrance", first=first,
                         count=count, nthreads=nthreads)


def config4(n_particles: int = 100000, first: int = 0, count: Optional[int] = None,
            nthreads: int = 0) -> Workload:
    """1e5 macro-particles, 200 pC, sigma_z=100 um, sigma_x=y=1 mm,
    gamma=300 +- 0.05%; lambda_u=0.3 m, 20 periods, K=3, 100 steps/period and
    0.5 m drifts; 200x200 pixels over 0.4x0.4 m at z=20 m; 4096 x 2 fs."""
    return _bunch_config("config4", n_particles=n_particles, total_charge=200e-12, sx=1e-3,
                         sy=1e-3, sz=100e-6, eps_n=10e-6, gamma0=300.0, rel_spread=5e-4, K=3.0,
                         lu=0.3, nper=20, spp=100, drift=0.5, z_screen=20.0, width=0.4,
                         npix=200, dt=2e-15, nots=4096, seed=20240604, t0_mode="entrance",
                         first=first, count=count, nthreads=nthreads)


def config5(n_particles: int = 1000, first: int = 0, count: Optional[int] = None,
            nthreads: int = 0) -> Workload:
    """1e3 macro-particles, sigma_x=y=50 um, sigma_z=20 um, gamma=2000 +- 0.01%;
    lambda_u=0.05 m, 50 periods, K=10, 400 steps/period, 0.5 m drifts;
    100x100 pixels over 0.05 m at z=30 m; 8192 x 1e-18 s centred on the
    on-axis arrival from the undulator centre."""
    return _bunch_config("config5", n_particles=n_particles, total_charge=100e-12, sx=50e-6,
                         sy=50e-6, sz=20e-6, eps_n=1e-6, gamma0=2000.0, rel_spread=1e-4, K=10.0,
                         lu=0.05, nper=50, spp=400, drift=0.5, z_screen=30.0, width=0.05,
                         npix=100, dt=1e-18, nots=8192, seed=20240605, t0_mode="centre",
                         first=first, count=count, nthreads=nthreads)


def config3_specs(seed: int = 20240603, n_screens: int = 16) -> List[dict]:
    """Seeded parameter draws for the batched uneven observers: per screen a
    particle count in [1e3, 1e5] (log-uniform), gamma U(20,100), periods
    U{4..40}, K U(0.5,2), lambda_u U(0.05,0.3), a step count in [2e3, 2e4]
    (log-uniform; sets the steps per period), a square mesh of 16..128 pixels
    per side (log-uniform), 512..8192 samples (power of two) and dt in
    [2e-15, 2e-14] s (log-uniform)."""
    u = uniform(seed, 8 * n_screens, 0.0, 1.0).reshape(n_screens, 8)
    specs = []
    for i in range(n_screens):
        r = u[i]
        n_part = int(round(10 ** (3 + 2 * r[0])))
        gamma0 = 20.0 + 80.0 * r[1]
        nper = 4 + int(r[2] * 37) if r[2] < 1 else 40
        K = 0.5 + 1.5 * r[3]
        lu = 0.05 + 0.25 * r[4]
        n_steps_target = 10 ** (math.log10(2e3) + r[5])
        npix = int(round(2 ** (4 + 3 * r[6])))
        nots = int(2 ** int(9 + min(4.999, 5 * r[7])))
        dt = 10 ** (math.log10(2e-15) + ((r[0] + r[7]) % 1.0))
        specs.append(dict(n_particles=n_part, gamma0=gamma0, n_periods=nper, K=K,
                          lambda_u=lu, n_steps_target=n_steps_target, npix=npix, nots=nots,
                          dt=dt, seed=seed * 100 + i))
    return specs


def config3_screen(spec: dict, count: Optional[int] = None, nthreads: int = 0) -> Workload:
    drift = 0.5
    lat = undulator(spec["K"], spec["lambda_u"], spec["n_periods"])
    length = lat.z2 - lat.z1 + 2 * drift
    spp = max(8, int(round(spec["n_steps_target"] * spec["lambda_u"] / length)))
    return _bunch_config("config3", n_particles=spec["n_particles"], total_charge=100e-12,
                         sx=0.5e-3, sy=0.5e-3, sz=300e-6, eps_n=10e-6, gamma0=spec["gamma0"],
                         rel_spread=1e-3, K=spec["K"], lu=spec["lambda_u"],
                         nper=spec["n_periods"], spp=spp, drift=drift, z_screen=10.0,
                         width=0.2, npix=spec["npix"], dt=spec["dt"], nots=spec["nots"],
                         seed=spec["seed"], t0_mode="entrance", count=count, nthreads=nthreads)
