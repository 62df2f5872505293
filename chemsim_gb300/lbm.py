"""Host-side mirror of taktoa/chemsim's src/lbm.rs API over the C ABI.

Names, argument meaning and error behaviour follow lbm.rs:

  Discretization (src/lbm.rs:75-86), D2Q9.directions (:202-282),
  compute_equilibrium (:43-71), BGK (:345-370), TRT (:374-451),
  State.initial / step / density / velocity / speed / momentum_density /
  pressure / equilibrium / non_equilibrium / is_unstable (:670-819).

Fields are numpy arrays shaped (h, w) — row = y, column = x, the layout of
Matrix (src/matrix.rs:24-30) — and populations are shaped (9, h, w) in
D2Q9 direction order.  Where lbm.rs panics (assert!/assert_eq!), this module
raises; where the C ABI returns a negative status, LBMError is raised.
Every computation runs in liblbm_cuda.so on the GPU.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import (BF16DEV, COLLISION_BGK, COLLISION_TRT, F16DEV, F32, F64,  # noqa: F401
                   FAST, FRAME_REF, FRAME_XY, REFERENCE_FLAGS, ROUND_NEAREST, SOLID_FULLWAY,
                   SOLID_HALFWAY, X_PERIODIC, X_WALL, X_ZEROPAD, Y_PERIODIC,
                   Y_WALL, Y_ZEROPAD, LBMError, LBMHealth, check)

# render modes (src/main.rs:158-173 DisplayMode)
RENDER_DENSITY, RENDER_SPEED, RENDER_VELOCITY, RENDER_MOMENTUM = 0, 1, 2, 3

# src/lbm.rs:205-227 (as f32)
WEIGHTS = tuple(np.float32(n) / np.float32(36.0) for n in (16, 4, 4, 4, 4, 1, 1, 1, 1))
VELOCITIES = ((0, 0), (1, 0), (0, 1), (-1, 0), (0, -1), (1, 1), (-1, 1), (-1, -1), (1, -1))
OPPOSITE = (0, 3, 4, 1, 2, 7, 8, 5, 6)


def _f32ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class Lattice:
    """One device lattice (an lbm_lattice handle).

    The thin object wrapper the tests and the bench use; State below adds the
    lbm.rs surface on top of it.
    """

    def __init__(self, w: int, h: int, tau: float, precision: int = F32,
                 flags: int = REFERENCE_FLAGS):
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        check(self._lib.lbm_create(int(w), int(h), float(tau), int(precision),
                                   int(flags), ctypes.byref(self._h)))
        self.w, self.h, self.precision, self.flags = int(w), int(h), precision, flags

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if self._h:
            self._lib.lbm_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- configuration ----------------------------------------------------
    def set_discretization(self, dx: float, dt: float):
        check(self._lib.lbm_set_discretization(self._h, float(dx), float(dt)))

    def set_collision(self, kind: int, tau: float, tau_minus: float = 1.0):
        check(self._lib.lbm_set_collision(self._h, int(kind), float(tau), float(tau_minus)))

    def set_force(self, fx: float, fy: float):
        check(self._lib.lbm_set_force(self._h, float(fx), float(fy)))

    def set_geometry(self, solid):
        if solid is None:
            check(self._lib.lbm_set_geometry(self._h, None))
            return
        m = np.ascontiguousarray(solid, dtype=np.uint8)
        if m.shape != (self.h, self.w):
            raise ValueError(f"geometry must be shaped {(self.h, self.w)}")
        check(self._lib.lbm_set_geometry(self._h, _f32ptr(m)))

    def set_tile(self, cells_per_thread: int = 0, rows_per_block: int = 0):
        check(self._lib.lbm_set_tile(self._h, int(cells_per_thread), int(rows_per_block)))

    # -- state ------------------------------------------------------------
    def _field(self, a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        if a.shape != (self.h, self.w):
            raise ValueError(f"field must be shaped {(self.h, self.w)}")
        return a

    def init_equilibrium(self, rho, ux, uy):
        r, x, y = self._field(rho), self._field(ux), self._field(uy)
        check(self._lib.lbm_init_equilibrium(self._h, _f32ptr(r), _f32ptr(x), _f32ptr(y)))

    def set_populations(self, f):
        f = np.asarray(f)
        if f.shape != (9, self.h, self.w):
            raise ValueError(f"populations must be shaped {(9, self.h, self.w)}")
        if f.dtype == np.float64:
            f = np.ascontiguousarray(f)
            check(self._lib.lbm_set_populations_f64(self._h, _f32ptr(f)))
        else:
            f = np.ascontiguousarray(f, dtype=np.float32)
            check(self._lib.lbm_set_populations(self._h, _f32ptr(f)))

    def get_populations(self, dtype=np.float32) -> np.ndarray:
        out = np.empty((9, self.h, self.w), dtype=dtype)
        if out.dtype == np.float64:
            check(self._lib.lbm_get_populations_f64(self._h, _f32ptr(out)))
        else:
            check(self._lib.lbm_get_populations(self._h, _f32ptr(out)))
        return out

    def step(self, nsteps: int = 1):
        check(self._lib.lbm_step(self._h, int(nsteps)))

    def step_moments(self, nsteps: int = 1):
        check(self._lib.lbm_step_moments(self._h, int(nsteps)))

    def moments(self):
        rho = np.empty((self.h, self.w), dtype=np.float32)
        ux = np.empty_like(rho)
        uy = np.empty_like(rho)
        check(self._lib.lbm_read_moments(self._h, _f32ptr(rho), _f32ptr(ux), _f32ptr(uy), 0))
        return rho, ux, uy

    def read_moments_async(self, rho: np.ndarray, ux: np.ndarray, uy: np.ndarray):
        """Starts copying rho/u into these (h, w) float32 host arrays (pinned for
        overlap); they hold the fields of the current step once
        readback_wait() returns (lbm_read_moments_async)."""
        for a in (rho, ux, uy):
            if a.dtype != np.float32 or a.shape != (self.h, self.w) or not a.flags.c_contiguous:
                raise ValueError("expected contiguous (h, w) float32 arrays")
        check(self._lib.lbm_read_moments_async(self._h, _f32ptr(rho), _f32ptr(ux), _f32ptr(uy)))

    def step_moments_to(self, nsteps: int, rho_ptr: int, ux_ptr: int, uy_ptr: int):
        """nsteps steps; the last writes rho/u (w*h f32 each, row-major)
        straight to the given device or pinned-host addresses; wait with
        readback_wait() (lbm_step_moments_to)."""
        check(self._lib.lbm_step_moments_to(self._h, int(nsteps), ctypes.c_void_p(rho_ptr),
                                            ctypes.c_void_p(ux_ptr), ctypes.c_void_p(uy_ptr)))

    def readback_wait(self):
        check(self._lib.lbm_readback_wait(self._h))

    def moments_to_device(self, rho_ptr: int, ux_ptr: int, uy_ptr: int):
        check(self._lib.lbm_read_moments(self._h, ctypes.c_void_p(rho_ptr),
                                         ctypes.c_void_p(ux_ptr), ctypes.c_void_p(uy_ptr), 1))

    def save(self, path: str):
        """Checkpoint: exact state, geometry and parameters (lbm_save)."""
        check(self._lib.lbm_save(self._h, str(path).encode()))

    def load(self, path: str):
        """Resume from a checkpoint of a lattice of this size and precision."""
        check(self._lib.lbm_load(self._h, str(path).encode()))

    def render(self, mode: int = 0, geometry_overlay: bool = True) -> np.ndarray:
        """RGBA8 image (h, w, 4) of a moment field coloured as src/render.rs
        does (mode: RENDER_DENSITY, RENDER_SPEED, RENDER_VELOCITY,
        RENDER_MOMENTUM)."""
        img = np.empty((self.h, self.w, 4), dtype=np.uint8)
        check(self._lib.lbm_render(self._h, int(mode), int(bool(geometry_overlay)),
                                   img.ctypes.data_as(ctypes.c_void_p), 0))
        return img

    def render_async(self, img: np.ndarray, mode: int = 0, geometry_overlay: bool = True):
        """Starts rendering into this (h, w, 4) uint8 host array (pinned for
        overlap); it holds the frame once readback_wait() returns."""
        if img.dtype != np.uint8 or img.shape != (self.h, self.w, 4) or not img.flags.c_contiguous:
            raise ValueError("expected a contiguous (h, w, 4) uint8 array")
        check(self._lib.lbm_render_async(self._h, int(mode), int(bool(geometry_overlay)),
                                         img.ctypes.data_as(ctypes.c_void_p)))

    def render_to_device(self, rgba_ptr: int, mode: int = 0, geometry_overlay: bool = True):
        check(self._lib.lbm_render(self._h, int(mode), int(bool(geometry_overlay)),
                                   ctypes.c_void_p(rgba_ptr), 1))

    def health(self) -> dict:
        hs = LBMHealth()
        check(self._lib.lbm_check(self._h, ctypes.byref(hs)))
        return hs.as_dict()

    def time(self):
        t = ctypes.c_float()
        n = ctypes.c_int64()
        check(self._lib.lbm_get_time(self._h, ctypes.byref(t), ctypes.byref(n)))
        return t.value, n.value

    def synchronize(self):
        check(self._lib.lbm_synchronize(self._h))

    def set_stream(self, stream_ptr: int | None):
        check(self._lib.lbm_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def device_populations(self):
        base = ctypes.c_void_p()
        plane = ctypes.c_int64()
        pitch = ctypes.c_int()
        check(self._lib.lbm_device_populations(self._h, ctypes.byref(base), ctypes.byref(plane),
                                               ctypes.byref(pitch)))
        return base.value, plane.value, pitch.value


class _Member(Lattice):
    """A lattice owned by a Batch (not destroyed on its own)."""

    def __init__(self, lib, handle, w, h, flags):
        self._lib = lib
        self._h = handle
        self.w, self.h, self.precision, self.flags = w, h, F32, flags

    def close(self):
        self._h = ctypes.c_void_p()


class Batch:
    """Many independent f32 lattices stepped together (lbm_batch_*).

    specs: objects with w, h, tau, flags, force and solid (see
    chemsim_gb300.workloads.LatticeSpec).  `flags` of the batch carries
    FRAME_XY / FAST for every member.
    """

    def __init__(self, specs, flags: int = FRAME_XY | FAST):
        self._lib = _lib.load()
        descs = (_lib.LBMDesc * len(specs))()
        self._masks = []
        for d, sp in zip(descs, specs):
            d.w, d.h, d.tau = int(sp.w), int(sp.h), float(sp.tau)
            d.flags = int(sp.flags) & ~(FRAME_XY | FAST)
            d.fx, d.fy = float(sp.force[0]), float(sp.force[1])
            if sp.solid is not None and np.any(sp.solid):
                m = np.ascontiguousarray(sp.solid, dtype=np.uint8)
                self._masks.append(m)
                d.solid = m.ctypes.data
            else:
                d.solid = None
        self._b = ctypes.c_void_p()
        check(self._lib.lbm_batch_create(len(specs), descs, int(flags), ctypes.byref(self._b)))
        self._masks = []
        self.members = []
        for i, sp in enumerate(specs):
            hnd = ctypes.c_void_p()
            check(self._lib.lbm_batch_lattice(self._b, i, ctypes.byref(hnd)))
            self.members.append(_Member(self._lib, hnd, int(sp.w), int(sp.h),
                                        (int(sp.flags) & ~(FRAME_XY | FAST)) | flags))

    def __len__(self):
        return len(self.members)

    def __getitem__(self, i) -> Lattice:
        return self.members[i]

    def step(self, nsteps: int = 1):
        check(self._lib.lbm_batch_step(self._b, int(nsteps)))

    def synchronize(self):
        check(self._lib.lbm_batch_synchronize(self._b))

    def set_stream(self, stream_ptr):
        check(self._lib.lbm_batch_set_stream(self._b, ctypes.c_void_p(stream_ptr or 0)))

    def set_tile(self, cells_per_thread: int):
        """The batch kernel's tile width, 2 or 4 cells per thread."""
        check(self._lib.lbm_batch_set_tile(self._b, int(cells_per_thread)))

    def tile(self) -> int:
        v = ctypes.c_int32()
        check(self._lib.lbm_batch_tile(self._b, ctypes.byref(v)))
        return v.value

    def autotune(self, cache_path: str | None = None, steps_per_trial: int = 0):
        path = cache_path.encode() if cache_path else None
        check(self._lib.lbm_batch_autotune(self._b, path, int(steps_per_trial)))

    def close(self):
        if self._b:
            for m in self.members:
                m.close()
            self._lib.lbm_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# ---------------------------------------------------------------------------
# lbm.rs surface
# ---------------------------------------------------------------------------

@dataclass(frozen=True)
class Discretization:
    """src/lbm.rs:75-86."""
    delta_x: float = 1.0
    delta_t: float = 1.0

    def isothermal_speed_of_sound(self) -> float:
        return float(np.float32(self.delta_x) / (np.sqrt(np.float32(3.0)) * np.float32(self.delta_t)))


@dataclass(frozen=True)
class Direction:
    w_scalar: float
    c_vector: tuple


class D2Q9:
    """Host container of 9 population planes (src/lbm.rs:180-200)."""

    def __init__(self, populations):
        pops = [np.asarray(p, dtype=np.float32) for p in populations]
        assert len(pops) == 9, "D2Q9 needs 9 populations"            # src/lbm.rs:188
        for p in pops:
            assert p.shape == pops[0].shape, "population shapes differ"   # :191
        self.populations = np.stack(pops)

    @staticmethod
    def new(populations) -> "D2Q9":
        return D2Q9(populations)

    @staticmethod
    def directions():
        return [Direction(float(w), c) for w, c in zip(WEIGHTS, VELOCITIES)]

    def size(self):
        _, h, w = self.populations.shape
        return (w, h)


@dataclass(frozen=True)
class BGK:
    """src/lbm.rs:345-370."""
    tau: float

    def kinematic_shear_viscosity(self, disc: Discretization) -> float:
        dx, dt = disc.delta_x, disc.delta_t
        return (dx * dx / (3.0 * dt * dt)) * (self.tau - dt / 2.0)


@dataclass(frozen=True)
class TRT:
    """src/lbm.rs:374-451 (tau_minus, tau_plus)."""
    tau_minus: float
    tau_plus: float

    @staticmethod
    def new(lam: float, ks_viscosity: float, disc: Discretization) -> "TRT":
        dt = disc.delta_t
        cs = disc.isothermal_speed_of_sound()
        tau_plus = dt * ((ks_viscosity / (cs * cs)) + 0.5)
        tau_minus = dt * ((lam / ((tau_plus / dt) - 0.5)) + 0.5)
        return TRT(tau_minus=tau_minus, tau_plus=tau_plus)

    def kinematic_shear_viscosity(self, disc: Discretization) -> float:
        cs = disc.isothermal_speed_of_sound()
        return cs * cs * (self.tau_plus / disc.delta_t - 0.5)


def compute_equilibrium(density, velocity, directions=None,
                        discretization: Discretization = Discretization()):
    """src/lbm.rs:43-71, evaluated on the GPU; returns (9, h, w) f32."""
    density = np.asarray(density, dtype=np.float32)
    vx, vy = (np.asarray(v, dtype=np.float32) for v in velocity)
    assert density.shape == vx.shape and density.shape == vy.shape   # src/lbm.rs:51-52
    h, w = density.shape
    with Lattice(w, h, 1.0, F32, REFERENCE_FLAGS) as lat:
        lat.set_discretization(discretization.delta_x, discretization.delta_t)
        lat.init_equilibrium(density, vx, vy)
        return lat.get_populations()


class State:
    """src/lbm.rs:670-819 on a device lattice.

    `precision` and `flags` select the storage and the boundary treatment;
    the defaults are the reference's (f32, zero-padded streaming, full-way
    bounce-back on solid nodes, the reference frame and operation order).
    """

    def __init__(self, lattice: D2Q9, geometry, collision, discretization: Discretization,
                 precision: int = F32, flags: int = REFERENCE_FLAGS):
        w, h = lattice.size()
        tau = collision.tau if isinstance(collision, BGK) else collision.tau_plus
        self._lat = Lattice(w, h, tau, precision, flags)
        self._lat.set_discretization(discretization.delta_x, discretization.delta_t)
        if isinstance(collision, TRT):
            self._lat.set_collision(COLLISION_TRT, collision.tau_plus, collision.tau_minus)
        elif not isinstance(collision, BGK):
            raise TypeError("collision must be BGK or TRT")
        self._lat.set_populations(lattice.populations)
        self.collision = collision
        self.discretization = discretization
        self.geometry = geometry

    @staticmethod
    def initial(lattice, geometry, collision, discretization, **kw) -> "State":
        return State(lattice, geometry, collision, discretization, **kw)

    @property
    def device(self) -> Lattice:
        return self._lat

    @property
    def geometry(self):
        return self._geometry

    @geometry.setter
    def geometry(self, g):
        self._geometry = None if g is None else np.asarray(g, dtype=bool)
        self._lat.set_geometry(None if g is None else self._geometry.astype(np.uint8))

    @property
    def time(self) -> float:
        return self._lat.time()[0]

    def step(self, nsteps: int = 1):
        """State::step (src/lbm.rs:694-714), nsteps times."""
        self._lat.step(nsteps)

    def size(self):
        return (self._lat.w, self._lat.h)

    def delta_x(self):
        return self.discretization.delta_x

    def delta_t(self):
        return self.discretization.delta_t

    def populations(self) -> np.ndarray:
        return self._lat.get_populations()

    def isothermal_speed_of_sound(self) -> float:
        return self.discretization.isothermal_speed_of_sound()

    def density(self) -> np.ndarray:
        return self._lat.moments()[0]

    def velocity(self):
        _, ux, uy = self._lat.moments()
        return ux, uy

    def momentum_density(self):
        rho, ux, uy = self._lat.moments()
        return rho * ux, rho * uy

    def speed(self) -> np.ndarray:
        _, ux, uy = self._lat.moments()
        return np.sqrt(ux * ux + uy * uy)

    def pressure(self) -> np.ndarray:
        cs = np.float32(self.isothermal_speed_of_sound())
        return self.density() * (cs * cs)

    def equilibrium(self) -> np.ndarray:
        rho, ux, uy = self._lat.moments()
        return compute_equilibrium(rho, (ux, uy), None, self.discretization)

    def non_equilibrium(self) -> np.ndarray:
        return self.populations() - self.equilibrium()

    def is_unstable(self) -> bool:
        """src/lbm.rs:815-818: min over cells of f_eq[0] < 0."""
        hs = self._lat.health()
        return bool(hs["min_eq0"] < 0.0 or math.isnan(hs["min_eq0"]))

    def health(self) -> dict:
        return self._lat.health()
