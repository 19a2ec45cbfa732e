"""ctypes binding to the oracle libraries (test infrastructure only).

``Oracle`` wraps oracle/_build/libkpt_oracle.so (the C restatement);
``ReferenceHarness`` wraps oracle/_ref/libkpt_ref.so (the reference's own
sources compiled on the Kokkos-API shim) when it has been built.  Only tests,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs use this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libkpt_oracle.so")
# the same restatement on the C library's pow: the build timed as the CPU baseline
ORACLE_LIBM_SO = os.path.join(HERE, "_build", "libkpt_oracle_libm.so")
REF_SO = os.path.join(HERE, "_ref", "libkpt_ref.so")
# the reference on the shim with the C library's pow (timing only)
REF_LIBM_SO = os.path.join(HERE, "_ref", "libkpt_ref_libm.so")

PARTICLE_FIELDS = ("x", "y", "p", "t", "dt", "w", "mu", "status", "level")
DOUBLE_PARAMS = ("mhd_dt", "p0", "pmin", "pmax", "gamma_turb", "kpara0", "kperp_over_kpara",
                 "dt_min_rel", "dt_max_rel", "drift_param1", "drift_param2", "charge",
                 "particle_v0", "duu0", "split_ratio", "pmin_split_over_p0", "mu_max")
INT_PARAMS = ("max_steps", "momentum_dependency", "magnetic_dependency", "time_interpolation",
              "split_particles", "focused")
CLOSURE_INT = ("closure",)
CLOSURE_DOUBLE = ("qlt_sigma2", "qlt_spectral_index", "qlt_h0", "qlt_omega0", "qlt_lc")


class OracleParams(ctypes.Structure):
    _fields_ = [(name, ctypes.c_double) for name in DOUBLE_PARAMS] + \
               [(name, ctypes.c_int32) for name in INT_PARAMS + CLOSURE_INT] + \
               [(name, ctypes.c_double) for name in CLOSURE_DOUBLE]


class OracleSummary(ctypes.Structure):
    _fields_ = [("stored", ctypes.c_uint64), ("active", ctypes.c_uint64),
                ("inactive", ctypes.c_uint64), ("weight_sum", ctypes.c_double),
                ("p_min", ctypes.c_double), ("p_max", ctypes.c_double),
                ("p_avg", ctypes.c_double), ("dt_min", ctypes.c_double),
                ("dt_max", ctypes.c_double), ("dt_avg", ctypes.c_double),
                ("max_split_level", ctypes.c_int32), ("pad", ctypes.c_int32)]


class OracleGrid(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int * 2), ("stored", ctypes.c_int * 2),
                ("start", ctypes.c_double * 2), ("step", ctypes.c_double * 2),
                ("faces", ctypes.c_void_p * 2), ("centers", ctypes.c_void_p * 2),
                ("lower", ctypes.c_double * 2), ("upper", ctypes.c_double * 2),
                ("width", ctypes.c_double * 2), ("inv_width", ctypes.c_double * 2),
                ("ghost_lower", ctypes.c_double * 2), ("ghost_upper", ctypes.c_double * 2)]


def default_params(**overrides) -> Dict[str, float]:
    """Reference defaults (src/main.cpp:136-154) with overrides."""
    values = dict(mhd_dt=0.1, p0=0.1, pmin=1.0e-2, pmax=1.0e1, gamma_turb=1.6666667,
                  kpara0=0.00743592, kperp_over_kpara=0.01, dt_min_rel=1.0e-7,
                  dt_max_rel=1.0e-2, drift_param1=850964.408, drift_param2=13575468.975,
                  charge=-1.0, particle_v0=17.20195, duu0=5578.445, split_ratio=2.0,
                  pmin_split_over_p0=2.0, mu_max=0.99, max_steps=200000, momentum_dependency=1,
                  magnetic_dependency=1, time_interpolation=1, split_particles=1, focused=0,
                  closure=0, qlt_sigma2=0.1, qlt_spectral_index=5.0 / 3.0, qlt_h0=1.0e-6,
                  qlt_omega0=1000.0, qlt_lc=0.05)
    for key, value in overrides.items():
        if key not in values:
            raise KeyError(key)
        values[key] = value
    return values


def make_params(values: Dict[str, float]) -> OracleParams:
    params = OracleParams()
    for name in DOUBLE_PARAMS:
        setattr(params, name, float(values[name]))
    for name in INT_PARAMS + CLOSURE_INT:
        setattr(params, name, int(values[name]))
    for name in CLOSURE_DOUBLE:
        setattr(params, name, float(values[name]))
    return params


def _ptr(array: Optional[np.ndarray]):
    return None if array is None else array.ctypes.data_as(ctypes.c_void_p)


LIB_DOUBLE_FIELDS = ("x", "y", "prev_x", "prev_y", "prevstep_x", "prevstep_y", "p", "mu", "w",
                     "e0")
LIB_INT_FIELDS = ("status", "level", "key")


def lib_default_system(count: int, capacity: int) -> Dict[str, np.ndarray]:
    """ParticleSystem::initialize_default_state (ParticleSystem.hpp:1163-1198)."""
    out = {name: np.zeros(capacity, dtype=np.float64) for name in LIB_DOUBLE_FIELDS}
    out["w"][:] = 1.0
    out["id"] = np.arange(capacity, dtype=np.uint64)
    out["status"] = np.where(np.arange(capacity) < count, 0, 2).astype(np.int32)
    out["level"] = np.zeros(capacity, dtype=np.int32)
    out["key"] = np.zeros(capacity, dtype=np.int32)
    return out


def empty_particles(capacity: int) -> Dict[str, np.ndarray]:
    """Particle SoA as the reference allocates it (status 2, src/main.cpp:326-331)."""
    arrays = {name: np.zeros(capacity, dtype=np.float64) for name in PARTICLE_FIELDS[:7]}
    arrays["status"] = np.full(capacity, 2, dtype=np.int32)
    arrays["level"] = np.zeros(capacity, dtype=np.int32)
    return arrays


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return ORACLE_SO


class Oracle:
    """The C restatement (oracle/kpt_oracle.c).  libm_pow: the build on the C
    library's pow (the timed CPU baseline) instead of the project pow (the
    parity checker)."""

    def __init__(self, path: str = ORACLE_SO, libm_pow: bool = False):
        if libm_pow and path == ORACLE_SO:
            path = ORACLE_LIBM_SO
        if not os.path.exists(path):
            build_oracle()
        lib = ctypes.CDLL(path)
        self.lib = lib
        vp, dbl, u64, u32, i32 = (ctypes.c_void_p, ctypes.c_double, ctypes.c_uint64,
                                  ctypes.c_uint32, ctypes.c_int)
        lib.kpt_oracle_last_error.restype = ctypes.c_char_p
        lib.kpt_oracle_grid_init.argtypes = [vp, i32, i32, vp, vp, i32]
        lib.kpt_oracle_grid_free.argtypes = [vp]
        lib.kpt_oracle_table_from_cells.argtypes = [i32, i32, vp, vp, vp, vp, i32, i32, vp]
        lib.kpt_oracle_push.argtypes = [vp, vp, vp, vp, dbl, u32, u64, ctypes.c_size_t] + \
            [vp] * 8 + [i32]
        lib.kpt_oracle_inject.restype = u64
        lib.kpt_oracle_inject.argtypes = [vp, vp, dbl, u32, u64, u64, u64, u64, dbl, dbl] + \
            [vp] * 9
        lib.kpt_oracle_split.restype = u64
        lib.kpt_oracle_split.argtypes = [vp, u64, u64] + [vp] * 9 + [vp, vp]
        lib.kpt_oracle_histogram.argtypes = [dbl, dbl, i32, u64, vp, vp, vp, vp]
        lib.kpt_oracle_summarize.argtypes = [u64, vp, vp, vp, vp, vp, vp]
        lib.kpt_oracle_wrap.restype = dbl
        lib.kpt_oracle_wrap.argtypes = [dbl, dbl, dbl, dbl]
        lib.kpt_oracle_pow_array.argtypes = [u64, vp, vp, vp]
        lib.kpt_oracle_sample.argtypes = [vp, vp, vp, i32, dbl, dbl, dbl, i32, vp]
        lib.kpt_oracle_qlt_dmumu.restype = dbl
        lib.kpt_oracle_qlt_dmumu.argtypes = [dbl] * 7
        lib.kpt_oracle_qlt_dmumu_dmu.restype = dbl
        lib.kpt_oracle_qlt_dmumu_dmu.argtypes = [dbl] * 7

    def _error(self) -> str:
        return self.lib.kpt_oracle_last_error().decode()

    def grid(self, x_edges, y_edges, force_stored: bool = False) -> OracleGrid:
        grid = OracleGrid()
        xe = np.ascontiguousarray(x_edges, dtype=np.float64)
        ye = np.ascontiguousarray(y_edges, dtype=np.float64)
        if self.lib.kpt_oracle_grid_init(ctypes.byref(grid), xe.size - 1, ye.size - 1, _ptr(xe),
                                         _ptr(ye), int(force_stored)) != 0:
            raise ValueError(self._error())
        return grid

    def free_grid(self, grid: OracleGrid) -> None:
        self.lib.kpt_oracle_grid_free(ctypes.byref(grid))

    def table(self, field, focused: bool = False, force_stored: bool = False) -> np.ndarray:
        """Coefficient table (points, 16|21) for a fields.CompactField."""
        ncomp = 21 if focused else 16
        nx, ny = field.nx, field.ny
        out = np.zeros(((nx + 4) * (ny + 4), ncomp), dtype=np.float64)
        b = np.ascontiguousarray(field.b, dtype=np.float64)
        v = np.ascontiguousarray(field.v, dtype=np.float64)
        xe = np.ascontiguousarray(field.x_edges, dtype=np.float64)
        ye = np.ascontiguousarray(field.y_edges, dtype=np.float64)
        if self.lib.kpt_oracle_table_from_cells(nx, ny, _ptr(xe), _ptr(ye), _ptr(b), _ptr(v),
                                                int(focused), int(force_stored),
                                                _ptr(out)) != 0:
            raise ValueError(self._error())
        return out

    def push(self, grid: OracleGrid, lower: np.ndarray, upper: np.ndarray, params: dict,
             interval_start: float, frame: int, seed: int, count: int,
             particles: Dict[str, np.ndarray], threads: int = 0) -> np.ndarray:
        """In-place interval push; returns per-particle substep counts (uint32)."""
        steps = np.zeros(max(count, 1), dtype=np.uint32)
        prm = make_params(params)
        lo = np.ascontiguousarray(lower, dtype=np.float64)
        up = np.ascontiguousarray(upper, dtype=np.float64)
        self.lib.kpt_oracle_push(ctypes.byref(grid), _ptr(lo), _ptr(up), ctypes.byref(prm),
                                 float(interval_start), int(frame), int(seed), int(count),
                                 _ptr(particles["x"]), _ptr(particles["y"]),
                                 _ptr(particles["p"]), _ptr(particles["t"]),
                                 _ptr(particles["dt"]), _ptr(particles["mu"]),
                                 _ptr(particles["status"]), _ptr(steps), int(threads))
        return steps[:count]

    def inject(self, grid: OracleGrid, params: dict, interval_start: float, frame: int,
               seed: int, capacity: int, count: int, requested: int,
               particles: Dict[str, np.ndarray], band=(0.0, 0.0)) -> int:
        prm = make_params(params)
        return int(self.lib.kpt_oracle_inject(ctypes.byref(grid), ctypes.byref(prm),
                                              float(interval_start), int(frame), int(seed),
                                              int(capacity), int(count), int(requested),
                                              float(band[0]), float(band[1]),
                                              *[_ptr(particles[k]) for k in PARTICLE_FIELDS]))

    def split(self, params: dict, capacity: int, count: int, particles: Dict[str, np.ndarray]):
        prm = make_params(params)
        split = ctypes.c_uint64()
        skipped = ctypes.c_uint64()
        new_count = self.lib.kpt_oracle_split(ctypes.byref(prm), int(capacity), int(count),
                                              *[_ptr(particles[k]) for k in PARTICLE_FIELDS],
                                              ctypes.byref(split), ctypes.byref(skipped))
        return int(new_count), int(split.value), int(skipped.value)

    def histogram(self, pmin: float, pmax: float, nbins: int, count: int,
                  particles: Dict[str, np.ndarray]) -> np.ndarray:
        bins = np.zeros(nbins, dtype=np.float64)
        self.lib.kpt_oracle_histogram(float(pmin), float(pmax), int(nbins), int(count),
                                      _ptr(particles["p"]), _ptr(particles["w"]),
                                      _ptr(particles["status"]), _ptr(bins))
        return bins

    def summarize(self, count: int, particles: Dict[str, np.ndarray]) -> dict:
        out = OracleSummary()
        self.lib.kpt_oracle_summarize(int(count), _ptr(particles["p"]), _ptr(particles["dt"]),
                                      _ptr(particles["w"]), _ptr(particles["status"]),
                                      _ptr(particles["level"]), ctypes.byref(out))
        return {name: getattr(out, name) for name, _ in OracleSummary._fields_ if name != "pad"}

    def qlt(self, mu, omega, speed, sigma2, lc, gk, h0):
        """D_mumu and dD_mumu/dmu (LegencyModel.hpp:557-645) for arrays of inputs."""
        args = np.broadcast_arrays(*[np.asarray(a, dtype=np.float64)
                                     for a in (mu, omega, speed, sigma2, lc, gk, h0)])
        d = np.empty(args[0].shape)
        dd = np.empty(args[0].shape)
        for k in np.ndindex(args[0].shape):
            m, om, sp, s2, l, g, h = (float(a[k]) for a in args)
            d[k] = self.lib.kpt_oracle_qlt_dmumu(m, om, sp, s2, l, g, h)
            dd[k] = self.lib.kpt_oracle_qlt_dmumu_dmu(m, d[k], om, sp, l, g, h)
        return d, dd

    def wrap(self, value: float, lower: float, upper: float, width: float) -> float:
        return float(self.lib.kpt_oracle_wrap(value, lower, upper, width))

    def pow(self, x, y) -> np.ndarray:
        """The project pow (kpt_pow.h) on the host, elementwise."""
        x, y = np.broadcast_arrays(np.asarray(x, dtype=np.float64),
                                   np.asarray(y, dtype=np.float64))
        x, y = np.ascontiguousarray(x).ravel(), np.ascontiguousarray(y).ravel()
        out = np.empty_like(x)
        self.lib.kpt_oracle_pow_array(ctypes.c_uint64(x.size), _ptr(x), _ptr(y), _ptr(out))
        return out


class ReferenceHarness:
    """The reference's own driver functions on the Kokkos-API shim (oracle/_ref)."""

    def __init__(self, path: str = REF_SO, libm_pow: bool = False):
        if libm_pow and path == REF_SO:
            path = REF_LIBM_SO
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(path)
        self.lib = lib
        vp, cp, i32, ull, dbl, ll = (ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int,
                                     ctypes.c_ulonglong, ctypes.c_double, ctypes.c_longlong)
        lib.ref_last_error.restype = ctypes.c_char_p
        lib.ref_last_move_seconds.restype = ctypes.c_double
        lib.ref_table.restype = ll
        lib.ref_table.argtypes = [cp, i32, vp, ll]
        lib.ref_inject.restype = ll
        lib.ref_inject.argtypes = [cp, vp, vp, ull, i32, ull, ull, ull, dbl, dbl] + [vp] * 9
        lib.ref_push.restype = ll
        lib.ref_push.argtypes = [cp, vp, vp, ull, i32, ull, ull] + [vp] * 9
        lib.ref_split.restype = ll
        lib.ref_split.argtypes = [cp, vp, vp, i32, ull, ull] + [vp] * 9 + [vp, vp]
        lib.ref_table_stored.restype = ll
        lib.ref_table_stored.argtypes = [i32, i32, vp, vp, vp, vp, i32, vp, ll]
        lib.ref_push_stored.restype = ll
        lib.ref_push_stored.argtypes = [i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, ull, i32, ull,
                                        ull] + [vp] * 9
        lib.ref_qlt.restype = ll
        lib.ref_qlt.argtypes = [ll] + [vp] * 9
        lib.ref_main.restype = i32
        lib.ref_main.argtypes = [i32, ctypes.POINTER(ctypes.c_char_p), i32]
        lib.ref_lib_parker.restype = ll
        lib.ref_lib_parker.argtypes = [i32, i32, vp, vp, vp, vp, i32, vp, ull, i32, i32, i32, ll,
                                       ll, vp, vp, vp, vp, vp]
        lib.ref_lib_focus.restype = ll
        lib.ref_lib_focus.argtypes = [i32, i32, vp, vp, vp, vp, i32, vp, vp, ull, i32, i32, i32,
                                      ll, ll, vp, vp, vp, vp, vp]
        lib.ref_lib_system.restype = ll
        lib.ref_lib_system.argtypes = [i32, i32, vp, vp, vp, vp, i32, i32, i32, ll, ll, vp, vp,
                                       vp, vp]
        lib.ref_lib_generator.restype = ll
        lib.ref_lib_generator.argtypes = [i32, i32, vp, vp, vp, vp, i32, i32, vp, vp, vp, vp, vp,
                                          vp, i32, ull, ctypes.c_uint, ll, ll, vp, vp, vp, vp]
        lib.ref_lib_parker_coefficients.restype = ll
        lib.ref_lib_parker_coefficients.argtypes = [i32, i32, vp, vp, vp, vp, vp, i32, vp, vp,
                                                    vp, vp, dbl, i32, vp]
        lib.ref_lib_focus_coefficients.restype = ll
        lib.ref_lib_focus_coefficients.argtypes = [i32, i32, vp, vp, vp, vp, vp, vp, i32, vp, vp,
                                                   vp, vp, dbl, i32, vp]
        lib.ref_lib_candidates.restype = ll
        lib.ref_lib_candidates.argtypes = [i32, i32, vp, vp, vp, i32, i32, vp, vp, vp, vp, vp,
                                           vp, ll, vp]
        lib.ref_set_lib_stored_faces.restype = None
        lib.ref_set_lib_stored_faces.argtypes = [vp, vp]
        self._faces_alive = None

    def _lib_grid(self, grid: dict) -> None:
        """Select the grid of the library call that follows: a stored grid
        (StoredCoordinateGrid) when `grid` carries x_faces / y_faces (n + 5
        faces each, face -2 first; x_edges / y_edges are then the physical
        faces), else the analytic grid on the uniform x_edges / y_edges."""
        if "x_faces" in grid:
            xf = np.ascontiguousarray(grid["x_faces"], dtype=np.float64)
            yf = np.ascontiguousarray(grid["y_faces"], dtype=np.float64)
            self._faces_alive = (xf, yf)
            self.lib.ref_set_lib_stored_faces(_ptr(xf), _ptr(yf))
        else:
            self._faces_alive = None
            self.lib.ref_set_lib_stored_faces(None, None)

    @staticmethod
    def _param_arrays(params: dict):
        d = np.array([float(params[k]) for k in DOUBLE_PARAMS], dtype=np.float64)
        i = np.array([int(params[k]) for k in INT_PARAMS], dtype=np.int32)
        return d, i

    def _check(self, value):
        if value < 0:
            raise RuntimeError(self.lib.ref_last_error().decode())
        return value

    def table(self, path: str, focused: bool = False) -> np.ndarray:
        n = self._check(self.lib.ref_table(path.encode(), int(focused), None, 0))
        out = np.zeros(n, dtype=np.float64)
        self._check(self.lib.ref_table(path.encode(), int(focused), _ptr(out), n))
        return out.reshape(-1, 21 if focused else 16)

    def inject(self, field_dir: str, params: dict, seed: int, frame: int, capacity: int,
               count: int, requested: int, particles, band=(0.0, 0.0)) -> int:
        d, i = self._param_arrays(params)
        return int(self._check(self.lib.ref_inject(
            field_dir.encode(), _ptr(d), _ptr(i), seed, frame, capacity, count, requested,
            float(band[0]), float(band[1]), *[_ptr(particles[k]) for k in PARTICLE_FIELDS])))

    def push(self, field_dir: str, params: dict, seed: int, frame: int, capacity: int,
             count: int, particles) -> int:
        d, i = self._param_arrays(params)
        return int(self._check(self.lib.ref_push(
            field_dir.encode(), _ptr(d), _ptr(i), seed, frame, capacity, count,
            *[_ptr(particles[k]) for k in PARTICLE_FIELDS])))

    def last_move_seconds(self) -> float:
        """Seconds the last push spent in the interval push alone (the
        driver's move_seconds)."""
        return float(self.lib.ref_last_move_seconds())

    def split(self, field_dir: str, params: dict, frame: int, capacity: int, count: int,
              particles):
        d, i = self._param_arrays(params)
        split = ctypes.c_ulonglong()
        skipped = ctypes.c_ulonglong()
        new_count = self._check(self.lib.ref_split(
            field_dir.encode(), _ptr(d), _ptr(i), frame, capacity, count,
            *[_ptr(particles[k]) for k in PARTICLE_FIELDS], ctypes.byref(split),
            ctypes.byref(skipped)))
        return int(new_count), int(split.value), int(skipped.value)

    def table_stored(self, field, focused: bool = False) -> np.ndarray:
        """Coefficient table of a fields.CompactField on the stored-edge grid path."""
        xe = np.ascontiguousarray(field.x_edges, dtype=np.float64)
        ye = np.ascontiguousarray(field.y_edges, dtype=np.float64)
        b = np.ascontiguousarray(field.b, dtype=np.float64)
        v = np.ascontiguousarray(field.v, dtype=np.float64)
        args = (field.nx, field.ny, _ptr(xe), _ptr(ye), _ptr(b), _ptr(v), int(focused))
        n = self._check(self.lib.ref_table_stored(*args, None, 0))
        out = np.zeros(n, dtype=np.float64)
        self._check(self.lib.ref_table_stored(*args, _ptr(out), n))
        return out.reshape(-1, 21 if focused else 16)

    def push_stored(self, lower_field, upper_field, params: dict, seed: int, frame: int,
                    capacity: int, count: int, particles) -> int:
        d, i = self._param_arrays(params)
        xe = np.ascontiguousarray(lower_field.x_edges, dtype=np.float64)
        ye = np.ascontiguousarray(lower_field.y_edges, dtype=np.float64)
        arrays = [np.ascontiguousarray(a, dtype=np.float64) for a in
                  (lower_field.b, lower_field.v, upper_field.b, upper_field.v)]
        return int(self._check(self.lib.ref_push_stored(
            lower_field.nx, lower_field.ny, _ptr(xe), _ptr(ye), *[_ptr(a) for a in arrays],
            _ptr(d), _ptr(i), seed, frame, capacity, count,
            *[_ptr(particles[k]) for k in PARTICLE_FIELDS])))

    def qlt(self, mu, omega, speed, sigma2, lc, gk, h0):
        """The reference's own LegencyModel D_mumu and dD_mumu/dmu."""
        args = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a in
                np.broadcast_arrays(mu, omega, speed, sigma2, lc, gk, h0)]
        n = args[0].size
        d = np.empty(n)
        dd = np.empty(n)
        self._check(self.lib.ref_qlt(n, *[_ptr(a) for a in args], _ptr(d), _ptr(dd)))
        return d, dd

    @staticmethod
    def _lib_blocks(system: Dict[str, np.ndarray]):
        ids = np.ascontiguousarray(system["id"], dtype=np.uint64)
        d = np.ascontiguousarray(np.stack([system[k] for k in LIB_DOUBLE_FIELDS]),
                                 dtype=np.float64)
        i = np.ascontiguousarray(np.stack([system[k] for k in LIB_INT_FIELDS]), dtype=np.int32)
        return ids, d, i

    @staticmethod
    def _lib_unblock(system, ids, d, i):
        system["id"][:] = ids
        for k, name in enumerate(LIB_DOUBLE_FIELDS):
            system[name][:] = d[k]
        for k, name in enumerate(LIB_INT_FIELDS):
            system[name][:] = i[k]

    def lib_parker(self, grid: dict, basis: np.ndarray, constant_ratio: bool, props: dict,
                   seed: int, first_step: int, steps: int, stochastic: bool, count: int,
                   system: Dict[str, np.ndarray], normals=None) -> np.ndarray:
        """ParkerSolver steps (include/ParkerSolver.hpp) on a uniform Cartesian grid;
        updates `system` in place and returns the dt of each step.  normals
        ([steps][4][count], optional) replaces the keyed stream's normals."""
        self._lib_grid(grid)
        xe = np.ascontiguousarray(grid["x_edges"], dtype=np.float64)
        ye = np.ascontiguousarray(grid["y_edges"], dtype=np.float64)
        periodic = np.ascontiguousarray(grid["periodic"], dtype=np.int32)
        basis = np.ascontiguousarray(basis, dtype=np.float64)
        pr = np.array([props["rest_mass"], props["charge"], props["speed_of_light"],
                       props.get("energy_scale", 1.0), props["courant"]], dtype=np.float64)
        ids, d, i = self._lib_blocks(system)
        dts = np.zeros(max(1, steps), dtype=np.float64)
        self._check(self.lib.ref_lib_parker(
            len(xe) - 1, len(ye) - 1, _ptr(xe), _ptr(ye), _ptr(periodic), _ptr(basis),
            int(constant_ratio), _ptr(pr), seed, first_step, steps, 0 if stochastic else 1,
            count, ids.size, _ptr(ids), _ptr(d), _ptr(i), _ptr(dts),
            None if normals is None else _ptr(np.ascontiguousarray(normals, dtype=np.float64))))
        self._lib_unblock(system, ids, d, i)
        return dts[:steps]

    def lib_focus(self, grid: dict, basis: np.ndarray, constant_ratio: bool, props: dict,
                  scattering: dict, seed: int, first_step: int, steps: int, stochastic: bool,
                  count: int, system: Dict[str, np.ndarray], normals=None) -> np.ndarray:
        """FocusTransportSolver steps (include/FocusSolver.hpp) on a uniform Cartesian
        grid; updates `system` in place and returns the dt of each step.  normals
        ([steps][4][count], optional) replaces the keyed stream's normals."""
        self._lib_grid(grid)
        xe = np.ascontiguousarray(grid["x_edges"], dtype=np.float64)
        ye = np.ascontiguousarray(grid["y_edges"], dtype=np.float64)
        periodic = np.ascontiguousarray(grid["periodic"], dtype=np.int32)
        basis = np.ascontiguousarray(basis, dtype=np.float64)
        pr = np.array([props["rest_mass"], props["charge"], props["speed_of_light"],
                       props.get("energy_scale", 1.0), props["courant"]], dtype=np.float64)
        sc = np.array([scattering["spectral_index"], scattering["h0"],
                       scattering.get("min_b", 0.0), scattering.get("min_sigma2", 0.0),
                       scattering.get("min_lc", 0.0), scattering.get("min_speed", 0.0),
                       scattering.get("max_mu", 1.0)], dtype=np.float64)
        ids, d, i = self._lib_blocks(system)
        dts = np.zeros(max(1, steps), dtype=np.float64)
        self._check(self.lib.ref_lib_focus(
            len(xe) - 1, len(ye) - 1, _ptr(xe), _ptr(ye), _ptr(periodic), _ptr(basis),
            int(constant_ratio), _ptr(pr), _ptr(sc), seed, first_step, steps,
            0 if stochastic else 1, count, ids.size, _ptr(ids), _ptr(d), _ptr(i), _ptr(dts),
            None if normals is None else _ptr(np.ascontiguousarray(normals, dtype=np.float64))))
        self._lib_unblock(system, ids, d, i)
        return dts[:steps]

    def lib_system(self, grid: dict, props: dict, op: str, count: int,
                   system: Dict[str, np.ndarray], key_range=(0, 0)):
        """One ParticleSystem lifecycle call; returns (count after, split statistics)."""
        self._lib_grid(grid)
        ops = {"boundary": 0, "sort": 1, "compact": 2, "split": 3, "capture": 4}
        xe = np.ascontiguousarray(grid["x_edges"], dtype=np.float64)
        ye = np.ascontiguousarray(grid["y_edges"], dtype=np.float64)
        periodic = np.ascontiguousarray(grid["periodic"], dtype=np.int32)
        pr = np.array([props["rest_mass"], props["charge"], props["speed_of_light"],
                       props.get("energy_scale", 1.0), props.get("courant", 0.3),
                       props.get("split_ratio", 2.0), props.get("min_child_weight", 0.0)],
                      dtype=np.float64)
        ids, d, i = self._lib_blocks(system)
        stats = np.zeros(6, dtype=np.uint64)
        self._check(self.lib.ref_lib_system(
            len(xe) - 1, len(ye) - 1, _ptr(xe), _ptr(ye), _ptr(periodic), _ptr(pr), ops[op],
            int(key_range[0]), int(key_range[1]), count, ids.size, _ptr(ids), _ptr(d), _ptr(i),
            _ptr(stats)))
        self._lib_unblock(system, ids, d, i)
        return int(stats[0]), [int(v) for v in stats[1:]]

    # ParticleGenerator (include/ParticleGenerator.hpp): the reference's own
    # templates on the library grid, noise frame `frame`.
    GENERATOR_OPS = {"inject_uniform": 0, "inject_uniform_if": 1, "inject_where_field": 2,
                     "inject_in_grid": 3, "recycle_uniform": 4, "recycle_uniform_if": 5,
                     "recycle_where_field": 6, "recycle_in_grid": 7}

    @staticmethod
    def _generator_inputs(grid, field, centering, region, predicate):
        xe = np.ascontiguousarray(grid["x_edges"], dtype=np.float64)
        ye = np.ascontiguousarray(grid["y_edges"], dtype=np.float64)
        periodic = np.ascontiguousarray(grid["periodic"], dtype=np.int32)
        values = np.ascontiguousarray(field, dtype=np.float64)
        components = 1 if values.ndim == 1 else values.shape[1]
        cent = np.ascontiguousarray(centering, dtype=np.int32)
        reg = None if region is None else np.ascontiguousarray(region, dtype=np.float64)
        pred = np.array([predicate.get("threshold", 0.0), predicate.get("comparison", 1),
                         predicate.get("component", 0), predicate.get("domain", 0)],
                        dtype=np.float64)
        return xe, ye, periodic, values, components, cent, reg, pred

    def lib_generator(self, grid: dict, props: dict, op: str, count: int,
                      system: Dict[str, np.ndarray], *, field, centering=(0, 0), region=None,
                      predicate=None, kinematics=(1.0, 0.0, 1.0, 0), plan=(0, 0, 0, 64),
                      selection: int = 0, seed: int = 114514, frame: int = 0) -> int:
        """One injection or recycling call; returns the particle count after it."""
        self._lib_grid(grid)
        xe, ye, periodic, values, components, cent, reg, pred = self._generator_inputs(
            grid, field, centering, region, predicate or {})
        pr = np.array([props["rest_mass"], props["charge"], props["speed_of_light"],
                       props.get("energy_scale", 1.0)], dtype=np.float64)
        kin = np.ascontiguousarray(kinematics, dtype=np.float64)
        pl = np.ascontiguousarray(plan, dtype=np.uint64)
        ids, d, i = self._lib_blocks(system)
        out_count = np.zeros(1, dtype=np.uint64)
        self._check(self.lib.ref_lib_generator(
            len(xe) - 1, len(ye) - 1, _ptr(xe), _ptr(ye), _ptr(periodic), _ptr(pr),
            self.GENERATOR_OPS[op], components, _ptr(cent), _ptr(values),
            None if reg is None else _ptr(reg), _ptr(pred), _ptr(kin), _ptr(pl), int(selection),
            ctypes.c_ulonglong(seed), ctypes.c_uint(frame), count, ids.size, _ptr(ids), _ptr(d),
            _ptr(i), _ptr(out_count)))
        self._lib_unblock(system, ids, d, i)
        return int(out_count[0])

    def lib_candidates(self, grid: dict, kind: str, *, field=None, centering=(0, 0),
                       region=None, predicate=None):
        """Candidate set: kind "field" or "grid"; returns (indices, cumulative weights, total)."""
        self._lib_grid(grid)
        if field is None:
            field = np.zeros(1)
        xe, ye, periodic, values, components, cent, reg, pred = self._generator_inputs(
            grid, field, centering, region, predicate or {})
        cells = (len(xe) + 3) * (len(ye) + 3)
        max_out = max(cells, values.shape[0])
        idx = np.zeros(max_out, dtype=np.uint64)
        cum = np.zeros(max_out, dtype=np.float64)
        total = np.zeros(1, dtype=np.float64)
        n = self.lib.ref_lib_candidates(
            len(xe) - 1, len(ye) - 1, _ptr(xe), _ptr(ye), _ptr(periodic),
            0 if kind == "field" else 1, components, _ptr(cent), _ptr(values),
            None if reg is None else _ptr(reg), _ptr(pred), _ptr(idx), _ptr(cum), max_out,
            _ptr(total))
        self._check(0 if n >= 0 else -1)
        return idx[:n].copy(), cum[:n].copy(), float(total[0])

    def lib_parker_coefficients(self, grid: dict, b, v, *, turbulence=(0.5, 1.0, 1.0, -1.0),
                                turbulence_fields=None, props=None, params=None,
                                drift_floor: float = 0.0, ghost_mode: int = 0) -> np.ndarray:
        """The reference's Parker coefficient precompute and packed basis
        (points x 18) from cell-centred B and V (points x 3, ghosts as given)."""
        self._lib_grid(grid)
        xe = np.ascontiguousarray(grid["x_edges"], dtype=np.float64)
        ye = np.ascontiguousarray(grid["y_edges"], dtype=np.float64)
        periodic = np.ascontiguousarray(grid["periodic"], dtype=np.int32)
        b = np.ascontiguousarray(b, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        points = b.shape[0]
        props = props or dict(rest_mass=1.0, charge=1.0, speed_of_light=1.0)
        pr = np.array([props["rest_mass"], props["charge"], props["speed_of_light"],
                       props.get("energy_scale", 1.0)], dtype=np.float64)
        params = params or {}
        pa = np.array([params.get("model", 0), params.get("parallel_prefactor", 1.622),
                       params.get("perpendicular_prefactor", 0.198), params.get("ratio", 0.0),
                       params.get("minimum_b", 0.0), params.get("minimum_vsw", 0.0),
                       params.get("minimum_sigma2", 0.0)], dtype=np.float64)
        turb = np.ascontiguousarray(turbulence, dtype=np.float64)
        fields = None
        if turbulence_fields is not None:
            fields = np.ascontiguousarray(np.stack(turbulence_fields), dtype=np.float64)
        out = np.zeros((points, 18), dtype=np.float64)
        self._check(self.lib.ref_lib_parker_coefficients(
            len(xe) - 1, len(ye) - 1, _ptr(xe), _ptr(ye), _ptr(periodic), _ptr(b), _ptr(v),
            0 if fields is None else 1, _ptr(turb), None if fields is None else _ptr(fields),
            _ptr(pr), _ptr(pa), float(drift_floor), int(ghost_mode), _ptr(out)))
        return out

    def lib_focus_coefficients(self, grid: dict, b, v, dvdt=None, *,
                               turbulence=(0.5, 1.0, 1.0, -1.0), turbulence_fields=None,
                               props=None, params=None, builder_floor: float = 0.0,
                               ghost_mode: int = 0) -> np.ndarray:
        """The reference's focused coefficient precompute and packed basis
        (points x 27) from cell-centred B, V and dV/dt (points x 3)."""
        self._lib_grid(grid)
        xe = np.ascontiguousarray(grid["x_edges"], dtype=np.float64)
        ye = np.ascontiguousarray(grid["y_edges"], dtype=np.float64)
        periodic = np.ascontiguousarray(grid["periodic"], dtype=np.int32)
        b = np.ascontiguousarray(b, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        dv = None if dvdt is None else np.ascontiguousarray(dvdt, dtype=np.float64)
        points = b.shape[0]
        props = props or dict(rest_mass=1.0, charge=1.0, speed_of_light=1.0)
        pr = np.array([props["rest_mass"], props["charge"], props["speed_of_light"],
                       props.get("energy_scale", 1.0)], dtype=np.float64)
        params = params or {}
        pa = np.array([params.get("model", 0), params.get("parallel_prefactor", 1.622),
                       params.get("perpendicular_prefactor", 0.198), params.get("ratio", 0.0),
                       params.get("minimum_b", 0.0), params.get("minimum_vsw", 0.0),
                       params.get("minimum_sigma2", 0.0)], dtype=np.float64)
        turb = np.ascontiguousarray(turbulence, dtype=np.float64)
        fields = None
        if turbulence_fields is not None:
            fields = np.ascontiguousarray(np.stack(turbulence_fields), dtype=np.float64)
        out = np.zeros((points, 27), dtype=np.float64)
        self._check(self.lib.ref_lib_focus_coefficients(
            len(xe) - 1, len(ye) - 1, _ptr(xe), _ptr(ye), _ptr(periodic), _ptr(b), _ptr(v),
            None if dv is None else _ptr(dv), 0 if fields is None else 1, _ptr(turb),
            None if fields is None else _ptr(fields), _ptr(pr), _ptr(pa), float(builder_floor),
            int(ghost_mode), _ptr(out)))
        return out

    def main(self, argv, frame_base: int = 0) -> int:
        """Run the reference CLI (in-process); noise frames start at frame_base."""
        args = [b"kokkos_particle_transport_app"] + [a.encode() for a in argv]
        arr = (ctypes.c_char_p * len(args))(*args)
        return int(self.lib.ref_main(len(args), arr, int(frame_base)))
