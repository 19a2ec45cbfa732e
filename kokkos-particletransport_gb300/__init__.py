"""GB300-native Parker / focused-transport particle push — Python binding.

A thin ctypes layer over ``lib/libkpt.so`` (the C ABI declared in
``include/kpt.h``).  It mirrors the reference driver's objects: a coefficient
``Field`` per MHD frame (reference ``Field<Grid,16|21>`` built by
``load_*_coefficient_frame``), a ``ParticleStorage`` (reference
``ReconnectionParticleStorage``) and the per-frame operations ``inject``,
``push_interval``, ``split``, ``histogram`` and ``summarize``.

There is no CPU path: importing works without a GPU, but creating a
``Context`` raises ``KptError`` when no CUDA device or no built library is
available.
"""
from __future__ import annotations

import ctypes
import os
import weakref
from typing import Dict, Optional, Sequence

import numpy as np

from . import fields  # noqa: F401  (re-exported module)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libkpt.so")
HEADER_PATH = os.path.join(os.path.dirname(HERE), "include", "kpt.h")

TABLE_PARKER16 = 0
TABLE_FOCUSED21 = 1
PRECISION_F64 = 0
PRECISION_MIXED = 1
SCHEDULE_REFILL = 0
SCHEDULE_SIMPLE = 1
FP64_STRICT = 0       # FP64 push rounds as the reference's code is written (oracle-exact)
FP64_CONTRACTED = 1   # FP64 push with FMA contraction and CUDA's pow (faster)
RECORDS_AUTO = 0      # mixed pushes sample cell records when the population is dense enough
RECORDS_OFF = 1       # mixed pushes sample the point-major tables
RECORDS_ON = 2        # every refill-scheduled mixed push samples cell records
ENGINE_TCGEN05 = 0   # block-collective tcgen05.mma network, activations in tensor memory
ENGINE_MMA_SYNC = 1  # warp-collective mma.sync network, activations in registers

PARTICLE_FIELDS = ("x", "y", "p", "t", "dt", "w", "mu", "status", "level")
DOUBLE_SETTINGS = ("mhd_dt", "p0", "pmin", "pmax", "gamma_turb", "kpara0", "kperp_over_kpara",
                   "dt_min_rel", "dt_max_rel", "drift_param1", "drift_param2", "charge",
                   "particle_v0", "duu0", "split_ratio", "pmin_split_over_p0", "mu_max")
INT_SETTINGS = ("max_steps", "momentum_dependency", "magnetic_dependency", "time_interpolation",
                "split_particles", "focused")
CLOSURE_INT = ("closure",)
CLOSURE_DOUBLE = ("qlt_sigma2", "qlt_spectral_index", "qlt_h0", "qlt_omega0", "qlt_lc")
CLOSURE_DRIVER = 0
CLOSURE_QLT = 1
CLOSURE_SURROGATE = 2
SURROGATE_BF16 = 0
SURROGATE_FP16 = 1


class KptError(RuntimeError):
    """A libkpt call failed (message from kpt_last_error)."""


class Settings(ctypes.Structure):
    """kpt_settings: the reference Reconnection2DSettings physics block."""
    _fields_ = [(n, ctypes.c_double) for n in DOUBLE_SETTINGS] + \
               [(n, ctypes.c_int32) for n in INT_SETTINGS + CLOSURE_INT] + \
               [(n, ctypes.c_double) for n in CLOSURE_DOUBLE]

    def as_dict(self) -> Dict[str, float]:
        return {name: getattr(self, name) for name, _ in self._fields_}


class PushStats(ctypes.Structure):
    _fields_ = [("particle_steps", ctypes.c_uint64), ("pushed", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("max_steps", ctypes.c_uint32),
                ("pad", ctypes.c_uint32)]


class Summary(ctypes.Structure):
    _fields_ = [("stored", ctypes.c_uint64), ("active", ctypes.c_uint64),
                ("inactive", ctypes.c_uint64), ("weight_sum", ctypes.c_double),
                ("p_min", ctypes.c_double), ("p_max", ctypes.c_double),
                ("p_avg", ctypes.c_double), ("dt_min", ctypes.c_double),
                ("dt_max", ctypes.c_double), ("dt_avg", ctypes.c_double),
                ("max_split_level", ctypes.c_int32), ("pad", ctypes.c_int32)]

    def as_dict(self) -> Dict[str, float]:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "pad"}


class SurrogateConfig(ctypes.Structure):
    """kpt_surrogate_config: training set, optimiser and training box."""
    _fields_ = [("samples", ctypes.c_int32), ("steps", ctypes.c_int32),
                ("batch", ctypes.c_int32), ("element_type", ctypes.c_int32),
                ("quantization_aware", ctypes.c_int32), ("hidden_width", ctypes.c_int32)] + \
               [(n, ctypes.c_double) for n in (
                   "learning_rate", "mu_cut", "mu_max", "p_lo_over_p0", "p_hi_over_p0",
                   "sigma2_lo", "sigma2_hi", "gk_lo", "gk_hi", "b_lo", "b_hi")] + \
               [("seed", ctypes.c_uint64)]


class ParticleProperties(ctypes.Structure):
    """kpt_particle_properties (reference ParticleProperties)."""
    _fields_ = [(n, ctypes.c_double) for n in ("rest_mass", "charge", "speed_of_light",
                                               "energy_scale_erg")]


class ScatteringParameters(ctypes.Structure):
    """kpt_scattering_parameters (reference PitchAngleScatteringParameters)."""
    _fields_ = [(n, ctypes.c_double) for n in (
        "spectral_index", "h0", "minimum_magnetic_field_magnitude", "minimum_sigma2",
        "minimum_correlation_length", "minimum_speed")]


class BatchTuning(ctypes.Structure):
    """kpt_batch_tuning: the schedule the autotuner chose."""
    _fields_ = [("sort_tile", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32),
                ("sort_every", ctypes.c_int32), ("candidates", ctypes.c_int32),
                ("best_ms", ctypes.c_float), ("spread", ctypes.c_float),
                ("threads_per_block", ctypes.c_int32), ("particles_per_lane", ctypes.c_int32),
                ("repeats", ctypes.c_int32), ("pad", ctypes.c_int32)]


class SplitPolicy(ctypes.Structure):
    """kpt_split_policy (reference ParticleSplittingPolicy)."""
    _fields_ = [("energy_split_ratio", ctypes.c_double),
                ("minimum_child_weight", ctypes.c_double)]


class SplitStatistics(ctypes.Structure):
    """kpt_split_statistics (reference ParticleSplitStatistics)."""
    _fields_ = [(n, ctypes.c_uint64) for n in ("active_count", "split_count",
                                               "skipped_capacity_count",
                                               "skipped_invalid_baseline_count",
                                               "skipped_minimum_weight_count")]


SYSTEM_DOUBLE_FIELDS = ("x", "y", "prev_x", "prev_y", "prevstep_x", "prevstep_y", "p", "mu",
                        "w", "e0")
SYSTEM_INT_FIELDS = ("status", "level", "key")


class SystemArrays(ctypes.Structure):
    """kpt_system_arrays: host pointers of the ParticleSystem storage."""
    _fields_ = [("id", ctypes.c_void_p)] + \
               [(n, ctypes.c_void_p) for n in ("x", "y", "prev_x", "prev_y", "prevstep_x",
                                               "prevstep_y", "p", "mu", "weight", "e0",
                                               "status", "split_level", "sort_key")]


class ParticleArrays(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("x", "y", "p", "t", "step_dt", "weight", "mu", "status", "split_level")]


_LIB: Optional[ctypes.CDLL] = None


class Turbulence(ctypes.Structure):
    """TurbulenceProperties for the coefficient precompute: storage 0 = the
    constant state (sigma2, l2d, lslab, lc; lc <= 0 = the slab length),
    storage 1 = per-point fields over the ghosted cells."""
    _fields_ = [("storage", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("sigma2", ctypes.c_double), ("l2d", ctypes.c_double),
                ("lslab", ctypes.c_double), ("lc", ctypes.c_double),
                ("sigma2_field", ctypes.c_void_p), ("l2d_field", ctypes.c_void_p),
                ("lslab_field", ctypes.c_void_p), ("lc_field", ctypes.c_void_p)]


class DiffusionParameters(ctypes.Structure):
    """LegencyModel::DiffusionModelParameters plus the drift floor and the
    ghost-fill mode of make_legacy_transport_coefficient_fields."""
    _fields_ = [("perpendicular_model", ctypes.c_int32), ("ghost_fill_mode", ctypes.c_int32),
                ("parallel_prefactor", ctypes.c_double),
                ("perpendicular_prefactor", ctypes.c_double),
                ("perpendicular_parallel_ratio", ctypes.c_double),
                ("minimum_magnetic_field_magnitude", ctypes.c_double),
                ("minimum_solar_wind_speed", ctypes.c_double),
                ("minimum_sigma2", ctypes.c_double),
                ("minimum_magnetic_field_squared_for_drift", ctypes.c_double)]


class Region(ctypes.Structure):
    """AxisAlignedParticleRegion<2> (ParticleGenerator.hpp:18-62)."""
    _fields_ = [("lower", ctypes.c_double * 2), ("upper", ctypes.c_double * 2)]


class ParticleInjectionKinematics(ctypes.Structure):
    """Constant state of injected particles (ParticleGenerator.hpp:68-74);
    status 0 active, 1 escaped, 2 inactive."""
    _fields_ = [("momentum_magnitude", ctypes.c_double), ("mu", ctypes.c_double),
                ("weight", ctypes.c_double), ("status", ctypes.c_int32),
                ("pad", ctypes.c_int32)]

    def __init__(self, momentum_magnitude=0.0, mu=0.0, weight=1.0, status=0):
        super().__init__(float(momentum_magnitude), float(mu), float(weight), int(status), 0)


class ParticleInjectionPlan(ctypes.Structure):
    """Injection range and rejection-sampling attempts (ParticleGenerator.hpp:107-112)."""
    _fields_ = [("first_particle_index", ctypes.c_uint64), ("particle_count", ctypes.c_uint64),
                ("first_particle_id", ctypes.c_uint64), ("max_attempts", ctypes.c_int32),
                ("pad", ctypes.c_int32)]


class _FieldPredicate(ctypes.Structure):
    _fields_ = [("field", ctypes.c_void_p), ("threshold", ctypes.c_double),
                ("comparison", ctypes.c_int32), ("component", ctypes.c_int32),
                ("domain", ctypes.c_int32), ("pad", ctypes.c_int32)]


def library_path() -> str:
    return LIB_PATH


def load_library() -> ctypes.CDLL:
    """Load libkpt.so (raises KptError if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise KptError(f"libkpt.so not built at {LIB_PATH}; run __graft_entry__.build()")
    lib = ctypes.CDLL(LIB_PATH)
    vp, i32, u32, u64, dbl = (ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64,
                              ctypes.c_double)
    pvp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "kpt_abi_version": (i32, []),
        "kpt_last_error": (ctypes.c_char_p, []),
        "kpt_default_settings": (None, [vp]),
        "kpt_context_create": (i32, [i32, pvp]),
        "kpt_context_destroy": (i32, [vp]),
        "kpt_context_set_stream": (i32, [vp, vp]),
        "kpt_context_synchronize": (i32, [vp]),
        "kpt_context_fp64_fma_rate": (i32, [vp, ctypes.POINTER(ctypes.c_double)]),
        "kpt_math_pow": (i32, [vp, ctypes.c_uint64, vp, vp, vp]),
        "kpt_context_set_fp64_arithmetic": (i32, [vp, i32]),
        "kpt_context_set_cell_records": (i32, [vp, i32]),
        "kpt_context_set_push_schedule": (i32, [vp, i32, i32]),
        "kpt_field_create": (i32, [vp, i32, i32, vp, vp, vp, vp, i32, i32, pvp]),
        "kpt_field_load": (i32, [vp, ctypes.c_char_p, i32, i32, pvp]),
        "kpt_field_destroy": (i32, [vp]),
        "kpt_field_shape": (i32, [vp, vp, vp, vp, vp]),
        "kpt_field_download_table": (i32, [vp, vp, u64]),
        "kpt_particles_create": (i32, [vp, u64, pvp]),
        "kpt_particles_destroy": (i32, [vp]),
        "kpt_particles_count": (i32, [vp, vp, vp]),
        "kpt_particles_set_count": (i32, [vp, u64]),
        "kpt_particles_upload": (i32, [vp, u64] + [vp] * 9),
        "kpt_particles_download": (i32, [vp, u64] + [vp] * 9),
        "kpt_particles_device_arrays": (i32, [vp, vp]),
        "kpt_inject_uniform": (i32, [vp, vp, vp, vp, u64, u32, u64, dbl, dbl, vp]),
        "kpt_push_interval": (i32, [vp, vp, vp, vp, vp, u32, u64, vp]),
        "kpt_split": (i32, [vp, vp, vp, vp, vp]),
        "kpt_histogram": (i32, [vp, vp, dbl, dbl, i32, vp]),
        "kpt_summarize": (i32, [vp, vp, vp]),
        "kpt_sample_table": (i32, [vp, vp, vp, u64, vp, vp, vp, i32, vp]),
        "kpt_particles_sort": (i32, [vp, vp, vp, i32, i32]),
        "kpt_particles_clear_order": (i32, [vp]),
        "kpt_particles_wrap": (i32, [vp, u64, u64, vp, pvp]),
        "kpt_particles_pack_records": (i32, [vp, vp, dbl, vp, u64]),
        "kpt_surrogate_default_config": (None, [vp]),
        "kpt_surrogate_train": (i32, [vp, vp, vp, pvp, vp]),
        "kpt_surrogate_destroy": (i32, [vp]),
        "kpt_surrogate_evaluate": (i32, [vp, u64, vp, i32, vp, vp]),
        "kpt_surrogate_parameters": (i32, [vp, vp, i32, vp, i32]),
        "kpt_surrogate_gradient": (i32, [vp, i32, vp, u64, vp, vp, vp, vp]),
        "kpt_surrogate_shape": (i32, [vp, vp, vp]),
        "kpt_surrogate_set_engine": (i32, [vp, i32]),
        "kpt_surrogate_get_engine": (i32, [vp, vp]),
        "kpt_surrogate_check_timeout": (i32, [vp, u32, u32, vp, vp]),
        "kpt_surrogate_pack_tc": (i32, [vp, i32, i32, vp, u64]),
        "kpt_context_set_surrogate": (i32, [vp, vp]),
        "kpt_surrogate_judge": (i32, [vp, vp, vp, vp, vp]),
        "kpt_grid_create": (i32, [vp, i32, i32, vp, vp, vp, pvp]),
        "kpt_grid_create_stored": (i32, [vp, i32, i32, vp, vp, vp, pvp]),
        "kpt_grid_destroy": (i32, [vp]),
        "kpt_system_create": (i32, [vp, u64, u64, vp, vp, pvp]),
        "kpt_system_destroy": (i32, [vp]),
        "kpt_system_count": (i32, [vp, vp, vp]),
        "kpt_system_set_count": (i32, [vp, u64]),
        "kpt_system_upload": (i32, [vp, u64, vp]),
        "kpt_system_download": (i32, [vp, u64, vp]),
        "kpt_system_capture_previous_positions": (i32, [vp, vp]),
        "kpt_system_apply_boundary": (i32, [vp, vp, vp]),
        "kpt_system_sort_by_key": (i32, [vp, vp, ctypes.c_int32, ctypes.c_int32]),
        "kpt_system_compact": (i32, [vp, vp, vp]),
        "kpt_system_split_energy": (i32, [vp, vp, vp]),
        "kpt_system_reset_split_baselines": (i32, [vp, vp]),
        "kpt_parker_solver_create": (i32, [vp, vp, vp, i32, dbl, pvp]),
        "kpt_parker_solver_destroy": (i32, [vp]),
        "kpt_parker_solver_set_basis": (i32, [vp, vp, i32]),
        "kpt_parker_solver_set_courant": (i32, [vp, dbl]),
        "kpt_parker_solver_set_precision": (i32, [vp, i32]),
        "kpt_parker_compute_time_step": (i32, [vp, vp, vp, vp]),
        "kpt_parker_advance_stochastic": (i32, [vp, vp, vp, u64, u32, vp]),
        "kpt_parker_advance_deterministic": (i32, [vp, vp, vp, vp]),
        "kpt_parker_advance_stochastic_steps": (i32, [vp, vp, vp, u64, u32, u32, vp]),
        "kpt_parker_advance_with_noise": (i32, [vp, vp, vp, vp, vp]),
        "kpt_batch_create": (i32, [vp, pvp]),
        "kpt_batch_destroy": (i32, [vp]),
        "kpt_batch_add_run": (i32, [vp, vp, vp, vp, vp, u64, u32, vp]),
        "kpt_batch_set_schedule": (i32, [vp, i32, i32, i32]),
        "kpt_batch_get_schedule": (i32, [vp, vp, vp, vp]),
        "kpt_batch_set_launch_shape": (i32, [vp, i32, i32]),
        "kpt_batch_get_launch_shape": (i32, [vp, vp, vp]),
        "kpt_batch_run": (i32, [vp, u32, i32]),
        "kpt_batch_stats": (i32, [vp, i32, vp]),
        "kpt_batch_frame": (i32, [vp, i32, vp]),
        "kpt_batch_set_frame": (i32, [vp, i32, u32]),
        "kpt_batch_autotune": (i32, [vp, u32, vp]),
        "kpt_focus_solver_create": (i32, [vp, vp, vp, i32, dbl, vp, pvp]),
        "kpt_focus_solver_destroy": (i32, [vp]),
        "kpt_focus_solver_set_basis": (i32, [vp, vp, i32]),
        "kpt_focus_solver_set_courant": (i32, [vp, dbl]),
        "kpt_focus_solver_set_precision": (i32, [vp, i32]),
        "kpt_focus_solver_set_maximum_mu": (i32, [vp, dbl]),
        "kpt_focus_compute_time_step": (i32, [vp, vp, vp, vp]),
        "kpt_focus_advance_stochastic": (i32, [vp, vp, vp, u64, u32, vp]),
        "kpt_focus_advance_deterministic": (i32, [vp, vp, vp, vp]),
        "kpt_focus_advance_stochastic_steps": (i32, [vp, vp, vp, u64, u32, u32, vp]),
        "kpt_focus_advance_with_noise": (i32, [vp, vp, vp, vp, vp]),
        "kpt_default_diffusion_parameters": (None, [vp]),
        "kpt_parker_coefficients": (i32, [vp, vp, vp, vp, vp, vp, vp, vp]),
        "kpt_parker_solver_create_from_fields": (i32, [vp, vp, vp, vp, vp, vp, vp, dbl, pvp]),
        "kpt_focus_coefficients": (i32, [vp, vp, vp, vp, vp, vp, vp, vp, dbl, vp]),
        "kpt_focus_solver_create_from_fields": (i32, [vp, vp, vp, vp, vp, vp, vp, vp, dbl, dbl,
                                                      vp, pvp]),
        "kpt_lib_field_create": (i32, [vp, vp, i32, vp, vp, pvp]),
        "kpt_lib_field_destroy": (i32, [vp]),
        "kpt_lib_field_points": (i32, [vp, vp]),
        "kpt_region_from_grid": (i32, [vp, i32, vp]),
        "kpt_candidates_from_field": (i32, [vp, vp, vp, dbl, i32, i32, i32, pvp]),
        "kpt_candidates_from_grid": (i32, [vp, vp, i32, pvp]),
        "kpt_candidates_info": (i32, [vp, vp, vp]),
        "kpt_candidates_download": (i32, [vp, vp, vp, vp]),
        "kpt_candidates_destroy": (i32, [vp]),
        "kpt_generator_inject_uniform": (i32, [vp, vp, u64, u32, vp, vp, vp, vp]),
        "kpt_generator_inject_candidates": (i32, [vp, vp, u64, u32, vp, vp, vp]),
        "kpt_generator_recycle_uniform": (i32, [vp, vp, u64, u32, vp, vp, vp, i32, i32, vp]),
        "kpt_generator_recycle_candidates": (i32, [vp, vp, u64, u32, vp, vp, i32, vp]),
    }
    for name, (restype, argtypes) in sig.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    _LIB = lib
    return lib


def _check(rc: int) -> None:
    if rc != 0:
        raise KptError(f"libkpt error {rc}: {load_library().kpt_last_error().decode()}")


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def default_settings(**overrides) -> Settings:
    """Reference defaults (src/main.cpp:136-154) with keyword overrides."""
    s = Settings()
    load_library().kpt_default_settings(ctypes.byref(s))
    for key, value in overrides.items():
        if key not in DOUBLE_SETTINGS + INT_SETTINGS + CLOSURE_INT + CLOSURE_DOUBLE:
            raise KeyError(key)
        setattr(s, key, value)
    return s


def settings_from_dict(values: Dict[str, float]) -> Settings:
    """Settings from a dict; closure fields missing from it keep their defaults."""
    s = default_settings()
    for name in DOUBLE_SETTINGS + CLOSURE_DOUBLE:
        if name in values:
            setattr(s, name, float(values[name]))
    for name in INT_SETTINGS + CLOSURE_INT:
        if name in values:
            setattr(s, name, int(values[name]))
    return s


class Context:
    """One CUDA device and stream (kpt_context)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        self.handle = ctypes.c_void_p()
        self._children = weakref.WeakSet()
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_context_create(device, ctypes.byref(handle)))
        self.handle = handle

    def _adopt(self, child):
        self._children.add(child)
        return child

    def close(self) -> None:
        """Destroy the context after every field and store created from it."""
        for child in list(self._children):
            child.close()
        if self.handle:
            self.lib.kpt_context_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def synchronize(self) -> None:
        _check(self.lib.kpt_context_synchronize(self.handle))

    def set_fp64_arithmetic(self, mode: int) -> None:
        """FP64_STRICT (oracle-exact rounding, the default) or FP64_CONTRACTED
        (FMA contraction and CUDA's pow, faster) for the FP64 push."""
        _check(self.lib.kpt_context_set_fp64_arithmetic(self.handle, int(mode)))

    def set_cell_records(self, mode: int) -> None:
        """RECORDS_AUTO (default), RECORDS_OFF or RECORDS_ON: whether the
        mixed pushes sample per-cell records of the table pair (each
        component's eight corner values in one 32-byte sector) or the
        point-major tables.  The values are the same bit for bit."""
        _check(self.lib.kpt_context_set_cell_records(self.handle, int(mode)))

    def pow(self, x, y) -> np.ndarray:
        """x^y elementwise by the FP64 push's power function, on the GPU."""
        x, y = np.broadcast_arrays(np.asarray(x, dtype=np.float64),
                                   np.asarray(y, dtype=np.float64))
        x = np.ascontiguousarray(x).ravel()
        y = np.ascontiguousarray(y).ravel()
        out = np.empty_like(x)
        _check(self.lib.kpt_math_pow(self.handle, x.size, x.ctypes.data, y.ctypes.data,
                                     out.ctypes.data))
        return out

    def fp64_fma_rate(self) -> float:
        """FP64 FMA throughput of this context's GPU in TFLOP/s, measured now
        (the denominator of the FP64 pushes' roofline)."""
        out = ctypes.c_double()
        _check(self.lib.kpt_context_fp64_fma_rate(self.handle, ctypes.byref(out)))
        return out.value

    def set_stream(self, stream_handle: int) -> None:
        _check(self.lib.kpt_context_set_stream(self.handle, ctypes.c_void_p(stream_handle)))

    def set_push_schedule(self, schedule: int, blocks_per_sm: int) -> None:
        _check(self.lib.kpt_context_set_push_schedule(self.handle, schedule, blocks_per_sm))

    # -- fields ---------------------------------------------------------
    def field(self, field, kind: int = TABLE_PARKER16,
              precision: int = PRECISION_F64) -> "Field":
        """Device coefficient table for a fields.CompactField."""
        xe = np.ascontiguousarray(field.x_edges, dtype=np.float64)
        ye = np.ascontiguousarray(field.y_edges, dtype=np.float64)
        b = np.ascontiguousarray(field.b, dtype=np.float64)
        v = np.ascontiguousarray(field.v, dtype=np.float64)
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_field_create(self.handle, field.nx, field.ny, _ptr(xe), _ptr(ye),
                                         _ptr(b), _ptr(v), kind, precision,
                                         ctypes.byref(handle)))
        return self._adopt(Field(self, handle))

    def load_field(self, path: str, kind: int = TABLE_PARKER16,
                   precision: int = PRECISION_F64) -> "Field":
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_field_load(self.handle, path.encode(), kind, precision,
                                       ctypes.byref(handle)))
        return self._adopt(Field(self, handle))

    # -- particles ------------------------------------------------------
    def wrap_particles(self, capacity: int, count: int,
                       device_arrays: Dict[str, int]) -> "ParticleStorage":
        """Non-owning store over existing device arrays (pointers as ints)."""
        arr = ParticleArrays(**{k: device_arrays[k] for k, _ in ParticleArrays._fields_})
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_particles_wrap(self.handle, int(capacity), int(count),
                                           ctypes.byref(arr), ctypes.byref(handle)))
        return self._adopt(ParticleStorage(self, handle))

    def particles(self, capacity: int) -> "ParticleStorage":
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_particles_create(self.handle, int(capacity), ctypes.byref(handle)))
        return self._adopt(ParticleStorage(self, handle))

    # -- hot path -------------------------------------------------------
    def inject(self, parts: "ParticleStorage", grid: "Field", settings: Settings,
               requested: int, frame: int, seed: int, band=(0.0, 0.0)) -> int:
        n = ctypes.c_uint64()
        _check(self.lib.kpt_inject_uniform(self.handle, parts.handle, grid.handle,
                                           ctypes.byref(settings), int(requested), int(frame),
                                           int(seed), float(band[0]), float(band[1]),
                                           ctypes.byref(n)))
        return int(n.value)

    def push_interval(self, parts: "ParticleStorage", lower: "Field", upper: "Field",
                      settings: Settings, frame: int, seed: int,
                      stats: bool = True) -> Optional[PushStats]:
        out = PushStats() if stats else None
        _check(self.lib.kpt_push_interval(self.handle, parts.handle, lower.handle, upper.handle,
                                          ctypes.byref(settings), int(frame), int(seed),
                                          ctypes.byref(out) if out is not None else None))
        return out

    def split(self, parts: "ParticleStorage", settings: Settings):
        split = ctypes.c_uint64()
        skipped = ctypes.c_uint64()
        _check(self.lib.kpt_split(self.handle, parts.handle, ctypes.byref(settings),
                                  ctypes.byref(split), ctypes.byref(skipped)))
        return int(split.value), int(skipped.value)

    def sort(self, parts: "ParticleStorage", grid: "Field", tile_x: int = 16,
             tile_y: int = 16) -> None:
        """Order the work of later pushes by spatial tile (storage unchanged)."""
        _check(self.lib.kpt_particles_sort(self.handle, parts.handle, grid.handle, int(tile_x),
                                           int(tile_y)))

    def clear_order(self, parts: "ParticleStorage") -> None:
        _check(self.lib.kpt_particles_clear_order(parts.handle))

    def histogram(self, parts: "ParticleStorage", pmin: float, pmax: float,
                  nbins: int = 128) -> np.ndarray:
        bins = np.zeros(nbins, dtype=np.float64)
        _check(self.lib.kpt_histogram(self.handle, parts.handle, float(pmin), float(pmax),
                                      int(nbins), _ptr(bins)))
        return bins

    def summarize(self, parts: "ParticleStorage") -> Dict[str, float]:
        out = Summary()
        _check(self.lib.kpt_summarize(self.handle, parts.handle, ctypes.byref(out)))
        return out.as_dict()

    # -- learned closure --------------------------------------------------
    def train_surrogate(self, settings: Settings, **config) -> "Surrogate":
        """Train the QLT surrogate on the GPU (kpt_surrogate_train)."""
        cfg = SurrogateConfig()
        self.lib.kpt_surrogate_default_config(ctypes.byref(cfg))
        for key, value in config.items():
            if key not in dict(SurrogateConfig._fields_):
                raise KeyError(key)
            setattr(cfg, key, value)
        handle = ctypes.c_void_p()
        loss = ctypes.c_double()
        _check(self.lib.kpt_surrogate_train(self.handle, ctypes.byref(settings),
                                            ctypes.byref(cfg), ctypes.byref(handle),
                                            ctypes.byref(loss)))
        sg = self._adopt(Surrogate(self, handle))
        sg.final_loss = float(loss.value)
        return sg

    def set_surrogate(self, surrogate: Optional["Surrogate"]) -> None:
        _check(self.lib.kpt_context_set_surrogate(
            self.handle, surrogate.handle if surrogate is not None else None))

    def surrogate_judge(self) -> Dict[str, float]:
        """Judge counters of the pushes since the last call (then reset)."""
        ev, ju, fb = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        err = ctypes.c_double()
        _check(self.lib.kpt_surrogate_judge(self.handle, ctypes.byref(ev), ctypes.byref(ju),
                                            ctypes.byref(fb), ctypes.byref(err)))
        return {"evaluations": int(ev.value), "judged": int(ju.value),
                "fallbacks": int(fb.value), "max_rel_error": float(err.value)}

    def surrogate_gradient(self, params: np.ndarray, inputs: np.ndarray, targets: np.ndarray,
                           hidden_width: int = 0):
        """Loss and its gradient over (normalised) samples, on the GPU, for a
        network of the given hidden width (0 = the default)."""
        params = np.ascontiguousarray(params, dtype=np.float32)
        inputs = np.ascontiguousarray(inputs, dtype=np.float32)
        targets = np.ascontiguousarray(targets, dtype=np.float32)
        grad = np.zeros_like(params)
        loss = ctypes.c_float()
        _check(self.lib.kpt_surrogate_gradient(self.handle, int(hidden_width), _ptr(params),
                                               inputs.shape[0],
                                               _ptr(inputs), _ptr(targets), _ptr(grad),
                                               ctypes.byref(loss)))
        return float(loss.value), grad

    # -- header library (ParkerSolver / ParticleSystem) --------------------
    def grid(self, x_edges, y_edges, periodic=(1, 1)) -> "LibGrid":
        xe = np.ascontiguousarray(x_edges, dtype=np.float64)
        ye = np.ascontiguousarray(y_edges, dtype=np.float64)
        per = np.ascontiguousarray(periodic, dtype=np.int32)
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_grid_create(self.handle, xe.size - 1, ye.size - 1, _ptr(xe),
                                        _ptr(ye), _ptr(per), ctypes.byref(handle)))
        return self._adopt(LibGrid(self, handle, xe.size - 1, ye.size - 1))

    def stored_grid(self, x_faces, y_faces, periodic=(1, 1)) -> "LibGrid":
        """StoredCoordinateGrid on explicit face coordinates: nx + 5 / ny + 5
        faces in storage order, face -2 first (two ghost faces on each side),
        strictly ascending, possibly non-uniform."""
        xf = np.ascontiguousarray(x_faces, dtype=np.float64)
        yf = np.ascontiguousarray(y_faces, dtype=np.float64)
        per = np.ascontiguousarray(periodic, dtype=np.int32)
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_grid_create_stored(self.handle, xf.size - 5, yf.size - 5, _ptr(xf),
                                               _ptr(yf), _ptr(per), ctypes.byref(handle)))
        return self._adopt(LibGrid(self, handle, xf.size - 5, yf.size - 5))

    def system(self, count: int, capacity: int, rest_mass=1.0, charge=1.0, speed_of_light=1.0,
               energy_scale_erg=1.0, split_ratio=2.0, min_child_weight=0.0) -> "ParticleSystem":
        props = ParticleProperties(rest_mass, charge, speed_of_light, energy_scale_erg)
        policy = SplitPolicy(split_ratio, min_child_weight)
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_system_create(self.handle, int(count), int(capacity),
                                          ctypes.byref(props), ctypes.byref(policy),
                                          ctypes.byref(handle)))
        return self._adopt(ParticleSystem(self, handle))

    def parker_solver(self, grid: "LibGrid", basis: np.ndarray, constant_ratio: bool = False,
                      courant: float = 0.3) -> "ParkerSolver":
        basis = np.ascontiguousarray(basis, dtype=np.float64)
        if basis.shape != (grid.points, 18):
            raise ValueError(f"basis must be ({grid.points}, 18)")
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_parker_solver_create(self.handle, grid.handle, _ptr(basis),
                                                 int(constant_ratio), float(courant),
                                                 ctypes.byref(handle)))
        return self._adopt(ParkerSolver(self, handle))

    def batch(self) -> "Batch":
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_batch_create(self.handle, ctypes.byref(handle)))
        return self._adopt(Batch(self, handle))

    def focus_solver(self, grid: "LibGrid", basis: np.ndarray, constant_ratio: bool = False,
                     courant: float = 0.3, spectral_index: float = 5.0 / 3.0, h0: float = 1e-6,
                     floors=(0.0, 0.0, 0.0, 0.0), maximum_mu: float = 1.0) -> "FocusSolver":
        basis = np.ascontiguousarray(basis, dtype=np.float64)
        if basis.shape != (grid.points, 27):
            raise ValueError(f"basis must be ({grid.points}, 27)")
        sc = ScatteringParameters(spectral_index, h0, *floors)
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_focus_solver_create(self.handle, grid.handle, _ptr(basis),
                                                int(constant_ratio), float(courant),
                                                ctypes.byref(sc), ctypes.byref(handle)))
        solver = self._adopt(FocusSolver(self, handle))
        if maximum_mu != 1.0:
            solver.set_maximum_mu(maximum_mu)
        return solver

    # -- Parker coefficient precompute --------------------------------------
    def diffusion_parameters(self, **overrides) -> DiffusionParameters:
        p = DiffusionParameters()
        self.lib.kpt_default_diffusion_parameters(ctypes.byref(p))
        for k, v in overrides.items():
            setattr(p, k, v)
        return p

    @staticmethod
    def _turbulence(turbulence, keep: list) -> Turbulence:
        t = Turbulence()
        if turbulence is None:
            turbulence = {"sigma2": 0.5, "l2d": 1.0, "lslab": 1.0, "lc": -1.0}
        if isinstance(turbulence, Turbulence):
            return turbulence
        if "sigma2_field" in turbulence:
            t.storage = 1
            for name in ("sigma2", "l2d", "lslab", "lc"):
                arr = turbulence.get(f"{name}_field")
                if arr is not None:
                    arr = np.ascontiguousarray(arr, dtype=np.float64)
                    keep.append(arr)
                    setattr(t, f"{name}_field", arr.ctypes.data)
        else:
            t.storage = 0
            t.sigma2, t.l2d = float(turbulence["sigma2"]), float(turbulence["l2d"])
            t.lslab, t.lc = float(turbulence["lslab"]), float(turbulence.get("lc", -1.0))
        return t

    def parker_coefficients(self, grid: "LibGrid", b, v, turbulence=None, parameters=None,
                            rest_mass=1.0, charge=1.0, speed_of_light=1.0,
                            energy_scale_erg=1.0) -> np.ndarray:
        """make_legacy_transport_coefficient_fields + the solver's packed basis:
        (points, 18) from cell-centred B and V (points, 3), ghosts as given."""
        keep = []
        b = np.ascontiguousarray(b, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        if b.shape != (grid.points, 3) or v.shape != (grid.points, 3):
            raise ValueError(f"B and V must be ({grid.points}, 3)")
        t = self._turbulence(turbulence, keep)
        props = ParticleProperties(rest_mass, charge, speed_of_light, energy_scale_erg)
        params = parameters if parameters is not None else self.diffusion_parameters()
        out = np.zeros((grid.points, 18), dtype=np.float64)
        _check(self.lib.kpt_parker_coefficients(self.handle, grid.handle, _ptr(b), _ptr(v),
                                                ctypes.byref(t), ctypes.byref(props),
                                                ctypes.byref(params), _ptr(out)))
        return out

    def parker_solver_from_fields(self, grid: "LibGrid", b, v, turbulence=None,
                                  parameters=None, courant: float = 0.3, rest_mass=1.0,
                                  charge=1.0, speed_of_light=1.0,
                                  energy_scale_erg=1.0) -> "ParkerSolver":
        """ParkerSolver(particles, grid, B, V, make_legacy_transport_coefficient_
        fields(...)) with the basis built and kept on the device."""
        keep = []
        b = np.ascontiguousarray(b, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        if b.shape != (grid.points, 3) or v.shape != (grid.points, 3):
            raise ValueError(f"B and V must be ({grid.points}, 3)")
        t = self._turbulence(turbulence, keep)
        props = ParticleProperties(rest_mass, charge, speed_of_light, energy_scale_erg)
        params = parameters if parameters is not None else self.diffusion_parameters()
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_parker_solver_create_from_fields(
            self.handle, grid.handle, _ptr(b), _ptr(v), ctypes.byref(t), ctypes.byref(props),
            ctypes.byref(params), float(courant), ctypes.byref(handle)))
        return self._adopt(ParkerSolver(self, handle))

    def focus_coefficients(self, grid: "LibGrid", b, v, dvdt=None, turbulence=None,
                           parameters=None, minimum_magnetic_field_magnitude: float = 0.0,
                           rest_mass=1.0, charge=1.0, speed_of_light=1.0,
                           energy_scale_erg=1.0) -> np.ndarray:
        """FocusCoefficient::make_legacy_transport_coefficient_fields[_with_time_
        derivative] + the focused packed basis: (points, 27)."""
        keep = []
        b, v, dvdt = self._vectors(grid, b, v, dvdt)
        t = self._turbulence(turbulence, keep)
        props = ParticleProperties(rest_mass, charge, speed_of_light, energy_scale_erg)
        params = parameters if parameters is not None else self.diffusion_parameters()
        out = np.zeros((grid.points, 27), dtype=np.float64)
        _check(self.lib.kpt_focus_coefficients(
            self.handle, grid.handle, _ptr(b), _ptr(v), _ptr(dvdt), ctypes.byref(t),
            ctypes.byref(props), ctypes.byref(params),
            float(minimum_magnetic_field_magnitude), _ptr(out)))
        return out

    def focus_solver_from_fields(self, grid: "LibGrid", b, v, dvdt=None, turbulence=None,
                                 parameters=None, minimum_magnetic_field_magnitude: float = 0.0,
                                 courant: float = 0.3, spectral_index: float = 5.0 / 3.0,
                                 h0: float = 1e-6, floors=(0.0, 0.0, 0.0, 0.0),
                                 maximum_mu: float = 1.0, rest_mass=1.0, charge=1.0,
                                 speed_of_light=1.0, energy_scale_erg=1.0) -> "FocusSolver":
        """FocusTransportSolver(particles, grid, B, V, coefficients) with the
        coefficient precompute and packed basis built on the device."""
        keep = []
        b, v, dvdt = self._vectors(grid, b, v, dvdt)
        t = self._turbulence(turbulence, keep)
        props = ParticleProperties(rest_mass, charge, speed_of_light, energy_scale_erg)
        params = parameters if parameters is not None else self.diffusion_parameters()
        sc = ScatteringParameters(spectral_index, h0, *floors)
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_focus_solver_create_from_fields(
            self.handle, grid.handle, _ptr(b), _ptr(v), _ptr(dvdt), ctypes.byref(t),
            ctypes.byref(props), ctypes.byref(params), float(minimum_magnetic_field_magnitude),
            float(courant), ctypes.byref(sc), ctypes.byref(handle)))
        solver = self._adopt(FocusSolver(self, handle))
        if maximum_mu != 1.0:
            solver.set_maximum_mu(maximum_mu)
        return solver

    @staticmethod
    def _vectors(grid, b, v, dvdt):
        b = np.ascontiguousarray(b, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        if b.shape != (grid.points, 3) or v.shape != (grid.points, 3):
            raise ValueError(f"B and V must be ({grid.points}, 3)")
        if dvdt is not None:
            dvdt = np.ascontiguousarray(dvdt, dtype=np.float64)
            if dvdt.shape != (grid.points, 3):
                raise ValueError(f"dV/dt must be ({grid.points}, 3)")
        return b, v, dvdt

    # -- ParticleGenerator ---------------------------------------------------
    def lib_field(self, grid: "LibGrid", values, centering=(0, 0)) -> "LibField":
        """Field<Grid, C> on a library grid: values (points,) or (points, C),
        points in the field's flattened order (dim 0 fastest over the ghosted
        extent: cells n+4, faces n+5 per axis); centering 0 cell, 1 face."""
        values = np.asarray(values, dtype=np.float64)
        comps = 1 if values.ndim == 1 else values.shape[1]
        values = np.ascontiguousarray(values.reshape(-1, comps))
        cent = np.ascontiguousarray([_centering(c) for c in centering], dtype=np.int32)
        want = 1
        for n, c in zip((grid.nx, grid.ny), cent):
            want *= n + 4 + int(c)
        if values.shape[0] != want:
            raise ValueError(f"field needs {want} points for this grid and centering")
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_lib_field_create(self.handle, grid.handle, comps, _ptr(cent),
                                             _ptr(values), ctypes.byref(handle)))
        return self._adopt(LibField(self, handle, grid, comps, tuple(int(c) for c in cent)))

    def make_field_particle_candidate_set(self, field: "LibField", threshold: float,
                                          comparison="greater_equal", component: int = 0,
                                          domain=0, region: Optional[Region] = None
                                          ) -> "CandidateSet":
        """make_field_particle_candidate_set[_in_region] (ParticleGenerator.hpp:659-784)."""
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_candidates_from_field(
            self.handle, field.handle, None if region is None else ctypes.byref(region),
            float(threshold), _comparison(comparison), int(component), _domain(domain),
            ctypes.byref(handle)))
        return self._adopt(CandidateSet(self, handle, "field"))

    def make_grid_particle_candidate_set(self, grid: "LibGrid", domain=0) -> "CandidateSet":
        """make_grid_particle_candidate_set (ParticleGenerator.hpp:786-856)."""
        handle = ctypes.c_void_p()
        _check(self.lib.kpt_candidates_from_grid(self.handle, grid.handle, _domain(domain),
                                                 ctypes.byref(handle)))
        return self._adopt(CandidateSet(self, handle, "grid"))

    def sample(self, lower: "Field", upper: "Field", x, y, rt,
               time_interpolation: int = 1) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        rt = np.ascontiguousarray(rt, dtype=np.float64)
        ncomp = lower.shape()[3]
        out = np.zeros((x.size, ncomp), dtype=np.float64)
        _check(self.lib.kpt_sample_table(self.handle, lower.handle, upper.handle, x.size,
                                         _ptr(x), _ptr(y), _ptr(rt), int(time_interpolation),
                                         _ptr(out)))
        return out


class Field:
    """One frame's coefficient table on the device (kpt_field)."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p):
        self.ctx = ctx
        self.handle = handle

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.kpt_field_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shape(self):
        nx, ny, comps = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        points = ctypes.c_uint64()
        _check(self.ctx.lib.kpt_field_shape(self.handle, ctypes.byref(nx), ctypes.byref(ny),
                                            ctypes.byref(points), ctypes.byref(comps)))
        return nx.value, ny.value, int(points.value), comps.value

    def table(self) -> np.ndarray:
        _, _, points, comps = self.shape()
        out = np.zeros((points, comps), dtype=np.float64)
        _check(self.ctx.lib.kpt_field_download_table(self.handle, _ptr(out), out.size))
        return out


def surrogate_pack_tc(params: np.ndarray, hidden_width: int, fp16: bool = False) -> np.ndarray:
    """The tcgen05 engine's 16-bit weight block of an FP32 parameter block
    (kpt_surrogate_pack_tc; host only)."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    h = int(hidden_width)
    out = np.zeros(16 * h + h * (h + 16) + 16 * (h + 16), dtype=np.uint16)
    _check(load_library().kpt_surrogate_pack_tc(_ptr(params), h, 1 if fp16 else 0, _ptr(out),
                                                out.size))
    return out


class Surrogate:
    """A trained QLT surrogate (kpt_surrogate)."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p):
        self.ctx = ctx
        self.handle = handle
        self.final_loss = float("nan")
        hidden, count = ctypes.c_int32(), ctypes.c_int32()
        _check(ctx.lib.kpt_surrogate_shape(handle, ctypes.byref(hidden), ctypes.byref(count)))
        self.hidden_width = int(hidden.value)
        self.parameter_count = int(count.value)

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.kpt_surrogate_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def parameters(self):
        """(FP32 parameter block, normalisation dict)."""
        params = np.zeros(self.parameter_count, dtype=np.float32)
        norm = np.zeros(17, dtype=np.float32)
        _check(self.ctx.lib.kpt_surrogate_parameters(self.handle, _ptr(params), params.size,
                                                     _ptr(norm), norm.size))
        return params, {"in_lo": norm[0:5].astype(np.float64),
                        "in_hi": norm[5:10].astype(np.float64),
                        "out_offset": norm[10:13].astype(np.float64),
                        "out_scale": norm[13:16].astype(np.float64),
                        "mu_cut": float(norm[16])}

    @property
    def engine(self) -> int:
        """ENGINE_TCGEN05 (default) or ENGINE_MMA_SYNC: how the push and
        evaluate(tensor_cores=True) serve the network."""
        value = ctypes.c_int32()
        _check(self.ctx.lib.kpt_surrogate_get_engine(self.handle, ctypes.byref(value)))
        return int(value.value)

    @engine.setter
    def engine(self, value: int) -> None:
        _check(self.ctx.lib.kpt_surrogate_set_engine(self.handle, int(value)))

    def check_timeout(self, blocks: int = 8, polls: int = 64):
        """(blocks that timed out, blocks that finished the teardown) of the
        tcgen05 engine's failure-path check (kpt_surrogate_check_timeout)."""
        timed_out, finished = ctypes.c_uint32(), ctypes.c_uint32()
        _check(self.ctx.lib.kpt_surrogate_check_timeout(self.handle, int(blocks), int(polls),
                                                        ctypes.byref(timed_out),
                                                        ctypes.byref(finished)))
        return int(timed_out.value), int(finished.value)

    def evaluate(self, inputs: np.ndarray, tensor_cores: bool = True):
        """(n, 5) raw inputs (mu, ln p, ln|B|, dB^2/B^2, gamma_k) ->
        ((n, 3) D_mumu, dD_mumu/dmu, ln kappa_par; (n,) served-by-network)."""
        inputs = np.ascontiguousarray(inputs, dtype=np.float64)
        n = inputs.shape[0]
        out = np.zeros((n, 3), dtype=np.float64)
        served = np.zeros(n, dtype=np.int32)
        _check(self.ctx.lib.kpt_surrogate_evaluate(self.handle, n, _ptr(inputs),
                                                   1 if tensor_cores else 0, _ptr(out),
                                                   _ptr(served)))
        return out, served.astype(bool)


class _Handle:
    _destroy = ""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p):
        self.ctx = ctx
        self.handle = handle

    def close(self) -> None:
        if self.handle:
            getattr(self.ctx.lib, self._destroy)(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LibGrid(_Handle):
    """2D Cartesian grid of the header library (kpt_grid): analytic uniform
    axes (Context.grid) or explicit faces (Context.stored_grid)."""
    _destroy = "kpt_grid_destroy"

    def __init__(self, ctx, handle, nx, ny):
        super().__init__(ctx, handle)
        self.nx, self.ny = nx, ny
        self.points = (nx + 4) * (ny + 4)


class ParticleSystem(_Handle):
    """Header-library particle container (kpt_system, reference ParticleSystem<2>)."""
    _destroy = "kpt_system_destroy"

    @property
    def count(self) -> int:
        c = ctypes.c_uint64()
        _check(self.ctx.lib.kpt_system_count(self.handle, ctypes.byref(c), None))
        return int(c.value)

    @property
    def capacity(self) -> int:
        c = ctypes.c_uint64()
        _check(self.ctx.lib.kpt_system_count(self.handle, None, ctypes.byref(c)))
        return int(c.value)

    def set_count(self, count: int) -> None:
        _check(self.ctx.lib.kpt_system_set_count(self.handle, int(count)))

    @staticmethod
    def _arrays(data: Dict[str, np.ndarray]) -> SystemArrays:
        a = SystemArrays()
        a.id = data["id"].ctypes.data
        names = dict(zip(("x", "y", "prev_x", "prev_y", "prevstep_x", "prevstep_y", "p", "mu",
                          "weight", "e0", "status", "split_level", "sort_key"),
                         SYSTEM_DOUBLE_FIELDS + SYSTEM_INT_FIELDS))
        for field, key in names.items():
            setattr(a, field, data[key].ctypes.data)
        return a

    def upload(self, data: Dict[str, np.ndarray], n: Optional[int] = None) -> None:
        n = self.capacity if n is None else int(n)
        conv = {"id": np.ascontiguousarray(data["id"][:n], dtype=np.uint64)}
        for k in SYSTEM_DOUBLE_FIELDS:
            conv[k] = np.ascontiguousarray(data[k][:n], dtype=np.float64)
        for k in SYSTEM_INT_FIELDS:
            conv[k] = np.ascontiguousarray(data[k][:n], dtype=np.int32)
        _check(self.ctx.lib.kpt_system_upload(self.handle, n, ctypes.byref(self._arrays(conv))))

    def download(self, n: Optional[int] = None) -> Dict[str, np.ndarray]:
        n = self.capacity if n is None else int(n)
        out = {"id": np.zeros(n, dtype=np.uint64)}
        for k in SYSTEM_DOUBLE_FIELDS:
            out[k] = np.zeros(n, dtype=np.float64)
        for k in SYSTEM_INT_FIELDS:
            out[k] = np.zeros(n, dtype=np.int32)
        _check(self.ctx.lib.kpt_system_download(self.handle, n, ctypes.byref(self._arrays(out))))
        return out

    def capture_previous_positions(self) -> None:
        _check(self.ctx.lib.kpt_system_capture_previous_positions(self.ctx.handle, self.handle))

    def apply_boundary(self, grid: LibGrid) -> None:
        _check(self.ctx.lib.kpt_system_apply_boundary(self.ctx.handle, self.handle, grid.handle))

    def sort_by_key(self, lo: int, hi: int) -> None:
        _check(self.ctx.lib.kpt_system_sort_by_key(self.ctx.handle, self.handle, int(lo),
                                                   int(hi)))

    def compact(self) -> int:
        c = ctypes.c_uint64()
        _check(self.ctx.lib.kpt_system_compact(self.ctx.handle, self.handle, ctypes.byref(c)))
        return int(c.value)

    def split_energy(self) -> Dict[str, int]:
        st = SplitStatistics()
        _check(self.ctx.lib.kpt_system_split_energy(self.ctx.handle, self.handle,
                                                    ctypes.byref(st)))
        return {name: int(getattr(st, name)) for name, _ in SplitStatistics._fields_}

    def reset_split_baselines(self) -> None:
        _check(self.ctx.lib.kpt_system_reset_split_baselines(self.ctx.handle, self.handle))


class LibField(_Handle):
    """Lattice field on a library grid (kpt_lib_field, reference Field<Grid, C>)."""
    _destroy = "kpt_lib_field_destroy"

    def __init__(self, ctx, handle, grid, components, centering):
        super().__init__(ctx, handle)
        self.grid = grid
        self.components = components
        self.centering = centering


class CandidateSet(_Handle):
    """Field-point or grid-cell candidate set with cumulative physical-volume
    weights (kpt_candidates, ParticleGenerator.hpp:464-646)."""
    _destroy = "kpt_candidates_destroy"

    def __init__(self, ctx, handle, kind):
        super().__init__(ctx, handle)
        self.kind = kind

    def candidate_count(self) -> int:
        n = ctypes.c_uint64()
        _check(self.ctx.lib.kpt_candidates_info(self.handle, ctypes.byref(n), None))
        return int(n.value)

    def total_weight(self) -> float:
        t = ctypes.c_double()
        _check(self.ctx.lib.kpt_candidates_info(self.handle, None, ctypes.byref(t)))
        return float(t.value)

    def empty(self) -> bool:
        return self.candidate_count() == 0

    def download(self):
        """(point indices or cell ordinals, cumulative weights)."""
        n = self.candidate_count()
        idx = np.zeros(n, dtype=np.uint64)
        cum = np.zeros(n, dtype=np.float64)
        if n:
            _check(self.ctx.lib.kpt_candidates_download(self.ctx.handle, self.handle, _ptr(idx),
                                                        _ptr(cum)))
        return idx, cum


class ParkerSolver(_Handle):
    """Header-library Parker solver (kpt_parker_solver, reference ParkerSolver)."""
    _destroy = "kpt_parker_solver_destroy"

    def set_courant(self, courant: float) -> None:
        _check(self.ctx.lib.kpt_parker_solver_set_courant(self.handle, float(courant)))

    def set_precision(self, precision: int) -> None:
        """PRECISION_F64 (the reference's arithmetic) or PRECISION_MIXED (FP32
        basis, terms and noise; FP64 positions, momenta and dt)."""
        _check(self.ctx.lib.kpt_parker_solver_set_precision(self.handle, int(precision)))

    def set_basis(self, basis: np.ndarray, constant_ratio: bool = False) -> None:
        basis = np.ascontiguousarray(basis, dtype=np.float64)
        _check(self.ctx.lib.kpt_parker_solver_set_basis(self.handle, _ptr(basis),
                                                        int(constant_ratio)))

    def compute_time_step(self, system: ParticleSystem) -> float:
        dt = ctypes.c_double()
        _check(self.ctx.lib.kpt_parker_compute_time_step(self.ctx.handle, self.handle,
                                                         system.handle, ctypes.byref(dt)))
        return float(dt.value)

    def advance_stochastic(self, system: ParticleSystem, seed: int, step: int) -> float:
        dt = ctypes.c_double()
        _check(self.ctx.lib.kpt_parker_advance_stochastic(self.ctx.handle, self.handle,
                                                          system.handle, int(seed), int(step),
                                                          ctypes.byref(dt)))
        return float(dt.value)

    # advance_sde is the reference's alias of advance_stochastic (ParkerSolver.hpp:296-301)
    advance_sde = advance_stochastic

    def advance_deterministic(self, system: ParticleSystem) -> float:
        dt = ctypes.c_double()
        _check(self.ctx.lib.kpt_parker_advance_deterministic(self.ctx.handle, self.handle,
                                                             system.handle, ctypes.byref(dt)))
        return float(dt.value)

    def advance_stochastic_steps(self, system: ParticleSystem, seed: int, first_step: int,
                                 steps: int) -> np.ndarray:
        dts = np.zeros(max(1, steps), dtype=np.float64)
        _check(self.ctx.lib.kpt_parker_advance_stochastic_steps(
            self.ctx.handle, self.handle, system.handle, int(seed), int(first_step), int(steps),
            _ptr(dts)))
        return dts[:steps]

    def advance_with_noise(self, system: ParticleSystem, normals: np.ndarray) -> float:
        """One stochastic step driven by caller-supplied standard normals,
        normals[k][i] (k = 0..3) for particle slot i < system.count."""
        normals = np.ascontiguousarray(normals, dtype=np.float64)
        if normals.shape != (4, system.count):
            raise KptError(f"normals must have shape (4, {system.count})")
        dt = ctypes.c_double()
        _check(self.ctx.lib.kpt_parker_advance_with_noise(self.ctx.handle, self.handle,
                                                          system.handle, _ptr(normals),
                                                          ctypes.byref(dt)))
        return float(dt.value)


class Batch(_Handle):
    """Many independent runs pushed by one launch per interval (kpt_batch)."""
    _destroy = "kpt_batch_destroy"

    def __init__(self, ctx, handle):
        super().__init__(ctx, handle)
        self._keep = []

    def add_run(self, parts: "ParticleStorage", lower: "Field", upper: "Field",
                settings: Settings, seed: int, first_frame: int) -> int:
        idx = ctypes.c_int()
        _check(self.ctx.lib.kpt_batch_add_run(self.handle, parts.handle, lower.handle,
                                              upper.handle, ctypes.byref(settings), int(seed),
                                              int(first_frame), ctypes.byref(idx)))
        self._keep.append((parts, lower, upper, settings))
        return int(idx.value)

    def set_schedule(self, sort_tile: int = 16, blocks_per_sm: int = 0,
                     sort_every: int = 1) -> None:
        _check(self.ctx.lib.kpt_batch_set_schedule(self.handle, int(sort_tile),
                                                   int(blocks_per_sm), int(sort_every)))

    def schedule(self):
        t, b, e = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(self.ctx.lib.kpt_batch_get_schedule(self.handle, ctypes.byref(t), ctypes.byref(b),
                                                   ctypes.byref(e)))
        return {"sort_tile": t.value, "blocks_per_sm": b.value, "sort_every": e.value}

    def set_launch_shape(self, threads_per_block: int = 128, particles_per_lane: int = 1) -> None:
        _check(self.ctx.lib.kpt_batch_set_launch_shape(self.handle, int(threads_per_block),
                                                       int(particles_per_lane)))

    def launch_shape(self):
        t, p = ctypes.c_int(), ctypes.c_int()
        _check(self.ctx.lib.kpt_batch_get_launch_shape(self.handle, ctypes.byref(t),
                                                       ctypes.byref(p)))
        return {"threads_per_block": t.value, "particles_per_lane": p.value}

    def run(self, intervals: int, use_graph: bool = True) -> None:
        _check(self.ctx.lib.kpt_batch_run(self.handle, int(intervals), int(use_graph)))

    def stats(self, run: int) -> PushStats:
        st = PushStats()
        _check(self.ctx.lib.kpt_batch_stats(self.handle, int(run), ctypes.byref(st)))
        return st

    def frame(self, run: int) -> int:
        f = ctypes.c_uint32()
        _check(self.ctx.lib.kpt_batch_frame(self.handle, int(run), ctypes.byref(f)))
        return int(f.value)

    def set_frame(self, run: int, frame: int) -> None:
        _check(self.ctx.lib.kpt_batch_set_frame(self.handle, int(run), int(frame)))

    def autotune(self, intervals: int = 1) -> Dict[str, float]:
        t = BatchTuning()
        _check(self.ctx.lib.kpt_batch_autotune(self.handle, int(intervals), ctypes.byref(t)))
        return {name: getattr(t, name) for name, _ in BatchTuning._fields_ if name != "pad"}


class FocusSolver(_Handle):
    """Header-library focused-transport solver (kpt_focus_solver, reference FocusSolver)."""
    _destroy = "kpt_focus_solver_destroy"

    def set_courant(self, courant: float) -> None:
        _check(self.ctx.lib.kpt_focus_solver_set_courant(self.handle, float(courant)))

    def set_precision(self, precision: int) -> None:
        """PRECISION_F64 (the reference's arithmetic) or PRECISION_MIXED (FP32
        basis, terms, closure and noise; FP64 positions, momenta and dt)."""
        _check(self.ctx.lib.kpt_focus_solver_set_precision(self.handle, int(precision)))

    def set_maximum_mu(self, maximum_mu: float) -> None:
        _check(self.ctx.lib.kpt_focus_solver_set_maximum_mu(self.handle, float(maximum_mu)))

    def compute_time_step(self, system: ParticleSystem) -> float:
        dt = ctypes.c_double()
        _check(self.ctx.lib.kpt_focus_compute_time_step(self.ctx.handle, self.handle,
                                                        system.handle, ctypes.byref(dt)))
        return float(dt.value)

    def advance_stochastic(self, system: ParticleSystem, seed: int, step: int) -> float:
        dt = ctypes.c_double()
        _check(self.ctx.lib.kpt_focus_advance_stochastic(self.ctx.handle, self.handle,
                                                         system.handle, int(seed), int(step),
                                                         ctypes.byref(dt)))
        return float(dt.value)

    # advance_sde is the reference's alias of advance_stochastic (FocusSolver.hpp:298-303)
    advance_sde = advance_stochastic

    def advance_deterministic(self, system: ParticleSystem) -> float:
        dt = ctypes.c_double()
        _check(self.ctx.lib.kpt_focus_advance_deterministic(self.ctx.handle, self.handle,
                                                            system.handle, ctypes.byref(dt)))
        return float(dt.value)

    def advance_stochastic_steps(self, system: ParticleSystem, seed: int, first_step: int,
                                 steps: int) -> np.ndarray:
        dts = np.zeros(max(1, steps), dtype=np.float64)
        _check(self.ctx.lib.kpt_focus_advance_stochastic_steps(
            self.ctx.handle, self.handle, system.handle, int(seed), int(first_step), int(steps),
            _ptr(dts)))
        return dts[:steps]

    def advance_with_noise(self, system: ParticleSystem, normals: np.ndarray) -> float:
        """One stochastic step driven by caller-supplied standard normals,
        normals[k][i] (k = 0..3) for particle slot i < system.count."""
        normals = np.ascontiguousarray(normals, dtype=np.float64)
        if normals.shape != (4, system.count):
            raise KptError(f"normals must have shape (4, {system.count})")
        dt = ctypes.c_double()
        _check(self.ctx.lib.kpt_focus_advance_with_noise(self.ctx.handle, self.handle,
                                                         system.handle, _ptr(normals),
                                                         ctypes.byref(dt)))
        return float(dt.value)


class ParticleStorage:
    """Device SoA particle store (kpt_particles)."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p):
        self.ctx = ctx
        self.handle = handle

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.kpt_particles_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def count(self) -> int:
        c = ctypes.c_uint64()
        _check(self.ctx.lib.kpt_particles_count(self.handle, ctypes.byref(c), None))
        return int(c.value)

    @property
    def capacity(self) -> int:
        c = ctypes.c_uint64()
        _check(self.ctx.lib.kpt_particles_count(self.handle, None, ctypes.byref(c)))
        return int(c.value)

    def set_count(self, count: int) -> None:
        _check(self.ctx.lib.kpt_particles_set_count(self.handle, int(count)))

    def upload(self, arrays: Dict[str, np.ndarray], count: int) -> None:
        conv = {}
        for name in PARTICLE_FIELDS:
            dtype = np.int32 if name in ("status", "level") else np.float64
            conv[name] = np.ascontiguousarray(arrays[name][:count], dtype=dtype)
        _check(self.ctx.lib.kpt_particles_upload(self.handle, int(count),
                                                 *[_ptr(conv[n]) for n in PARTICLE_FIELDS]))

    def download(self, count: Optional[int] = None,
                 out: Optional[Dict[str, np.ndarray]] = None) -> Dict[str, np.ndarray]:
        """The first `count` particles (default: all stored), into new arrays or
        into `out` (contiguous arrays of the field dtypes, at least count long,
        e.g. views of pinned host memory)."""
        n = self.count if count is None else int(count)
        if out is None:
            out = {name: np.zeros(n, dtype=np.float64) for name in PARTICLE_FIELDS[:7]}
            out["status"] = np.zeros(n, dtype=np.int32)
            out["level"] = np.zeros(n, dtype=np.int32)
        for name in PARTICLE_FIELDS:
            dtype = np.int32 if name in ("status", "level") else np.float64
            a = out[name]
            if a.dtype != dtype or not a.flags.c_contiguous or a.shape[0] < n:
                raise KptError(f"download: out[{name!r}] must be contiguous {dtype.__name__} "
                               f"of length >= {n}")
        _check(self.ctx.lib.kpt_particles_download(self.handle, n,
                                                   *[_ptr(out[k]) for k in PARTICLE_FIELDS]))
        return out

    def pack_records(self, initial_kinetic_energy: float) -> np.ndarray:
        """The driver's v4 snapshot records of the stored particles (packed on the GPU)."""
        n = self.count
        out = np.zeros(n * 100, dtype=np.uint8)
        _check(self.ctx.lib.kpt_particles_pack_records(self.ctx.handle, self.handle,
                                                       float(initial_kinetic_energy), _ptr(out),
                                                       out.size))
        return out

    def device_arrays(self) -> Dict[str, int]:
        arr = ParticleArrays()
        _check(self.ctx.lib.kpt_particles_device_arrays(self.handle, ctypes.byref(arr)))
        return {name: getattr(arr, name) for name, _ in ParticleArrays._fields_}


# ---- ParticleGenerator (ParticleGenerator.hpp) ---------------------------------

COMPARISONS = {"greater": 0, "greater_equal": 1, "less": 2, "less_equal": 3,
               "abs_greater": 4, "abs_less": 5}
RECYCLE_SELECTIONS = {"escaped_only": 0, "inactive_only": 1, "recyclable": 2}
DOMAINS = {"physical": 0, "ghosted": 1}


def _comparison(value) -> int:
    return COMPARISONS[value] if isinstance(value, str) else int(value)


def _selection(value) -> int:
    return RECYCLE_SELECTIONS[value] if isinstance(value, str) else int(value)


def _domain(value) -> int:
    return DOMAINS[value] if isinstance(value, str) else int(value)


def _centering(value) -> int:
    if isinstance(value, str):
        return {"cell": 0, "face": 1}[value]
    return int(value)


class RandomManager:
    """Noise source of the generator calls (RandomManager.hpp): the seed and
    the frame that key every particle slot's stream, so results are the same
    for any thread schedule."""

    def __init__(self, seed: int = 114514, frame: int = 0):
        self.seed = int(seed)
        self.frame = int(frame)


class FieldThresholdParticlePredicate:
    """make_field_threshold_particle_predicate (ParticleGenerator.hpp:360-369)."""

    def __init__(self, field: LibField, threshold: float, comparison="greater_equal",
                 component: int = 0, domain=0):
        self.field = field
        self.struct = _FieldPredicate(field.handle.value, float(threshold),
                                      _comparison(comparison), int(component), _domain(domain), 0)


def make_field_threshold_particle_predicate(field, threshold, comparison="greater_equal",
                                            component=0, domain=0):
    return FieldThresholdParticlePredicate(field, threshold, comparison, component, domain)


def make_particle_region(lower, upper) -> Region:
    """make_particle_region (ParticleGenerator.hpp:196-203)."""
    r = Region((ctypes.c_double * 2)(*map(float, lower)), (ctypes.c_double * 2)(*map(float, upper)))
    for dim in range(2):
        if not (np.isfinite(r.lower[dim]) and np.isfinite(r.upper[dim])
                and r.upper[dim] > r.lower[dim]):
            raise KptError("AxisAlignedParticleRegion: bounds must be finite and ascending.")
    return r


def make_particle_region_from_grid(grid: LibGrid, domain=0) -> Region:
    """make_particle_region_from_grid (ParticleGenerator.hpp:208-226)."""
    r = Region()
    _check(grid.ctx.lib.kpt_region_from_grid(grid.handle, _domain(domain), ctypes.byref(r)))
    return r


def make_particle_injection_plan(first_particle_index: int, particle_count: int,
                                 max_attempts: int = 64) -> ParticleInjectionPlan:
    """make_particle_injection_plan (ParticleGenerator.hpp:169-179)."""
    return ParticleInjectionPlan(int(first_particle_index), int(particle_count),
                                 int(first_particle_index), int(max_attempts), 0)


def make_particle_append_plan(system: ParticleSystem, particle_count: int,
                              max_attempts: int = 64) -> ParticleInjectionPlan:
    """make_particle_append_plan (ParticleGenerator.hpp:183-191)."""
    return make_particle_injection_plan(system.count, particle_count, max_attempts)


def _kin(kinematics) -> ParticleInjectionKinematics:
    return ParticleInjectionKinematics() if kinematics is None else kinematics


def inject_particles_uniform_if(system: ParticleSystem, random: RandomManager, region: Region,
                                plan: ParticleInjectionPlan, kinematics=None,
                                predicate: Optional[FieldThresholdParticlePredicate] = None
                                ) -> None:
    """inject_particles_uniform_if (ParticleGenerator.hpp:885-960); no
    predicate = AlwaysAcceptParticlePredicate."""
    lib = system.ctx.lib
    _check(lib.kpt_generator_inject_uniform(
        system.ctx.handle, system.handle, random.seed, random.frame, ctypes.byref(region),
        ctypes.byref(plan), ctypes.byref(_kin(kinematics)),
        None if predicate is None else ctypes.byref(predicate.struct)))


def inject_particles_uniform(system, random, region, plan, kinematics=None) -> None:
    """inject_particles_uniform (ParticleGenerator.hpp:1106-1119)."""
    inject_particles_uniform_if(system, random, region, plan, kinematics, None)


def inject_particles_from_field_candidates(system: ParticleSystem, random: RandomManager,
                                           candidates: CandidateSet,
                                           plan: ParticleInjectionPlan, kinematics=None) -> None:
    """inject_particles_from_field_candidates (ParticleGenerator.hpp:962-1032)."""
    _check(system.ctx.lib.kpt_generator_inject_candidates(
        system.ctx.handle, system.handle, random.seed, random.frame, candidates.handle,
        ctypes.byref(plan), ctypes.byref(_kin(kinematics))))


inject_particles_from_grid_candidates = inject_particles_from_field_candidates


def inject_particles_uniform_in_grid(system, random, grid: LibGrid, plan, kinematics=None,
                                     domain=0) -> None:
    """inject_particles_uniform_in_grid (ParticleGenerator.hpp:1121-1137)."""
    candidates = system.ctx.make_grid_particle_candidate_set(grid, domain)
    try:
        inject_particles_from_field_candidates(system, random, candidates, plan, kinematics)
    finally:
        candidates.close()


def inject_particles_uniform_where_field(system, random, plan, kinematics, field: LibField,
                                         threshold: float, comparison="greater_equal",
                                         component: int = 0, domain=0,
                                         region: Optional[Region] = None) -> None:
    """inject_particles_uniform_where_field, both overloads
    (ParticleGenerator.hpp:1139-1184): region None = the grid's domain."""
    candidates = system.ctx.make_field_particle_candidate_set(field, threshold, comparison,
                                                              component, domain, region)
    try:
        inject_particles_from_field_candidates(system, random, candidates, plan, kinematics)
    finally:
        candidates.close()


def recycle_particles_uniform_if(system: ParticleSystem, random: RandomManager, region: Region,
                                 kinematics=None, predicate=None, selection="escaped_only",
                                 max_attempts: int = 64) -> int:
    """recycle_particles_uniform_if (ParticleGenerator.hpp:1186-1258); returns
    how many particles were rewritten."""
    n = ctypes.c_uint64()
    _check(system.ctx.lib.kpt_generator_recycle_uniform(
        system.ctx.handle, system.handle, random.seed, random.frame, ctypes.byref(region),
        ctypes.byref(_kin(kinematics)),
        None if predicate is None else ctypes.byref(predicate.struct), _selection(selection),
        int(max_attempts), ctypes.byref(n)))
    return int(n.value)


def recycle_particles_uniform(system, random, region, kinematics=None,
                              selection="escaped_only") -> int:
    """recycle_particles_uniform (ParticleGenerator.hpp:1260-1272)."""
    return recycle_particles_uniform_if(system, random, region, kinematics, None, selection)


def recycle_particles_from_field_candidates(system: ParticleSystem, random: RandomManager,
                                            candidates: CandidateSet, kinematics=None,
                                            selection="escaped_only") -> int:
    """recycle_particles_from_field_candidates / _from_grid_candidates
    (ParticleGenerator.hpp:1305-1447)."""
    n = ctypes.c_uint64()
    _check(system.ctx.lib.kpt_generator_recycle_candidates(
        system.ctx.handle, system.handle, random.seed, random.frame, candidates.handle,
        ctypes.byref(_kin(kinematics)), _selection(selection), ctypes.byref(n)))
    return int(n.value)


recycle_particles_from_grid_candidates = recycle_particles_from_field_candidates


def recycle_particles_uniform_in_grid(system, random, grid: LibGrid, kinematics=None,
                                      selection="escaped_only", domain=0) -> int:
    """recycle_particles_uniform_in_grid (ParticleGenerator.hpp:1283-1299)."""
    candidates = system.ctx.make_grid_particle_candidate_set(grid, domain)
    try:
        return recycle_particles_from_field_candidates(system, random, candidates, kinematics,
                                                       selection)
    finally:
        candidates.close()


def recycle_particles_uniform_where_field(system, random, kinematics, field: LibField,
                                          threshold: float, comparison="greater_equal",
                                          component: int = 0, domain=0,
                                          selection="escaped_only",
                                          region: Optional[Region] = None) -> int:
    """recycle_particles_uniform_where_field, both overloads
    (ParticleGenerator.hpp:1449-1493)."""
    candidates = system.ctx.make_field_particle_candidate_set(field, threshold, comparison,
                                                              component, domain, region)
    try:
        return recycle_particles_from_field_candidates(system, random, candidates, kinematics,
                                                       selection)
    finally:
        candidates.close()


def header_functions(path: str = HEADER_PATH) -> Sequence[str]:
    """Names of the functions declared in include/kpt.h."""
    import re
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(kpt_[a-z0-9_]+)\s*\(", text)))
