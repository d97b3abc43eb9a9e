"""ctypes mirror of include/sosb.h and the loader of the in-tree libsosb.so.

The library is built in-tree by `sosfuse2_gb300.build.build()` (nvcc, sm_103a). Loading fails loudly when it is
missing: there is no CPU fallback for the transport.
"""

import ctypes
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_DIR = PKG / '_lib'
LIB_PATH = LIB_DIR / 'libsosb.so'

c_int = ctypes.c_int32
c_i64 = ctypes.c_int64
c_dbl = ctypes.c_double
P_f32 = ctypes.POINTER(ctypes.c_float)
P_f64 = ctypes.POINTER(ctypes.c_double)
P_i64 = ctypes.POINTER(ctypes.c_int64)
P_i32 = ctypes.POINTER(ctypes.c_int32)
P_u8 = ctypes.POINTER(ctypes.c_uint8)

CELLS = 0
OBSERVER = 1
KERNEL_CLASSES = ('transport', 'projection', 'plane', 'composition', 'boxes', 'anderson', 'other', 'transport_table',
                  'corner')


class Dims(ctypes.Structure):
    _fields_ = [(n, c_int) for n in (
        'L', 'W', 'nh', 'nc', 'nq', 'nq_query', 'strato', 'density_rows', 'density_mask', 'n_sun_h', 'n_sun_x',
        'monitors', 'n_monitor_rows', 'n_dirs', 'box_points')] + [(n, c_dbl) for n in (
        'top_km', 'profile_step_km', 'mix', 'g', 'height', 'albedo', 'air_surface', 'strato_center', 'strato_sigma',
        'strato_norm', 'lower_end_km', 'air_end_km')]


class Constants(ctypes.Structure):
    _fields_ = [
        ('u', P_f64), ('wu', P_f64), ('uq', P_f64), ('wuq', P_f64),
        ('h', P_f32), ('chi', P_f32), ('hr', P_f32), ('ha', P_f32), ('ext', P_f32), ('asca', P_f32),
        ('density_table', P_f32), ('sun_h', P_f32), ('sun_col', P_f32), ('gm', P_f32),
        ('goff', P_i64), ('gdir', P_f32), ('gval', P_f32),
        ('rf', P_f32), ('af', P_f32), ('ext0', P_f32), ('solar', P_f64), ('box_ww', P_f64),
        ('strato_ext', P_f32), ('strato_sca', P_f32), ('strato_chi', P_f32), ('strato_density', P_f32),
        ('strato_sun_col', P_f32), ('strato_eigen', P_f32), ('strato_sca_source', P_f32), ('aer2', P_f32),
        ('tropo_bins', c_int), ('tropo_lut', P_f32), ('tropo_eigen', P_f32),
    ]


class Bundle(ctypes.Structure):
    _fields_ = [
        ('ncell', c_int), ('nray', c_i64), ('nseg', c_i64),
        ('cell_off', P_i64), ('p', P_f64), ('target', P_f64), ('d', P_f64), ('dloc', P_f64), ('weight', P_f64),
        ('seg_off', P_i64), ('seg_a', P_f64), ('seg_b', P_f64), ('seg_lower', P_u8),
        ('end_j', P_i32), ('end_f', P_f64), ('end_col', P_f32), ('end_st', P_f32), ('hits', P_u8),
    ]


class GroundRays(ctypes.Structure):
    _fields_ = [
        ('n', c_i64), ('cell', P_i32), ('loc', P_f64), ('weight', P_f64), ('cols', P_f64), ('cos_sun', P_f64),
        ('ok', P_u8),
    ]


class ProfileShape(ctypes.Structure):
    _fields_ = [('top', c_dbl), ('aerosol_height', c_dbl), ('ozone_peak', c_dbl), ('ozone_norm', c_dbl),
                ('no2_center', c_dbl), ('strato', c_int), ('strato_center', c_dbl), ('strato_sigma', c_dbl),
                ('strato_norm', c_dbl)]


class ColumnGrid(ctypes.Structure):
    _fields_ = [('n_h', c_int), ('n_x', c_int), ('top', c_dbl), ('h', P_f64), ('up', P_f64), ('down', P_f64)]


class Stats(ctypes.Structure):
    _fields_ = [
        ('evaluations', c_int), ('converged', c_int), ('seconds', c_dbl),
        ('observer_relative', c_dbl * 64), ('source_relative', c_dbl * 64), ('done', c_int * 64),
        ('kernel_launches', c_i64), ('start_fallback', c_int),
    ]


# exported symbols and their signatures (argtypes, restype)
SIGNATURES = {
    'sosb_create': ([ctypes.POINTER(Dims), ctypes.POINTER(ctypes.c_void_p)], c_int),
    'sosb_destroy': ([ctypes.c_void_p], c_int),
    'sosb_set_stream': ([ctypes.c_void_p, ctypes.c_void_p], c_int),
    'sosb_set_node_tables': ([ctypes.c_void_p, c_int], c_int),
    'sosb_set_projection': ([ctypes.c_void_p, c_int], c_int),
    'sosb_set_graphs': ([ctypes.c_void_p, c_int], c_int),
    'sosb_set_autotune': ([ctypes.c_void_p, c_int], c_int),
    'sosb_set_pairs': ([ctypes.c_void_p, c_int], c_int),
    'sosb_set_constants': ([ctypes.c_void_p, ctypes.POINTER(Constants)], c_int),
    'sosb_set_bundle': ([ctypes.c_void_p, c_int, ctypes.POINTER(Bundle)], c_int),
    'sosb_set_ground_rays': ([ctypes.c_void_p, ctypes.POINTER(GroundRays)], c_int),
    'sosb_prepare_ground': ([ctypes.c_void_p, c_dbl, P_f64, P_f64], c_int),
    'sosb_ray_segments': ([c_i64, P_f64, P_f64, c_dbl, P_f64, c_int, c_int, P_f64, ctypes.POINTER(ColumnGrid), P_f64,
                           P_u8, P_u8, P_i32, P_f64, P_f32, P_f32, P_u8, c_int], c_int),
    'sosb_ray_segments_device': ([c_i64, ctypes.c_void_p, ctypes.c_void_p, c_dbl, ctypes.c_void_p, c_int, c_int,
                                  ctypes.c_void_p, ctypes.POINTER(ColumnGrid), ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_void_p], c_int),
    'sosb_ring_quadrature': ([c_int, P_f64, P_f64, c_int, c_int, P_f64, c_int, c_int, c_dbl, P_f64, P_f64, P_i64,
                              P_f64, P_f64, c_i64, c_int], c_int),
    'sosb_column_table': ([c_int, P_f64, c_int, P_f64, P_f64, c_int, P_f64, P_f64, c_int, ctypes.POINTER(ProfileShape),
                           P_f64, P_f64, c_int], c_int),
    'sosb_column_table_device': ([c_int, ctypes.c_void_p, c_int, ctypes.c_void_p, P_f64, c_int, ctypes.c_void_p,
                                  ctypes.c_void_p, c_int, ctypes.POINTER(ProfileShape), ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_void_p], c_int),
    'sosb_evaluate': ([ctypes.c_void_p, c_int, c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                       ctypes.c_void_p, ctypes.c_void_p], c_int),
    'sosb_apply': ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], c_int),
    'sosb_boxes': ([ctypes.c_void_p, ctypes.c_void_p, P_f64], c_int),
    'sosb_solve': ([ctypes.c_void_p, c_int, c_dbl, ctypes.c_void_p, ctypes.c_void_p, c_int, ctypes.POINTER(Stats)],
                   c_int),
    'sosb_set_corner_mma': ([ctypes.c_void_p, c_int], c_int),
    'sosb_set_ground_mma': ([ctypes.c_void_p, c_int], c_int),
    'sosb_phase_factors': ([P_f64, c_int, c_int, c_int, c_dbl, P_f64, P_f64, ctypes.POINTER(c_int)], c_int),
    'sosb_set_warm_history': ([ctypes.c_void_p, c_int], c_int),
    'sosb_history': ([ctypes.c_void_p, c_int, P_i32, P_f64, P_f64], c_int),
    'sosb_compose_static': ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                             ctypes.c_void_p, P_i64, P_f64], c_int),
    'sosb_solve_warm': ([ctypes.c_void_p, c_int, c_dbl, ctypes.c_void_p, c_dbl, ctypes.c_void_p, ctypes.c_void_p, c_int,
                         ctypes.POINTER(Stats)], c_int),
    'sosb_apply_batch': ([ctypes.POINTER(ctypes.c_void_p), c_int, ctypes.POINTER(ctypes.c_void_p),
                          ctypes.POINTER(ctypes.c_void_p), P_i32, c_int], c_int),
    'sosb_solve_warm_batch': ([ctypes.POINTER(ctypes.c_void_p), c_int, c_int, c_dbl, ctypes.POINTER(ctypes.c_void_p),
                               c_dbl, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p), c_int,
                               ctypes.POINTER(Stats), P_i32, c_int], c_int),
    'sosb_solve_batch': ([ctypes.POINTER(ctypes.c_void_p), c_int, c_int, c_dbl, ctypes.POINTER(ctypes.c_void_p),
                          ctypes.POINTER(ctypes.c_void_p), c_int, ctypes.POINTER(Stats), P_i32, c_int], c_int),
    'sosb_gemm_bf16': ([ctypes.c_void_p, ctypes.c_void_p, c_int, c_int, c_int, ctypes.c_void_p, c_int,
                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], c_int),
    'sosb_tc_check': ([ctypes.c_void_p], c_int),
    'sosb_tc_last_error': ([], ctypes.c_char_p),
    'sosb_mlp_gelu_backward': ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                                ctypes.c_void_p, ctypes.c_void_p], c_int),
    'sosb_mlp_transpose': ([ctypes.c_void_p, c_int, c_int, c_int, ctypes.c_void_p, ctypes.c_void_p], c_int),
    'sosb_mlp_column_sum': ([ctypes.c_void_p, c_int, c_int, ctypes.c_void_p, ctypes.c_void_p], c_int),
    'sosb_mlp_adam': ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong,
                       ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, c_int, ctypes.c_float,
                       ctypes.c_void_p, ctypes.c_void_p], c_int),
    'sosb_mlp_mse': ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_float, ctypes.c_void_p,
                      ctypes.c_void_p, c_int, ctypes.c_void_p], c_int),
    'sosb_mlp_to_bf16': ([ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p], c_int),
    'sosb_set_timing': ([ctypes.c_void_p, c_int], c_int),
    'sosb_get_timing': ([ctypes.c_void_p, P_f64, P_i64, c_int], c_int),
    'sosb_last_error': ([ctypes.c_void_p], ctypes.c_char_p),
    'sosb_shape': ([ctypes.c_void_p, P_i64, P_i32, P_i32], c_int),
    'sosb_version': ([], ctypes.c_char_p),
}

_LIB = None


def library(path=None):
    """The loaded libsosb (built in-tree); raises when it is missing."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path or os.environ.get('SOSB_LIBRARY', LIB_PATH))
    if not p.exists():
        raise RuntimeError(f'E_NATIVE_MISSING: {p} is not built; run sosfuse2_gb300.build.build() (nvcc, sm_103a)')
    lib = ctypes.CDLL(str(p))
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _LIB = lib
    return lib


def ptr(a, ctype):
    """ctypes pointer to a C-contiguous NumPy array (None stays NULL)."""
    if a is None:
        return None
    if not a.flags['C_CONTIGUOUS']:
        raise ValueError('E_LAYOUT: array must be C-contiguous')
    return a.ctypes.data_as(ctype)
