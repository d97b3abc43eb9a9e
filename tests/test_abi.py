"""The C ABI without a GPU: libsosb builds for sm_103a, loads, exports every entry point include/sosb.h declares,
and the ctypes mirror (sosfuse2_gb300._abi) lays its structs out field for field like the header."""

import ctypes
import re
from pathlib import Path

import pytest

from conftest import ROOT
from sosfuse2_gb300 import _abi, build

HEADER = (ROOT / 'include' / 'sosb.h').read_text()


def declared_functions():
    return sorted(set(re.findall(r'^\s*(?:int|const char \*)\s*(sosb_\w+)\s*\(', HEADER, re.M)))


def header_struct_fields(name):
    body = re.search(r'typedef struct \{([^}]*)\}\s*' + name + ';', HEADER).group(1)
    body = re.sub(r'/\*.*?\*/', '', body, flags=re.S)
    fields = []
    for decl in body.split(';'):
        decl = decl.strip()
        if not decl:
            continue
        decl = re.sub(r'^(const\s+)?\w+\s*', '', decl)
        for part in decl.split(','):
            nm = re.sub(r'[\s*]|\[.*\]', '', part)
            if nm:
                fields.append(nm)
    return fields


@pytest.fixture(scope='module')
def lib():
    path = build.build()
    return ctypes.CDLL(str(path))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_abi.SIGNATURES)


def test_version_string(lib):
    lib.sosb_version.restype = ctypes.c_char_p
    assert lib.sosb_version().decode().endswith('sm_103a')


@pytest.mark.parametrize('cname,pytype', [('sosb_dims', _abi.Dims), ('sosb_constants', _abi.Constants),
                                           ('sosb_bundle', _abi.Bundle), ('sosb_stats', _abi.Stats),
                                           ('sosb_ground_rays', _abi.GroundRays),
                                           ('sosb_profile_shape', _abi.ProfileShape),
                                           ('sosb_column_grid', _abi.ColumnGrid)])
def test_struct_layout_matches_header(cname, pytype):
    assert header_struct_fields(cname) == [f[0] for f in pytype._fields_]


def test_null_handle_is_an_error(lib):
    lib.sosb_last_error.restype = ctypes.c_char_p
    lib.sosb_last_error.argtypes = [ctypes.c_void_p]
    assert lib.sosb_last_error(None).startswith(b'E_HANDLE')
    assert lib.sosb_destroy(None) == 0


def test_ground_entry_points_reject_null_handles(lib):
    lib.sosb_set_ground_rays.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.sosb_prepare_ground.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    rays = _abi.GroundRays(n=0)
    assert lib.sosb_set_ground_rays(None, ctypes.byref(rays)) == 1
    ext = (ctypes.c_double * 5)()
    assert lib.sosb_prepare_ground(None, 0.3, ext, None) == 1



def test_handle_free_entry_points_reject_bad_arguments():
    """The entry points without a handle check their arguments on the host before any CUDA call: an empty grid, more
    than eight shells, a missing array or fewer than two solar-zenith nodes return 1 with nothing launched (so this
    runs without a GPU); the per-handle switches reject a NULL handle."""
    import numpy as np

    lib = _abi.library()
    a = np.zeros(64)
    p = a.ctypes.data_as(ctypes.c_void_p)
    pd = _abi.ptr(a, _abi.P_f64)
    shape = _abi.ProfileShape()
    col = lib.sosb_column_table_device
    assert col(0, p, 2, p, None, 0, p, p, 4, ctypes.byref(shape), p, p, None) == 1  # no heights
    assert col(2, p, 2, p, pd, 9, p, p, 4, ctypes.byref(shape), p, p, None) == 1  # nine shells
    assert col(2, p, 2, p, None, 1, p, p, 4, ctypes.byref(shape), p, p, None) == 1  # shells missing
    assert col(2, p, 2, p, None, 0, p, p, 4, None, p, p, None) == 1  # no profile shape
    assert col(2, p, 2, p, None, 0, p, p, 4, ctypes.byref(shape), p, None, None) == 1  # no down table
    seg = lib.sosb_ray_segments_device
    outs = [p] * 9
    assert seg(1, p, p, 80.0, None, 0, 1, p, None, *outs) == 1  # one solar-zenith node
    assert seg(1, p, p, 80.0, pd, 9, 4, p, None, *outs) == 1  # nine shells
    assert seg(-1, p, p, 80.0, None, 0, 4, p, None, *outs) == 1  # negative ray count
    grid = _abi.ColumnGrid(n_h=1, n_x=2)
    assert seg(1, p, p, 80.0, None, 0, 4, p, ctypes.byref(grid), *outs) == 1  # a one-height table
    assert lib.sosb_set_ground_mma(None, 1) == 1
    assert lib.sosb_set_corner_mma(None, 1) == 1
    rank = ctypes.c_int(-1)
    assert lib.sosb_phase_factors(pd, 0, 4, 8, 2e-6, pd, pd, ctypes.byref(rank)) == 1
