"""The ground-ray arrays handed to sosb_prepare_ground carry everything the preparation needs: a NumPy restatement
of the device algorithm (per-ray FP64 values, kept rays per cell in ray order, per-cell factor sums times
2 C ext[0]) over `synth.Family.ground_rays()` reproduces the host preparation `synth.Family.ground` of the same
state (engine_core.Solver.prepare_ground, src/sosfuse2/solve/engine_core.py:103-147); and, pinned to the reference,
the same restatement over the reference's own ground rays of two golden states (tests/golden/ground_*.npz, written by
tests/golden/make_ground_fixture.py from precompute/host_cache._ground_values and atmosphere/stratosphere.attach)
reproduces the gm, goff, gdir and gval those reference functions produced."""

import math

import numpy as np
import pytest

from conftest import GOLDEN


def _prepare(rays, ns, albedo, ext, strato_ext):
    cols = rays['cols']
    od = sum(cols[:, k, None] * ext[k][None, :] for k in range(5))
    if strato_ext is not None:
        od = od + cols[:, 5, None] * strato_ext[None, :]
    value = albedo / math.pi * rays['cos_sun'][:, None] * np.exp(-od) * rays['ok'][:, None] * rays['weight'][:, None]
    lo = rays['loc']
    factor = np.stack([(1 - lo[:, 0] ** 2) / 2, (1 - lo[:, 1] ** 2) / 2, (1 - lo[:, 2] ** 2) / 2,
                       -lo[:, 0] * lo[:, 2] / 2], -1)
    W = ext.shape[1]
    gm = np.zeros((ns, 4, W))
    for k in range(4):
        for w in range(W):
            gm[:, k, w] = np.bincount(rays['cell'], weights=factor[:, k] * value[:, w], minlength=ns)
    gm *= (2 * (3 / (16 * math.pi)) * ext[0])[None, None, :]
    take = np.any(value > 0, axis=1)
    goff = np.r_[0, np.cumsum(np.bincount(rays['cell'][take], minlength=ns))]
    return gm.astype(np.float32), goff, lo[take].astype(np.float32), value[take].astype(np.float32)


def test_ground_rays_reproduce_host_preparation():
    from sosfuse2_gb300 import synth

    atm = synth.Atmosphere(np.array([450.0, 650.0]), seed=5, top=80.0, strato_tau=0.02, albedo=0.35)
    h = np.r_[0.0, np.geomspace(0.5, 80.0, 4)]
    fam = synth.Family(h, [0.0, 60.0, 90.0, 96.0, 110.0, 180.0], 16, 1, 2, 4, atm, sun_scale=1)
    rays = fam.ground_rays()
    ns = len(h) * 6
    assert np.all(np.diff(rays['cell']) >= 0) and rays['cell'].min() >= 0 and rays['cell'].max() < ns
    want = fam.ground(atm, atm.ext())
    got = _prepare(rays, ns, atm.albedo, atm.ext(), atm.strato_ext)
    assert np.array_equal(got[1], want[1]) and np.array_equal(got[2], want[2])
    for a, b in ((got[0], want[0]), (got[3], want[3])):
        assert np.max(np.abs(a - b)) <= 1e-6 * np.abs(b).max()


def reference_ground(name):
    """The reference's ground rays of a golden state in the sosb_set_ground_rays layout, and its prepared arrays."""
    z = np.load(GOLDEN / f'ground_{name}.npz')
    rays = dict(cell=z['ray_cell'], loc=z['ray_loc'], weight=z['ray_weight'], cols=z['ray_cols'],
                cos_sun=z['ray_cos_sun'], ok=z['ray_ok'])
    strato_ext = z['strato_ext'] if len(z['strato_ext']) else None
    return rays, float(z['albedo']), z['ext'], strato_ext, (z['gm'], z['goff'], z['gdir'], z['gval'])


@pytest.mark.parametrize('name', ['walk1', 'strato15'])
def test_restatement_reproduces_reference_prepare_ground(name):
    rays, albedo, ext, strato_ext, want = reference_ground(name)
    got = _prepare(rays, len(want[1]) - 1, albedo, ext, strato_ext)
    assert np.array_equal(got[1], want[1]) and np.array_equal(got[2], want[2])
    assert np.array_equal(got[3], want[3])
    assert np.max(np.abs(got[0] - want[0])) <= 1e-6 * np.abs(want[0]).max()
