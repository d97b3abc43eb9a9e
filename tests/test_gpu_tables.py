"""Node tables: warm launches that read the stored per-node frame angles, corner fractions and attenuation give the
radiance of launches that recompute them, for the warp kernels (W <= 4) and the wavelength-chunk kernels (W > 4), on
the cell and the observer bundles. The operations are the same; the compiler may contract multiply-adds differently
in the two kernels, so the bound is relative 1e-5 of each wavelength's largest value, not bit equality."""

import numpy as np
import pytest

from test_gpu_synth import small_state

pytestmark = pytest.mark.gpu

CASES = {
    'w1_l16': dict(W=1, L=16, top=80.0, nh=6),
    'w3_l32_top120': dict(W=3, L=32, top=120.0, nh=7),
    'w8_l24': dict(W=8, L=24, top=80.0, nh=6),
    'w33_l16': dict(W=33, L=16, top=80.0, nh=5),
}


def _run(arrays, tables, pairs=True, corner=False):
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    solver = Solver(PackedState(dict(arrays)), device='cuda:0')
    k = solver.kernel
    k.set_node_tables(tables)
    k._check(k.lib.sosb_set_pairs(k.h, int(pairs)))
    k._check(k.lib.sosb_set_corner_mma(k.h, int(corner)))
    x = k.field(np.zeros(solver.state.shape, np.float32))
    out = []
    for _ in range(2):                      # the first pass over each bundle builds the table, the second reads it
        g = solver.apply(x)
        out.append(g.cpu().numpy())
        out.append(k.launch(2, False, g)[2].cpu().numpy())
        x = g
    k.close()
    return out


def _close(a, b):
    err = np.abs(a - b)
    ref = max(np.abs(b).max(), 1e-30)
    return err.max() <= 1e-5 * ref, err.max() / ref


@pytest.mark.parametrize('case', sorted(CASES))
def test_tables_match_recompute(case):
    arrays = small_state(**CASES[case])
    on = _run(arrays, True)
    off = _run(arrays, False)
    for i, (a, b) in enumerate(zip(on, off)):
        ok, rel = _close(a, b)
        assert ok, (case, i, rel)


@pytest.mark.parametrize('case', sorted(CASES))
def test_pairs_match_node_synthesis(case):
    """Corner SH from the per-pair contractions (W > 4) against the per-lane corner cache (same sums); with W <= 4
    pairs are not used and both runs take the per-node synthesis. The cell bundle's contractions serve its ground and
    warm passes and are redone for every new plane (the observer pass between two applications builds its own), so a
    stale contraction would show here."""
    arrays = small_state(**CASES[case])
    on = _run(arrays, True, pairs=True)
    off = _run(arrays, True, pairs=False)
    for i, (a, b) in enumerate(zip(on, off)):
        ok, rel = _close(a, b)
        assert ok, (case, i, rel)


@pytest.mark.parametrize('case', ['w8_l24', 'w33_l16', 'w6_l48'])
def test_corner_mma_matches_pairs(case):
    """Corner SH values from the tensor-core products (bf16x3: BF16 high and low parts, three products, FP32
    accumulation) against the FP32 pair contractions, over two applications and their observer passes (the corner
    values are redone for every new plane): within 1e-4 of each output's largest value (the split keeps about 16 bits
    of every operand)."""
    c = dict(CASES, w6_l48=dict(W=6, L=48, top=120.0, nh=4))[case]
    arrays = small_state(**c)
    mma = _run(arrays, True, pairs=True, corner=True)
    fp32 = _run(arrays, True, pairs=True, corner=False)
    for i, (a, b) in enumerate(zip(mma, fp32)):
        err = np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)
        assert err <= 1e-4, (case, i, err)
