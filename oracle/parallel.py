"""The oracle over a pool of host processes (TEST INFRASTRUCTURE ONLY, like the rest of oracle/).

Only the tests, `__graft_entry__.smoke()` and the `cpu_baseline` / `--impl reference` legs of `bench.py` use it, as
the checker or the timed CPU baseline of a state too large for one core (the 1,010-cell config-0 state: about 76 s
of first light and 8.6 s an evaluation on one core).

The transport and the projection of every cell are independent of the other cells (numpy_reference.transport runs
per ray, numpy_reference.project sums per cell: src/sosfuse2/backends/numpy_reference.py:467-711), so the cells are
dealt round-robin to the processes, each runs sos_oracle on its share, and the per-cell results are put back in cell
order: the same arithmetic as one process, bit for bit. Composition, observer sums and the Anderson loop run in the
calling process (sos_oracle.compose / boxes' reduction / anderson_solve).

The pool uses the `spawn` start method, so it may be created after CUDA is initialised in the caller.
"""

import contextlib
import multiprocessing as mp
import os
import tempfile

import numpy as np

from . import sos_oracle as so

_PK = None
_FP64 = False


def _init(path, fp64):
    global _PK, _FP64
    for k in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
        os.environ[k] = '1'
    _PK = so.StatePack(path)
    _FP64 = fp64


def _bundle(prefix, cells):
    """The rays and segments of the listed cells of bundle `prefix`, in order."""
    b = _PK.bundle(prefix)
    off = b['cell_off']
    rays = np.concatenate([np.arange(off[i], off[i + 1]) for i in cells])
    seg_off = b['seg_off']
    segs = np.concatenate([np.arange(seg_off[r], seg_off[r + 1]) for r in rays]) if len(rays) else np.zeros(0, int)
    counts = seg_off[rays + 1] - seg_off[rays]
    out = dict(cell_off=np.r_[0, np.cumsum([off[i + 1] - off[i] for i in cells])].astype(np.int64),
               p=b['p'][cells], target=b['target'][cells], seg_off=np.r_[0, np.cumsum(counts)].astype(np.int64),
               seg_a=b['seg_a'][segs], seg_b=b['seg_b'][segs], seg_lower=b['seg_lower'][segs])
    for k in ('d', 'dloc', 'weight', 'end_j', 'end_f', 'end_col', 'end_st', 'hits'):
        if k in b:
            out[k] = b[k][rays]
    return out


def _run(job):
    kind, cells, field, first, boundary, ground_only = job
    if _FP64:
        from .fp64 import float64

        ctx = float64()
    else:
        ctx = contextlib.nullcontext()
    with ctx:
        if kind == 'cell':
            b = _bundle('cell', cells)
            rad = so.transport(_PK, b, field, first, boundary)
            return so.project(_PK, b, rad, ground_only=ground_only)
        b = _bundle('query', cells)
        return so.transport(_PK, b, field, first=False, query=True)


class ParallelOracle:
    """Solver.initialize/apply/boxes/solve of sos_oracle.Oracle with the per-cell work on `procs` processes
    (default: every host core). fp64=True runs every process's share in float64 (oracle/fp64.py)."""

    def __init__(self, arrays, procs=None, fp64=False):
        self.pk = so.StatePack(dict(arrays) if isinstance(arrays, dict) else arrays)
        with tempfile.NamedTemporaryFile(suffix='.npz', delete=False) as f:
            np.savez(f, **self.pk.arrays)
            self.path = f.name
        self.procs = int(procs or os.cpu_count() or 1)
        self.fp64 = fp64
        self.pool = mp.get_context('spawn').Pool(self.procs, initializer=_init, initargs=(self.path, fp64))
        self.first_moments = None
        self.first_flux = None

    def close(self):
        if self.pool is not None:
            self.pool.terminate()
            self.pool.join()
            self.pool = None
            os.unlink(self.path)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _deal(self, n):
        parts = min(self.procs, n)
        return [list(range(i, n, parts)) for i in range(parts)]

    def evaluate(self, field, first=False, phase=0, boundary=None):
        """TransientGeometry.evaluate over the whole cell bundle (phase 1: the nc surface cells, flux only)."""
        pk = self.pk
        n = pk.nc if phase == 1 else pk.ns
        shares = self._deal(n)
        field = np.asarray(field, np.float64 if self.fp64 else np.float32)
        res = self.pool.map(_run, [('cell', c, field, first, boundary, phase == 1) for c in shares])
        moments = np.zeros((n, 4 + pk.K, pk.W))
        flux = np.zeros((n, pk.W))
        for c, (m, f) in zip(shares, res):
            moments[c] = m
            flux[c] = f
        return moments, flux

    def initialize(self):
        if self.first_moments is None:
            pk = self.pk
            self.first_moments, self.first_flux = self.evaluate(np.zeros(pk.shape, np.float32), first=True)

    def apply(self, field):
        self.initialize()
        pk = self.pk
        _, flux = self.evaluate(field, phase=1)
        moment, _ = self.evaluate(field, phase=0, boundary=flux + self.first_flux[: pk.nc])
        if self.fp64:
            from .fp64 import float64

            with float64():
                return so.compose(pk, moment + self.first_moments)
        return so.compose(pk, moment + self.first_moments)

    def radiance(self, field):
        """Observer-ray radiance [rays, W, 4] of the query bundle (its cells are the observer positions)."""
        pk = self.pk
        nq = len(pk['query_cell_off']) - 1
        shares = self._deal(nq)
        field = np.asarray(field, np.float64 if self.fp64 else np.float32)
        res = self.pool.map(_run, [('query', c, field, False, None, False) for c in shares])
        off = pk['query_cell_off']
        out = np.zeros((int(off[-1]), pk.W, 4))
        for c, r in zip(shares, res):
            rays = np.concatenate([np.arange(off[i], off[i + 1]) for i in c])
            out[rays] = r
        return out

    def boxes(self, field):
        """sos_oracle.boxes with the observer transport on the pool."""
        pk = self.pk
        rad = self.radiance(field)
        I = rad[..., :3].astype(np.float64).sum(-1) * pk['solar'][None, :]
        pts = int(pk.meta['box_points'])
        I = I.reshape(-1, pk.meta['n_dirs'], pts, pk.W)
        return np.einsum('hdnw,n->hdw', I, pk['box_ww'])

    def solve(self, max_eval=None, tolerance=None, initial=None, log=None):
        pk = self.pk
        return so.anderson_solve(self.apply, self.boxes, pk.shape,
                                 pk.meta['max_eval'] if max_eval is None else max_eval,
                                 pk.meta['tolerance'] if tolerance is None else tolerance, initial,
                                 monitors=int(pk.meta.get('monitors', 5)), log=log)
