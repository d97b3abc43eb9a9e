#!/usr/bin/env python
"""Benchmark: converged solves per second on one GB300, learned start + batched solves against plain solves.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--batch S]

Workload (the batched configuration): 64 seeded states of uneven sizes (state i: seed 1000 + i, height levels
U{121..481} on 0-120 km, 8-64 wavelengths on 400-700 nm, L in {16, 24, 32, 48}, observer solar elevations +6 to -18
deg at 1 or 2 deg, AOD U(0.02, 0.5), g U(0.5, 0.8), ozone U(250, 400) DU, albedo U(0.05, 0.8); sosfuse2_gb300.synth
.config3), built before the timed region. A step solves one slice of S states (steps cycle through the 64 states)
from their uploaded handles: the learned start (one network per SH order, trained before the timed region on solves
the method generates) and the batched driver (every state's first evaluation, then its solve graph, on its own
stream). Every form stops at tolerance 1e-4 (TOL); `value` counts the converged solves whose observer radiance lies within
1e-3 of the state's fixed point (its plain solve to tolerance 1e-6).
`forms` times the same slices with the plain start batched and solved one at a time (`sequential`, the plain
GB300 SOS), and adds the plain config-0 solve (its dominant kernel's roofline), the projection precision forms,
make_table and the ground preparation. `e2e` is the headline form through the public API with host buffers: handles
created from host arrays, ground preparation, learned batched solve, fields read back.
`cpu_baseline` and the `--impl reference` arm time the CPU port of the reference algorithm (oracle/) on the host
cores, on a bounded sample of the same workload (sample cells of a state, one per process; geometry by the NumPy
restatements, so no native library is loaded) and scale it to whole solves.

Multi-GPU: solves are independent, so N ranks run N replicas (weak scaling, no collective on the data path); the
barrier and the max over ranks only bracket the timing.
"""

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = 'converged solves/s on 1 GB300 at ≤1e-3 rel err: learned-start+batched vs plain'
# Every form stops at TOL (the reference's stopping rule, max(observer change, source change) <= TOL from the second
# evaluation); its error is then checked against the state's fixed point (a solve to TRUTH_TOL). At the reference's
# default 1e-3 the rule bounds the last change, not the error: plain solves stopped there land up to 4.3e-3 from the
# fixed point on these states, so the timed forms stop at 1e-4, within the reference's budget of 64 evaluations.
TOL = 1e-4
TRUTH_TOL = 1e-6
MAX_EVAL = 64
L2_BYTES = 129 << 20
N_STATES = 64
WORKLOAD = ('batched configuration: 64 seeded states (seeds 1000-1063) of uneven sizes: heights U{121..481} on 0-120 '
            'km x 10 solar-zenith nodes, 8-64 wavelengths 400-700 nm, L in {16,24,32,48}, observer elevations +6..-18 '
            'deg at 1 or 2 deg, AOD 0.02-0.5, g 0.5-0.8, ozone 250-400 DU, albedo 0.05-0.8, NO2 and O4 on, '
            'stratospheric layer, nmu 1, nphi 2, path_n 4; stop tolerance 1e-4, at most 64 evaluations')


# ------------------------------------------------------------------------------------------------ helpers
def args_():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=8)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='gb300', choices=('gb300', 'reference'))
    p.add_argument('--batch', type=int, default=8, help='states per step (a slice of the 64)')
    p.add_argument('--states', type=int, default=N_STATES, help='states of the workload used (first n)')
    p.add_argument('--train-solves', type=int, default=48, help='training solves per SH order')
    p.add_argument('--epochs', type=int, default=30)
    p.add_argument('--no-cpu-baseline', action='store_true')
    p.add_argument('--no-forms', action='store_true', help='the headline form only')
    p.add_argument('--precision-only', action='store_true',
                   help='only the precision form (projection forms on a 30-wavelength state), one JSON line')
    p.add_argument('--ground-only', action='store_true',
                   help='only the ground-preparation form (host against device, a config-0 family state)')
    p.add_argument('--plain-only', action='store_true', help='only the plain config-0 single-state solve')
    p.add_argument('--profile-state', default=None, metavar='NH,W,L',
                   help='the capture target of the committed ncu summaries: a state of the batched construction with '
                        'NH heights, W wavelengths and order L (amounts of state 3), solved twice with every kernel '
                        'launched directly (no solve graph)')
    return p.parse_args()


def _c3_build(i):
    """Batched state i for the GPU arm (spawned worker): packed arrays without ground arrays, and the inputs of its
    device ground preparation (the geometry's ground rays, FP64 extinction, albedo)."""
    from sosfuse2_gb300 import synth

    sp = synth.config3_spec(i)
    fam = synth.config3_family(i)
    arrays = synth.config3(i, fam, ground=False)
    a = {k: sp[k] for k in ('aod', 'g', 'ozone_du', 'albedo')}
    atm = synth.Atmosphere(fam.shape.wl, seed=sp['seed'], top=synth.CONFIG3_TOP, no2_column=5e15, o4=True, **a)
    ground = dict(rays=fam.ground_rays(), ext=atm.ext(), strato_ext=atm.strato_ext if atm.strato else None,
                  albedo=atm.albedo)
    return i, arrays, ground


def build_config3(indices):
    """The batched states `indices` (in order), built on every host core."""
    import multiprocessing as mp

    procs = max(1, min(len(indices), os.cpu_count() or 1, 16))
    with mp.get_context('spawn').Pool(procs) as pool:
        out = pool.map(_c3_build, list(indices))
    return [(arrays, ground) for _, arrays, ground in sorted(out, key=lambda r: r[0])]


def pinned_item(arrays, ground):
    """A copy of a state's host arrays (and its ground rays) in page-locked memory, the e2e form's inputs."""
    import torch

    def pin(v):
        if isinstance(v, np.ndarray) and v.nbytes >= 4096:
            return torch.from_numpy(np.ascontiguousarray(v)).pin_memory().numpy()
        return v

    return ({k: pin(v) for k, v in arrays.items()},
            dict(ground, rays={k: pin(v) for k, v in ground['rays'].items()}))


def state_bytes(arrays, ground):
    """Host bytes a handle uploads: the packed arrays and the ground rays."""
    n = sum(v.nbytes for k, v in arrays.items() if hasattr(v, 'nbytes'))
    return n + sum(v.nbytes for v in ground['rays'].values())



class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, device_index=0):
        self.file = tempfile.NamedTemporaryFile('w+', suffix='.csv', delete=False)
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(device_index), '--query-gpu=' + self.FIELDS,
                                          '--format=csv,noheader,nounits', '-lms', '200'], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return dict(sm_mhz=None, sm_max_mhz=None, reasons=['nvidia-smi unavailable'])
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.file.seek(0)
        rows = [r.split(', ') for r in self.file.read().strip().splitlines() if r.count(',') >= 8]
        os.unlink(self.file.name)
        if not rows:
            return dict(sm_mhz=None, sm_max_mhz=None, reasons=['no samples'])
        sm = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace('.', '').isdigit()]
        names = ('hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap')
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.strip() == 'Active'})
        return dict(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=max(mx) if mx else None,
                    reasons=reasons, samples=len(rows))


def peaks():
    try:
        m = json.loads((ROOT / 'MEASURED_PEAKS.json').read_text())
        return float(m['hbm_gbs']), 'measured'
    except (OSError, ValueError, KeyError):
        return 6800.0, 'fallback'


def profiled_traffic(kernel, key='traffic_bytes_per_launch'):
    """DRAM bytes per launch of `kernel` from the committed ncu summary (profiles/*.txt, 'traffic_bytes_per_launch'),
    or per unit of work with key 'traffic_bytes_per_unit'."""
    for f in sorted((ROOT / 'profiles').glob('*.txt')):
        for line in f.read_text().splitlines():
            if line.startswith(f'{key} {kernel} '):
                try:
                    return float(line.split()[2])
                except ValueError:
                    pass
    return None


def transport_bytes(state):
    """Algorithmic (compulsory) DRAM bytes of one transport launch of each kind.

    first (full geometry, one launch per solve; it also writes the node table): per ray its geometry (48 B direction
    words, 16 B local direction, 4+4+4+4 B azimuth, cell, offsets, end interval, 24 B end columns, 1 B hit flag), per
    segment 16 B ends and 1 B flag, per cell 24 B start and 36 B frame, the node table written (32 + 4 W B per node)
    and the output radiance (16 B per ray and wavelength).
    ground, warm, observer (node-table launches, 4 per evaluation): per node the table (32 + 4 W B), per ray 48 B
    direction words, 16 B local direction, 4 B cell, 4 B segment offset and the 16 W B output, per cell 60 B, the
    field's 4 Rayleigh slots and the SH plane (4 + K floats per cell and wavelength) read once, and for rays that
    end on the ground 29 B of boundary data."""
    a = state.arrays
    W, K, ns, nc = state.W, state.K, state.ns, state.nc
    node_b = 32 + 4 * W

    def bundle(prefix, nq, cells=None):
        off = a[prefix + '_cell_off']
        seg = a[prefix + '_seg_off']
        n = len(off) - 1 if cells is None else cells
        rays = int(off[n])
        segs = int(seg[rays])
        hits = int(np.count_nonzero(a[prefix + '_hits'][:rays]))
        return rays, segs, segs * nq, n, hits

    nq, nqq = int(state.meta['nq']), int(state.meta['nq_query'])
    field = ns * (4 + K) * W * 4
    r, sg, nodes, n, _ = bundle('cell', nq)
    first = r * (48 + 16 + 16 + 24 + 1) + sg * 17 + n * 60 + nodes * node_b + r * W * 16

    def table(prefix, q, cells=None, boundary=False):
        rays, _, nodes, n, hits = bundle(prefix, q, cells)
        return nodes * node_b + rays * (48 + 16 + 8 + 16 * W) + n * 60 + field + (hits * 29 if boundary else 0)

    return dict(first=first, ground=table('cell', nq, nc), warm=table('cell', nq, boundary=True),
                observer=table('query', nqq))


def whole_job(value, world, dist=None):
    """Whole-job throughput of `world` replicas from this rank's own: the slowest rank's rate times the ranks (the
    max-over-ranks time of equal work per rank)."""
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64)
    if dist is not None and world > 1:
        if dist.get_backend() == 'nccl':
            t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.MIN)
    return float(t.item()) * world


def bracket(dist):
    """Barrier and device synchronisation on both sides of a timed region."""
    import torch

    if dist is not None:
        dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


# ------------------------------------------------------------------------------------------------ CPU baseline
# Evaluations of each batched state's plain GB300 solve (tolerance 1e-4, at most 64 evaluations) and whether it
# converged, measured by this benchmark's GPU arm (forms.sequential.per_state): the CPU port's per-evaluation cost is
# scaled to whole solves with them, because the CPU port's own solve of one of these states takes hours; on the
# config-0-grid states the parity tests show the CUDA solve and the oracle reach the same evaluation count.
CONFIG3_EVALUATIONS = {0: (64, False), 1: (13, True), 2: (15, True), 3: (11, True), 4: (10, True), 5: (16, True),
    6: (20, True), 7: (12, True), 8: (64, False), 9: (10, True), 10: (12, True), 11: (14, True), 12: (64, False),
    13: (64, False), 14: (64, False), 15: (22, True), 16: (13, True), 17: (64, False), 18: (64, False),
    19: (13, True), 20: (19, True), 21: (11, True), 22: (10, True), 23: (64, False), 24: (13, True), 25: (64, False),
    26: (12, True), 27: (9, True), 28: (64, False), 29: (64, False), 30: (10, True), 31: (64, False),
    32: (64, False), 33: (64, False), 34: (64, False), 35: (15, True), 36: (64, False), 37: (13, True),
    38: (11, True), 39: (64, False), 40: (64, False), 41: (64, False), 42: (15, True), 43: (11, True),
    44: (11, True), 45: (55, True), 46: (14, True), 47: (23, True), 48: (14, True), 49: (18, True), 50: (14, True),
    51: (64, False), 52: (17, True), 53: (64, False), 54: (11, True), 55: (64, False), 56: (64, False),
    57: (17, True), 58: (10, True), 59: (15, True), 60: (64, False), 61: (64, False), 62: (14, True),
    63: (64, False)}

_TABLE = None


def _cpu_init(table):
    global _TABLE
    for k in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
        os.environ[k] = '1'
    _TABLE = table


def _cpu_cell(job):
    """One process, one sample cell of batched state i: the CPU port's (oracle/) first light and one evaluation of
    that cell (its warm pass, and its ground pass when it is a surface cell) on the state's own optics, and with
    row >= 0 the observer transport of that observer row. Geometry by the NumPy restatements (no native library).
    Returns the core-seconds of each part."""
    i, cell, row = job
    from oracle import sos_oracle as so
    from sosfuse2_gb300 import synth

    with synth.numpy_geometry():
        fam = synth.config3_family(i, cells=[cell], table=_TABLE)
        arrays = synth.config3(i, fam)
    pk = so.StatePack(arrays)
    x = np.full(pk.shape, 1e-3, np.float32)  # a nonzero source: the warm pass's trace blend takes its full path
    b = pk.bundle('cell')
    t0 = time.process_time()
    so.project(pk, b, so.transport(pk, b, x, first=True))
    t1 = time.process_time()
    so.project(pk, b, so.transport(pk, b, x, first=False, boundary=np.ones((pk.nc, pk.W))))
    t2 = time.process_time()
    surface = cell < pk.nc
    if surface:
        so.project(pk, b, so.transport(pk, b, x, first=False), ground_only=True)
    t3 = time.process_time()
    obs = 0.0
    if row >= 0:
        q = pk.bundle('query')
        off, so_ = q['cell_off'], q['seg_off']
        r0, r1 = int(off[row]), int(off[row + 1])
        s0, s1 = int(so_[r0]), int(so_[r1])
        sub = dict(cell_off=np.array([0, r1 - r0]), p=q['p'][row:row + 1], target=q['target'][row:row + 1],
                   seg_off=so_[r0:r1 + 1] - s0, seg_a=q['seg_a'][s0:s1], seg_b=q['seg_b'][s0:s1],
                   seg_lower=q['seg_lower'][s0:s1])
        for k in ('d', 'dloc', 'weight', 'end_j', 'end_f', 'end_col', 'end_st', 'hits'):
            if k in q:
                sub[k] = q[k][r0:r1]
        t4 = time.process_time()
        so.transport(pk, sub, x, first=False, query=True)
        obs = time.process_time() - t4
    return dict(first=t1 - t0, warm=t2 - t1, ground=t3 - t2, surface=bool(surface), obs=obs)


def cpu_state(pool, procs, i):
    """The CPU port on batched state i: one sample cell per process (cells spread evenly over the state's grid) and
    one observer row, timed in core-seconds and scaled by cell and row counts to one solve: first light + E x
    (ground pass + warm pass + 2 observer passes), E the state's evaluations (CONFIG3_EVALUATIONS)."""
    from sosfuse2_gb300 import synth

    sp = synth.config3_spec(i)
    nc = len(synth.REDUCED_CHI_DEG)
    ns = sp['nh'] * nc
    cells = np.unique(np.linspace(0, ns - 1, max(procs, 2)).astype(int))
    cells = np.unique(np.r_[cells, np.arange(0, nc, max(1, nc // 2))])  # surface cells for the ground pass
    t = time.perf_counter()
    res = pool.map(_cpu_cell, [(i, int(c), 0 if k == 0 else -1) for k, c in enumerate(cells)])
    wall = time.perf_counter() - t
    surf = [r for r in res if r['surface']]
    rows = len(np.arange(6.0, -18.0 - 1e-9, -float(sp['solar_step'])))
    E, conv = CONFIG3_EVALUATIONS[i]
    first = sum(r['first'] for r in res) / len(res) * ns
    warm = sum(r['warm'] for r in res) / len(res) * ns
    ground = (sum(r['ground'] for r in surf) / max(len(surf), 1)) * nc
    obs = res[0]['obs'] * rows
    solve = first + E * (ground + warm + 2 * obs)
    return dict(state=i, core_seconds=solve, evaluations=E, converged=bool(conv), wall=wall, cells=len(cells),
                first_per_cell=first / ns, warm_per_cell=warm / ns, observer_row=res[0]['obs'])


def native_loaded():
    """Shared objects of this repository mapped into this process (none on the CPU arm)."""
    try:
        maps = Path('/proc/self/maps').read_text()
    except OSError:
        return None
    return sorted({line.split()[-1] for line in maps.splitlines() if str(ROOT) in line and '.so' in line})


class CpuPort:
    """The pool of the CPU port (spawned, one process per host core) with the shared solar column table."""

    def __init__(self, procs=None):
        import multiprocessing as mp

        from sosfuse2_gb300 import synth

        self.procs = int(procs or os.cpu_count() or 1)
        with synth.numpy_geometry():
            table = synth.config3_table()
        self.pool = mp.get_context('spawn').Pool(self.procs, initializer=_cpu_init, initargs=(table,))

    def close(self):
        self.pool.terminate()
        self.pool.join()

    def run(self, states):
        """Samples of `states` (one step each): (whole-machine converged solves/s of the workload, per-step records):
        the processes over the mean core-seconds of a solve of the sampled states, times the workload's fraction of
        converged solves (CONFIG3_EVALUATIONS)."""
        recs = [cpu_state(self.pool, self.procs, i) for i in states]
        mean_core = sum(r['core_seconds'] for r in recs) / len(recs)
        frac = sum(c for _, c in CONFIG3_EVALUATIONS.values()) / len(CONFIG3_EVALUATIONS)
        return self.procs * frac / mean_core, recs


def cpu_description(procs, recs):
    return (f'{len(recs)} batched states (indices {[r["state"] for r in recs]}), each {recs[0]["cells"]} sample '
            f'cells (one per process on {procs} processes) and one observer row timed in core-seconds (first light '
            f'and one evaluation), scaled by cells and rows to one solve with the state\'s plain GB300 evaluation '
            f'count; solves/s = processes / mean core-seconds per solve x the workload\'s converged fraction')


def run_reference(a, rank):
    """The CPU port (oracle/) of the reference algorithm on the host cores: one step = one batched state's sample
    (states in order), as cpu_state; value = whole-machine converged solves/s of the timed steps."""
    if rank != 0:
        return
    port = CpuPort()
    try:
        n = max(a.states, 1)
        for s in range(a.warmup):
            port.run([s % n])
        t0 = time.perf_counter()
        value, recs = port.run([(a.warmup + s) % n for s in range(a.steps)])
        wall = time.perf_counter() - t0
    finally:
        port.close()
    cb = dict(value=value, unit='solves/s', cores=port.procs, kind='port', nproc=os.cpu_count(),
              sample=cpu_description(port.procs, recs), states=recs, native_libraries_loaded=native_loaded())
    print(json.dumps(dict(
        impl='reference', metric=METRIC, value=value, unit='solves/s', n_gpus=a.gpus, steps=a.steps, warmup=a.warmup,
        ms_per_step=wall / max(a.steps, 1) * 1e3, higher_is_better=True, scaling='weak', vs_baseline=None,
        dtype='f32', data='synthetic', config=dict(workload=WORKLOAD, note='CPU port of the reference algorithm '
                                                   '(oracle/); each step a bounded sample of one state'),
        cpu_baseline=cb, e2e=dict(value=value, unit='solves/s', h2d_bytes_per_step=0, d2h_bytes_per_step=0))),
        flush=True)


PRECISION_MODES = {'fp32': 0, 'bf16x3': 1, 'tf32': 2, 'bf16': 3}


def _precision_form(device):
    """Projection forms on a 30-wavelength state (400-700 nm, L=32, 61 heights on 0-120 km, the config-0 solar-zenith
    grid, nmu 1, nphi 2, path_n 4, NO2 and O4 on): per form one converged solve, its evaluations and time, the
    projection time per warm evaluation, and the max / RMS relative error of the converged observer radiance (box
    values above 1e-6 of the largest) against the FP32 CUDA-core form."""
    import torch

    from sosfuse2_gb300 import _abi, synth
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    arrays = synth.config1(seed=0, nh=61, nmu=1, nphi=2, path_n=4, chi_deg=synth.REDUCED_CHI_DEG)
    state = PackedState(arrays)
    out, boxes = {}, {}
    for name, mode in PRECISION_MODES.items():
        solver = Solver(state, device=device)
        k = solver.kernel
        k._check(k.lib.sosb_set_projection(k.h, mode))
        solver.solve(64, 1e-3, device_out=True)  # warm-up: tables and basis
        torch.cuda.synchronize()
        ncls = len(_abi.KERNEL_CLASSES)
        k.lib.sosb_set_timing(k.h, 1)
        t0 = time.perf_counter()
        x, st = solver.solve(64, 1e-3, device_out=True)
        torch.cuda.synchronize()
        seconds = time.perf_counter() - t0
        ms = (_abi.c_dbl * ncls)()
        cnt = (_abi.c_i64 * ncls)()
        k.lib.sosb_get_timing(k.h, ms, cnt, ncls)
        k.lib.sosb_set_timing(k.h, 0)
        boxes[name] = solver.boxes(x)
        out[name] = dict(evaluations=st['evaluations'], solve_ms=seconds * 1e3,
                         projection_ms_per_evaluation=ms[1] / max(st['evaluations'] + 1, 1))
        k.close()
    ref = boxes['fp32']
    big = np.abs(ref) > 1e-6 * np.abs(ref).max()
    for name in out:
        rel = np.abs(boxes[name][big] - ref[big]) / np.abs(ref[big])
        out[name].update(max_rel=float(rel.max()), rms_rel=float(np.sqrt(np.mean(rel ** 2))))
    return dict(workload=f'30 wavelengths 400-700 nm, L=32, 61 heights 0-120 km x 10 solar-zenith nodes, nmu 1, '
                         f'nphi 2, path_n 4 ({state.meta["rays"]} rays); errors of the converged observer radiance '
                         f'against the fp32 form', forms=out)


def _table_form(fam, device):
    """make_table on the reference's full table axes (25 solar elevations +6..-18 deg, 100 x 180 views, one
    wavelength) for the converged source of a config-0 family state: the call's seconds (view rays built on the host,
    a handle, first-order and multiple-scattering phase-2 transports) and table entries per second."""
    import torch

    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState
    from sosfuse2_gb300.synth import family_state
    from sosfuse2_gb300.table import axes, make_table

    for seed in range(90001, 90017):  # the first held-out state the plain iteration converges on
        state = PackedState(family_state(fam, seed))
        solver = Solver(state, device=device)
        try:
            field, st = solver.solve(int(state.meta['max_eval']), float(state.meta['tolerance']), device_out=True)
            break
        except RuntimeError as exc:
            solver.kernel.close()
            if not str(exc).startswith('E_NOT_CONVERGED'):
                raise
    _, hs, el, az = axes(False)
    make_table(solver, field, hs[:1], el[:4], az[:4], log=lambda m: None, family=fam)  # warm-up: module and handle
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    table, seconds = make_table(solver, field, hs, el, az, log=lambda m: None, family=fam)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    solver.kernel.close()
    rays = len(hs) * len(el) * len(az)
    return dict(workload=f'config-0 family state {seed} ({st["evaluations"]} evaluations), {len(hs)} solar elevations x '
                         f'{len(el)} x {len(az)} views, W={state.W}', rays=rays, seconds=dt,
                rays_per_s=rays / dt, batches=len(seconds))


def _ground_form(fam, device):
    """Per-state ground preparation (engine_core.Solver.prepare_ground) of a config-0 family state: the host form
    (synth.Family.ground, NumPy FP64) against sosb_prepare_ground on the device (CUDA events not needed: the call
    synchronises), each the mean of five calls after one untimed call."""
    import torch

    from sosfuse2_gb300.solver import Kernel
    from sosfuse2_gb300.state import PackedState
    from sosfuse2_gb300.synth import family_atmosphere

    atm = family_atmosphere(fam, 90002)
    ext = atm.ext()
    fam.ground(atm, ext)
    t0 = time.perf_counter()
    for _ in range(5):
        fam.ground(atm, ext)
    host_ms = (time.perf_counter() - t0) / 5 * 1e3
    k = Kernel(PackedState(fam.state(atm, 90002, ground=False)), device)
    rays = fam.ground_rays()
    k.set_ground_rays(rays)
    st_ext = atm.strato_ext if atm.strato else None
    k.prepare_ground(atm.albedo, ext, st_ext)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(5):
        k.prepare_ground(atm.albedo, ext, st_ext)
    dev_ms = (time.perf_counter() - t0) / 5 * 1e3
    k.close()
    return dict(workload=f'config-0 family state 90002: {len(rays["cell"])} ground rays over {fam.h.size * fam.chi.size} '
                         f'cells, W={atm.W}', host_ms=host_ms, device_ms=dev_ms)


# ------------------------------------------------------------------------------------------------ GPU arm
def make_kernels(items, device):
    """One handle per state (arrays, ground inputs): bundles and constants uploaded, ground prepared on the device,
    then each handle on its own stream."""
    from sosfuse2_gb300.solver import Kernel
    from sosfuse2_gb300.state import PackedState

    ks, sts = [], []
    for arrays, ground in items:
        st = PackedState(arrays)
        k = Kernel(st, device)
        k.set_ground_rays(ground['rays'])
        k.prepare_ground(ground['albedo'], ground['ext'], ground['strato_ext'])
        ks.append(k)
        sts.append(st)
    import torch

    torch.cuda.synchronize()
    for k in ks:
        k._check(k.lib.sosb_set_stream(k.h, None))
    return ks, sts


def truth_boxes(slices, items, device, tol=TRUTH_TOL, max_eval=256):
    """Observer radiance of each state's fixed point (plain start, batched, stopped at TRUTH_TOL), the reference the
    timed solves' observer radiance is held to (<= 1e-3): {state: boxes or None when it does not converge}."""
    import torch

    from sosfuse2_gb300 import _abi
    from sosfuse2_gb300.solver import Solver

    out = {}
    for idx in slices:
        ks, sts = make_kernels([items[i] for i in idx], device)
        n = len(ks)
        lib = ks[0].lib
        outs = [k.field() for k in ks]
        stats = (_abi.Stats * n)()
        status = (ctypes.c_int32 * n)()
        lib.sosb_solve_batch((ctypes.c_void_p * n)(*[k.h.value for k in ks]), n, max_eval, tol, None,
                             (ctypes.c_void_p * n)(*[o.data_ptr() for o in outs]), 1, stats, status, 0)
        for j, (i, k, st) in enumerate(zip(idx, ks, sts)):
            out[i] = None if status[j] else Solver(st, kernel=k).boxes(outs[j])
        for k in ks:
            k.close()
        del ks, sts, outs
        torch.cuda.empty_cache()
    return out


def solve_slice(form, ks, sts, nets):
    """One step of `form` on handles `ks`: 'learned' (learned start, batched), 'batched' (plain start, batched) or
    'sequential' (plain start, one solve in flight). Returns [(field, stats) or RuntimeError], kernel launches."""
    from sosfuse2_gb300 import _abi, learned

    n = len(ks)
    if form == 'learned':
        g0 = sum(w.mlp.gemm_launches for w in nets.values())
        r = learned.solve_batch(nets, ks, sts, max_eval=MAX_EVAL, tolerance=TOL)
        nl = sum(x[1]['kernel_launches'] for x in r if not isinstance(x, Exception))
        return r, nl + sum(w.mlp.gemm_launches for w in nets.values()) - g0
    lib = ks[0].lib
    handles = (ctypes.c_void_p * n)(*[k.h.value for k in ks])
    outs = [k.field() for k in ks]
    stats = (_abi.Stats * n)()
    status = (ctypes.c_int32 * n)()
    lib.sosb_solve_batch(handles, n, MAX_EVAL, TOL, None, (ctypes.c_void_p * n)(*[o.data_ptr() for o in outs]), 1,
                         stats, status, 1 if form == 'sequential' else 0)
    res = []
    for i, k in enumerate(ks):
        if status[i]:
            res.append(RuntimeError(lib.sosb_last_error(k.h).decode()))
        else:
            res.append((outs[i], dict(evaluations=int(stats[i].evaluations),
                                      kernel_launches=int(stats[i].kernel_launches))))
    return res, sum(int(stats[i].kernel_launches) for i in range(n))


def time_form(form, slices, items, nets, device, dist, clocks=None):
    """Times `form` on the listed slices (one step each): per step the handles are created and uploaded before the
    timer, the step is bracketed by a barrier and device synchronisation. After each step the observer radiance of
    every converged solve is computed (outside the timing). Returns the per-step seconds, the per-state results
    {state: (evaluations or None, boxes or None)} and the kernel launches of the timed steps."""
    import torch

    from sosfuse2_gb300.solver import Solver

    times, per_state, launches = [], {}, 0
    for idx in slices:
        ks, sts = make_kernels([items[i] for i in idx], device)
        bracket(dist)
        t0 = time.perf_counter()
        res, nl = solve_slice(form, ks, sts, nets)
        bracket(dist)
        times.append(time.perf_counter() - t0)
        launches += nl
        for i, k, st, r in zip(idx, ks, sts, res):
            if isinstance(r, Exception):
                if not str(r).startswith('E_NOT_CONVERGED'):
                    raise r
                per_state[i] = (None, None)
            else:
                per_state[i] = (r[1]['evaluations'], Solver(st, kernel=k).boxes(r[0]))
        for k in ks:
            k.close()
        del ks, sts, res
        torch.cuda.empty_cache()
    return times, per_state, launches


def rel_boxes(b, ref):
    big = np.abs(ref) > 1e-6 * np.abs(ref).max()
    return float(np.max(np.abs(b[big] - ref[big]) / np.abs(ref[big])))


def plain_config0(a, device, dist):
    """The plain config-0 solve (550 nm, 101 heights x 10 solar-zenith nodes, L=16): CUDA events around each solve
    with the L2 flushed between solves, then one more solve with per-class kernel timing (the roofline of its
    dominant kernel)."""
    import torch

    from sosfuse2_gb300 import _abi, synth
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    state = PackedState(synth.config0())
    solver = Solver(state, device=device)
    k = solver.kernel
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=k.device)
    tol, max_eval = float(state.meta['tolerance']), int(state.meta['max_eval'])
    for _ in range(max(a.warmup, 0)):
        solver.solve(max_eval, tol, device_out=True)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    step_ms, evaluations, launches = [], [], 0
    bracket(dist)
    for _ in range(a.steps):
        flush.fill_(1.0)  # L2 flush between timed solves, outside the events
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, st = solver.solve(max_eval, tol, device_out=True)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        evaluations.append(st['evaluations'])
        launches += st['kernel_launches']
    bracket(dist)
    ncls = len(_abi.KERNEL_CLASSES)
    ms = (_abi.c_dbl * ncls)()
    cnt = (_abi.c_i64 * ncls)()
    flush.fill_(1.0)
    k.lib.sosb_set_timing(k.h, 1)
    solver.solve(max_eval, tol, device_out=True)
    k.lib.sosb_get_timing(k.h, ms, cnt, ncls)
    k.lib.sosb_set_timing(k.h, 0)
    k.close()
    classes = _abi.KERNEL_CLASSES
    times = {classes[i]: dict(ms=ms[i], launches=int(cnt[i]), share=ms[i] / max(sum(ms), 1e-30)) for i in range(ncls)}
    b = transport_bytes(state)
    per_launch = (b['ground'] + b['warm'] + 2 * b['observer']) / 4
    i_tab = classes.index('transport_table')
    mean_ms = ms[i_tab] / max(cnt[i_tab], 1)
    peak, peak_kind = peaks()
    achieved = per_launch / (mean_ms / 1e3) / 1e9
    roof = dict(kernel='transport_table_kernel', bound='hbm', achieved=achieved, peak=peak, unit='GB/s',
                frac=achieved / peak, peak_source=peak_kind, traffic=profiled_traffic('transport_table_kernel'),
                bytes_per_launch=per_launch, mean_launch_ms=mean_ms,
                measured_on='CUDA events around each launch of one more plain config-0 solve')
    return dict(solves_per_s=1e3 / statistics.mean(step_ms), ms_per_solve=statistics.mean(step_ms),
                evaluations=statistics.mean(evaluations), rays=state.meta['rays'], cells=state.ns,
                kernel_times=times, roofline=roof, launches=launches,
                l2='flushed between timed solves (512 MiB write outside the events)')


def profile_state(nh, W, L, device):
    """Two plain solves (tolerance 1e-3) of one state of the batched construction (heights nh on 0-120 km, W
    wavelengths on 400-700 nm, order L, observer rows every 2 deg, the amounts of batched state 3), every kernel
    launched directly: the capture target of the ncu summaries."""
    import torch

    from sosfuse2_gb300 import synth
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

    sp = synth.config3_spec(3)
    wl = np.linspace(400.0, 700.0, W)
    shape = synth.Atmosphere(wl, seed=sp['seed'], top=synth.CONFIG3_TOP, no2_column=5e15, o4=True)
    fam = synth.Family(np.linspace(0.0, synth.CONFIG3_TOP, nh), synth.REDUCED_CHI_DEG, L, 1, 2, 4, shape,
                       name='profile', monitor_elevations=np.arange(6.0, -18.0 - 1e-9, -2.0))
    a = {k: sp[k] for k in ('aod', 'g', 'ozone_du', 'albedo')}
    atm = synth.Atmosphere(wl, seed=sp['seed'], top=synth.CONFIG3_TOP, no2_column=5e15, o4=True, **a)
    solver = Solver(PackedState(fam.state(atm, sp['seed'])), device=device)
    solver.kernel.set_graphs(False)
    out = []
    for _ in range(2):
        torch.cuda.synchronize()
        t = time.perf_counter()
        _, st = solver.solve(64, 1e-3, device_out=True)
        torch.cuda.synchronize()
        out.append(dict(seconds=time.perf_counter() - t, evaluations=st['evaluations']))
    meta = solver.state.meta
    solver.kernel.close()
    return dict(nh=nh, W=W, L=L, rays=meta['rays'], segments=meta['segments'], solves=out)


def tensor_peak():
    try:
        m = json.loads((ROOT / 'MEASURED_PEAKS.json').read_text())
        return float(m['bf16_tflops']), 'measured'
    except (OSError, ValueError, KeyError):
        return 1900.0, 'fallback'


def corner_roofline(item, device):
    """Roofline of the dominant kernel of the batched workload, the tensor-core corner values (corner_tc_kernel), on
    one of its states: CUDA events around every launch of one solve (timing mode). Algorithmic work per evaluation:
    2 K W flops per (node, corner) entry, the cell bundle once (its ground and warm pass share the plane) and the
    observer bundle twice (boxes of x and of g); executed tensor work adds the bf16x3 split (x3) and the padding of K
    to 64 and W to 16."""
    from sosfuse2_gb300 import _abi

    ks, sts = make_kernels([item], device)
    k, st = ks[0], sts[0]
    from sosfuse2_gb300.solver import Solver

    solver = Solver(st, kernel=k)
    k._check(k.lib.sosb_set_stream(k.h, None))
    try:
        solver.solve(MAX_EVAL, TOL, device_out=True)  # tables, entries, tuning
    except RuntimeError:
        pass
    ncls = len(_abi.KERNEL_CLASSES)
    ms = (_abi.c_dbl * ncls)()
    cnt = (_abi.c_i64 * ncls)()
    k.lib.sosb_set_timing(k.h, 1)
    try:
        _, stt = solver.solve(MAX_EVAL, TOL, device_out=True)
        E = stt['evaluations']
    except RuntimeError:
        E = len(solver.history())
    k.lib.sosb_get_timing(k.h, ms, cnt, ncls)
    k.lib.sosb_set_timing(k.h, 0)
    k.close()
    m = st.meta
    K, W = st.K, st.W
    cell_entries = 4 * len(st['cell_seg_a']) * int(m['nq'])
    obs_entries = 4 * len(st['query_seg_a']) * int(m['nq_query'])
    i = _abi.KERNEL_CLASSES.index('corner')
    flops = 2.0 * K * W * (cell_entries + 2 * obs_entries) * E
    executed = flops * 3 * (math.ceil(K / 64) * 64 / K) * (math.ceil(W / 16) * 16 / W)
    sec = ms[i] / 1e3
    peak, kind = tensor_peak()
    achieved = flops / sec / 1e12
    classes = _abi.KERNEL_CLASSES
    share = {classes[j]: ms[j] / max(sum(ms[c] for c in range(ncls) if classes[c] != 'corner'), 1e-30)
             for j in range(ncls)}
    per_unit = profiled_traffic('corner_tc_kernel', 'traffic_bytes_per_unit')
    # DRAM bytes of the average launch (cell bundle once, observer bundle twice per evaluation): the bytes per
    # (entry, wavelength) of the committed capture (profiles/corner_tc_kernel_profile_state.txt, a smaller state)
    # times this state's units per launch
    traffic = per_unit * (cell_entries + 2 * obs_entries) / 3.0 * W if per_unit is not None else None
    return dict(kernel='corner_tc_kernel', bound='tensor', achieved=achieved, peak=peak, unit='TFLOP/s',
                frac=achieved / peak, peak_source=kind, traffic=traffic,
                traffic_source='profiles/corner_tc_kernel_profile_state.txt: DRAM bytes per (entry, wavelength) of '
                               'the profile state, scaled by this state\'s entries x W per launch',
                flops_per_evaluation=flops / max(E, 1), executed_tflops=executed / sec / 1e12,
                mean_launch_ms=ms[i] / max(cnt[i], 1), launches=int(cnt[i]), evaluations=E,
                state=m['config3'], class_ms={classes[j]: ms[j] for j in range(ncls)},
                note='the corner class is also inside transport_table (nested timer); shares exclude it',
                shares=share,
                measured_on='CUDA events around each launch of one more solve of the state (timing mode)')


def run_gb300(a, rank, world):
    import torch

    from sosfuse2_gb300 import build, learned, synth

    build.build()
    local = int(os.environ.get('LOCAL_RANK', 0))
    torch.cuda.set_device(local)
    device = f'cuda:{local}'
    if a.precision_only:
        if rank == 0:
            print(json.dumps(dict(precision=_precision_form(device))), flush=True)
        return
    if a.ground_only:
        if rank == 0:
            print(json.dumps(dict(ground=_ground_form(synth.config0_family(), device))), flush=True)
        return
    if a.profile_state:
        nh, W, L = (int(v) for v in a.profile_state.split(','))
        print(json.dumps(dict(profile_state=profile_state(nh, W, L, device))), flush=True)
        return
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group('nccl')
    plain0 = plain_config0(a, device, dist)
    if a.plain_only:
        if rank == 0:
            print(json.dumps(dict(plain_config0=plain0)), flush=True)
        return
    # ---------------------------------------------------------------- the batched configuration
    n_states = max(1, min(a.states, N_STATES))
    t0 = time.perf_counter()
    items = build_config3(range(n_states))
    build_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    orders = sorted({synth.config3_spec(i)['L'] for i in range(n_states)})
    nets, train = learned.train_config3(orders, n_train=a.train_solves, epochs=a.epochs, device=device, tolerance=TOL)
    train_s = time.perf_counter() - t0
    S = max(1, min(a.batch, n_states))
    nslices = (n_states + S - 1) // S
    slice_of = lambda s: list(range((s % nslices) * S, min((s % nslices + 1) * S, n_states)))  # noqa: E731
    warm = [slice_of(s) for s in range(a.warmup)]
    timed = [slice_of(a.warmup + s) for s in range(a.steps)]
    time_form('learned', warm, items, nets, device, dist)
    clocks = Clocks(local)
    t_learn, r_learn, l_learn = time_form('learned', timed, items, nets, device, dist)
    clk = clocks.stop()
    one_pass = []  # the comparison forms: the timed slices, each once
    for sl in timed:
        if sl not in one_pass:
            one_pass.append(sl)
    forms = {}
    if not a.no_forms:
        t_seq, r_seq, l_seq = time_form('sequential', one_pass, items, nets, device, dist)
        t_bat, r_bat, l_bat = time_form('batched', one_pass, items, nets, device, dist)
    # accepted solves: converged, with observer radiance within 1e-3 of the state's fixed point (a plain solve to
    # TRUTH_TOL; a state whose tight solve does not converge keeps its converged solves unchecked)
    truth = truth_boxes(one_pass, items, device)

    def accepted(per_state, slices):
        ok, errs = [], []
        for sl in slices:
            n = 0
            for i in sl:
                ev, bx = per_state[i]
                if ev is None:
                    continue
                err = None
                if truth.get(i) is not None:
                    err = rel_boxes(bx, truth[i])
                    errs.append(err)
                n += err is None or err <= 1e-3
            ok.append(n)
        return ok, errs

    ok_learn, err_learn = accepted(r_learn, timed)
    value = sum(ok_learn) / sum(t_learn)
    value = whole_job(value, world, dist)
    launches = plain0['launches'] + l_learn
    if not a.no_forms:
        ok_seq, err_seq = accepted(r_seq, one_pass)
        ok_bat, err_bat = accepted(r_bat, one_pass)
        launches += l_seq + l_bat
        evals = lambda r, sl: [r[i][0] for s in sl for i in s if r[i][0] is not None]  # noqa: E731
        forms = dict(
            learned=dict(value=value / world, seconds_per_step=statistics.mean(t_learn), states_per_step=S,
                         steps=len(timed), converged_accepted=sum(ok_learn),
                         evaluations_mean=statistics.mean(evals(r_learn, timed) or [0]),
                         max_rel_observer_vs_fixed_point=max(err_learn) if err_learn else None),
            batched=dict(value=sum(ok_bat) / sum(t_bat), seconds_per_step=statistics.mean(t_bat), steps=len(one_pass),
                         converged_accepted=sum(ok_bat), evaluations_mean=statistics.mean(evals(r_bat, one_pass) or [0]),
                         max_rel_observer_vs_fixed_point=max(err_bat) if err_bat else None),
            sequential=dict(value=sum(ok_seq) / sum(t_seq), seconds_per_step=statistics.mean(t_seq),
                            steps=len(one_pass), converged_accepted=sum(ok_seq),
                            max_rel_observer_vs_fixed_point=max(err_seq) if err_seq else None,
                            evaluations_mean=statistics.mean(evals(r_seq, one_pass) or [0]),
                            per_state={i: r_seq[i][0] for s in one_pass for i in s}),
            training=dict(seconds=train_s, per_order={L: r for L, r in train.items()}),
            build_seconds=build_s)
        both = sorted(i for s_ in one_pass for i in s_
                      if r_learn.get(i, (None, None))[0] is not None and r_seq.get(i, (None, None))[0] is not None)
        forms['paired_evaluations'] = dict(
            states=len(both), plain=statistics.mean([r_seq[i][0] for i in both]) if both else None,
            learned=statistics.mean([r_learn[i][0] for i in both]) if both else None,
            note='states both starts converge on; learned counts the apply(0) that feeds the network')
        forms['learned_vs_plain_batched'] = forms['learned']['value'] / max(forms['batched']['value'], 1e-30)
        forms['learned_batched_vs_plain_sequential'] = (forms['learned']['value']
                                                         / max(forms['sequential']['value'], 1e-30))
        forms['batched_vs_sequential'] = forms['batched']['value'] / max(forms['sequential']['value'], 1e-30)
        forms['plain_config0'] = plain0
        forms['precision'] = _precision_form(device)
        fam = synth.config0_family()
        forms['table'] = _table_form(fam, device)
        forms['ground'] = _ground_form(fam, device)
    # ---------------------------------------------------------------- end to end through the public API
    # Every step: handles created from the host arrays in page-locked memory (bundles, constants, ground rays
    # uploaded), ground prepared on the device, the learned batched solve, and the converged fields read back into
    # page-locked host buffers. The page-locked copies and buffers are made before the timer.
    from sosfuse2_gb300.state import PackedState

    e2e_t, e2e_conv, h2d, d2h = [], 0, 0, 0
    e2e_parts = dict(create_s=0.0, solve_s=0.0, read_s=0.0)
    for sl in timed:  # the states of the timed steps of `value`, so that both count the same solves
        host = [pinned_item(*items[i]) for i in sl]
        outs = [torch.empty(tuple(PackedState(arr).shape), dtype=torch.float32, pin_memory=True) for arr, _ in host]
        bracket(dist)
        t0 = time.perf_counter()
        ks, sts = make_kernels(host, device)
        t1 = time.perf_counter()
        res, _ = solve_slice('learned', ks, sts, nets)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        fields = []
        for o, r in zip(outs, res):
            if not isinstance(r, Exception):
                o.copy_(r[0])
                fields.append(o.numpy())
        bracket(dist)
        e2e_parts['create_s'] += t1 - t0
        e2e_parts['solve_s'] += t2 - t1
        e2e_parts['read_s'] += time.perf_counter() - t2
        e2e_t.append(time.perf_counter() - t0)
        e2e_conv += len(fields)
        h2d += sum(state_bytes(*items[i]) for i in sl)
        d2h += sum(f.nbytes for f in fields)
        for k in ks:
            k.close()
        torch.cuda.empty_cache()
    e2e = dict(value=world * e2e_conv / sum(e2e_t), unit='solves/s', h2d_bytes_per_step=int(h2d / len(e2e_t)),
               d2h_bytes_per_step=int(d2h / len(e2e_t)),
               seconds_per_step={k: v / len(e2e_t) for k, v in e2e_parts.items()},
               host_memory='inputs and outputs page-locked')
    if rank != 0:
        return
    cb = None
    if world == 1 and not a.no_cpu_baseline:
        port = CpuPort()
        try:
            v, recs = port.run([timed[0][0], timed[0][-1]])
        finally:
            port.close()
        cb = dict(value=v, unit='solves/s', cores=port.procs, kind='port', nproc=os.cpu_count(),
                  sample=cpu_description(port.procs, recs))
    roof = corner_roofline(items[3 if n_states > 3 else 0], device)
    out = dict(
        metric=METRIC, value=value, unit='solves/s', n_gpus=world, steps=a.steps, warmup=a.warmup,
        ms_per_step=statistics.mean(t_learn) * 1e3, higher_is_better=True, scaling='weak', vs_baseline=None,
        dtype='f32', data='synthetic (seeded states on the reference geometry rules, sosfuse2_gb300.synth.config3)',
        config=dict(workload=WORKLOAD, states_per_step=S, form='learned start + batched solves (solve graphs)',
                    tolerance=TOL, max_eval=MAX_EVAL,
                    value_counts='converged solves whose observer radiance is within 1e-3 of the fixed point (a plain '
                                 'solve of the state to tolerance 1e-6)',
                    l2='each step reads more than the 129 MB L2 (states of 0.1-2 GB of source fields)',
                    parallelism=f'replicas x{world}'),
        forms=forms or None, roofline=roof, kernel_times=roof.pop('class_ms'), cpu_baseline=cb,
        e2e=e2e, gpu_launches=int(launches), clocks=clk)
    print(json.dumps(out, default=float), flush=True)


def main():
    a = args_()
    rank = int(os.environ.get('RANK', 0))
    world = int(os.environ.get('WORLD_SIZE', 1))
    if a.impl == 'reference':
        run_reference(a, rank)
    else:
        run_gb300(a, rank, world)


if __name__ == '__main__':
    main()
