#!/usr/bin/env python
"""Benchmark: converged SOS solves per second on one GB300 (one step = one complete Solver.solve).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--config 0|1]

Workload: the config-0 family batch (64 held-out seeded states on the config-0 grid, learned start + the batch
driver; `value` counts converged solves) with the plain single-state config-0 solve beside it, built before the timed
region and made device-resident; a plain step is one complete solve (first light, evaluations until every wavelength
meets the tolerance, Anderson mixing). `e2e` = the same through the public API with host buffers: handles created
once with the shared geometry, every step uploading each state's constants from host arrays, solving and reading the
fields back. The dominant kernel is timed with CUDA events recorded by the library on its own work stream;
`roofline.achieved` is its algorithmic bytes per launch over its mean launch time.
`forms` adds the plain and learned batched solves, the training report, the projection precision forms on a
30-wavelength state, `make_table` on the reference's full table axes and the per-state ground preparation on the host
and on the device.
`cpu_baseline` and the `--impl reference` arm time the CPU port of the reference algorithm (oracle/) on the host
cores, one process per core, on a bounded sample of the same workload (first light plus one evaluation per process,
extrapolated by the GPU run's evaluation count).

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
L2_BYTES = 129 << 20


# ------------------------------------------------------------------------------------------------ helpers
def args_():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=5)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='gb300', choices=('gb300', 'reference'))
    p.add_argument('--config', type=int, default=0, choices=(0, 1))
    p.add_argument('--seed', type=int, default=0)
    p.add_argument('--no-cpu-baseline', action='store_true')
    p.add_argument('--no-forms', action='store_true', help='plain single-state solve only')
    p.add_argument('--precision-only', action='store_true',
                   help='only the precision form (projection forms on a 30-wavelength state), one JSON line')
    p.add_argument('--ground-only', action='store_true',
                   help='only the ground-preparation form (host against device, a config-0 family state)')
    p.add_argument('--batch', type=int, default=64, help='states per batched step')
    p.add_argument('--train-solves', type=int, default=512)
    p.add_argument('--epochs', type=int, default=30)
    return p.parse_args()


def workload(config, seed):
    from sosfuse2_gb300 import synth

    if config == 0:
        return synth.config0(seed=seed), ('config0: plain SOS, 550 nm, 101 heights 0-100 km x 10 solar-zenith nodes, '
                                          'nmu 1, nphi 2, path_n 4, L=16, stratospheric layer, tolerance 1e-3')
    return synth.config1(seed=seed), ('config1: plain SOS, 30 wavelengths 400-700 nm, 241 heights 0-120 km x 75 '
                                      'solar-zenith nodes, nmu 12, nphi 16, path_n 12, L=32, tolerance 1e-3')


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


def profiled_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary (profiles/*.txt, 'traffic_bytes_per_launch')."""
    for f in sorted((ROOT / 'profiles').glob('*.txt')):
        for line in f.read_text().splitlines():
            if line.startswith(f'traffic_bytes_per_launch {kernel} '):
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


# ------------------------------------------------------------------------------------------------ CPU baseline
def _oracle_sample(job):
    """One process: first light and one warm pass of the oracle on a strided 1/parts share of the cells, plus the full
    observer boxes; returns (first-light seconds, warm-pass seconds) scaled to all cells, and the boxes seconds."""
    path, part, parts = job
    os.environ.setdefault('OMP_NUM_THREADS', '1')
    from oracle import sos_oracle as so

    pk = so.StatePack(path)
    cells = list(range(part, pk.ns, parts))
    b = pk.subset(cells)
    frac = len(b['d']) / len(pk['cell_d'])
    x = np.zeros(pk.shape, np.float32)
    t0 = time.perf_counter()
    rad = so.transport(pk, b, x, first=True)
    so.project(pk, b, rad)
    t1 = time.perf_counter()
    boundary = np.ones((pk.nc, pk.W))
    rad = so.transport(pk, b, x, first=False, boundary=boundary)
    so.project(pk, b, rad)
    t2 = time.perf_counter()
    so.boxes(pk, x)
    t3 = time.perf_counter()
    return (t1 - t0) / frac, (t2 - t1) / frac, t3 - t2


def cpu_baseline(arrays, evaluations, procs=None):
    """Solves/s of the CPU port over `procs` host cores, one independent solve per core: each core's solve time is
    first light + E x (ground pass + warm pass + 2 observer passes), measured on a bounded sample (strided cell
    shares, one per process) and extrapolated linearly by ray count."""
    import multiprocessing as mp

    procs = procs or min(os.cpu_count() or 1, 16)
    with tempfile.NamedTemporaryFile(suffix='.npz', delete=False) as f:
        np.savez(f, **arrays)
        path = f.name
    from sosfuse2_gb300.state import PackedState

    st = PackedState(arrays)
    ground_frac = float(st['cell_cell_off'][st.nc]) / float(st['cell_cell_off'][-1])
    ctx = mp.get_context('spawn')
    env = dict(OMP_NUM_THREADS='1', OPENBLAS_NUM_THREADS='1', MKL_NUM_THREADS='1')
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        t = time.perf_counter()
        with ctx.Pool(procs) as pool:
            res = pool.map(_oracle_sample, [(path, i, procs) for i in range(procs)])
        wall = time.perf_counter() - t
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        os.unlink(path)
    first = statistics.mean(r[0] for r in res)
    warm = statistics.mean(r[1] for r in res)
    boxes = statistics.mean(r[2] for r in res)
    per_eval = warm * (1 + ground_frac) + 2 * boxes
    solve_s = first + evaluations * per_eval
    return dict(value=procs / solve_s, unit='solves/s', cores=procs, kind='port',
                sample=f'{procs} processes, each: first light and one warm pass on a strided 1/{procs} share of the '
                       f'cells plus the observer boxes ({wall:.1f} s wall); per core {first:.1f} s first light + '
                       f'{per_eval:.2f} s per evaluation, extrapolated by ray count to {evaluations} evaluations per '
                       f'solve'), wall


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


# ------------------------------------------------------------------------------------------------ arms
def run_reference(a, rank):
    if rank != 0:
        return
    arrays, desc = workload(a.config, a.seed)
    from sosfuse2_gb300.state import PackedState

    # evaluations of one converged solve of this state: 8 for config 0 (the GPU arm's solve of the same seeded state,
    # same algorithm and tolerance); config 1 assumes the same
    evaluations = int(PackedState(arrays).meta.get('evaluations_hint', 8))
    values = []
    for _ in range(a.warmup):
        cpu_baseline(arrays, evaluations)  # process start-up, imports and page cache, not timed
    wall_total = 0.0
    for _ in range(a.steps):
        cb, wall = cpu_baseline(arrays, evaluations)
        values.append(cb['value'])
        wall_total += wall
    v = statistics.mean(values)
    cb['value'] = v
    print(json.dumps(dict(
        impl='reference', metric=METRIC, value=v, unit='solves/s', n_gpus=a.gpus, steps=a.steps, warmup=a.warmup,
        ms_per_step=1e3 / v if v else None, higher_is_better=True, scaling='weak', vs_baseline=None, dtype='f32',
        data='synthetic', config=dict(workload=desc, note='CPU port of the reference algorithm (oracle/), the '
                                                           'reference itself being Python on the same path'),
        cpu_baseline=cb, e2e=dict(value=v, unit='solves/s', h2d_bytes_per_step=0, d2h_bytes_per_step=0))), flush=True)


def _batch_kernels(fam, seeds, device):
    from sosfuse2_gb300.solver import Kernel
    from sosfuse2_gb300.state import PackedState
    from sosfuse2_gb300.synth import family_state

    states = [PackedState(family_state(fam, sd)) for sd in seeds]
    kernels = [Kernel(st, device) for st in states]
    for k in kernels:
        k._check(k.lib.sosb_set_stream(k.h, None))
    return states, kernels


def _time_batched(a, fam, ws, device, seeds, dist=None):
    """Plain and learned-start batched solves of the held-out family states, and the plain solves one state at a
    time (`sequential`: the batch driver with one solve in flight): converged solves/s of each form (each step
    bracketed by a barrier over the ranks and a device synchronisation)."""
    import torch

    from sosfuse2_gb300 import _abi, learned

    states, kernels = _batch_kernels(fam, seeds, device)
    n = len(kernels)
    lib = kernels[0].lib
    handles = (ctypes.c_void_p * n)(*[k.h.value for k in kernels])
    outs = [k.field() for k in kernels]
    out_ptrs = (ctypes.c_void_p * n)(*[o.data_ptr() for o in outs])
    res = {}
    for form in ('plain', 'learned', 'sequential'):
        times, conv, evals, launches = [], [], [], 0
        for step in range(a.warmup + a.steps):
            for k, st in zip(kernels, states):
                k.update(st)  # no first light carried between steps
            bracket(dist)
            t0 = time.perf_counter()
            if form in ('plain', 'sequential'):
                stats = (_abi.Stats * n)()
                status = (ctypes.c_int32 * n)()
                lib.sosb_solve_batch(handles, n, 64, 1e-3, None, out_ptrs, 1, stats, status,
                                     1 if form == 'sequential' else 0)
                ok = [not status[i] for i in range(n)]
                ev = [stats[i].evaluations for i in range(n) if not status[i]]
                nl = sum(stats[i].kernel_launches for i in range(n))
            else:
                g0 = ws.mlp.gemm_launches
                r = learned.solve_batch(ws, kernels, states)
                ok = [not isinstance(x, Exception) for x in r]
                ev = [x[1]['evaluations'] for x in r if not isinstance(x, Exception)]
                # warm solves + the apply(0) of every state (about a tenth of a solve's launches) + network GEMMs
                nl = sum(x[1]['kernel_launches'] for x in r if not isinstance(x, Exception)) + ws.mlp.gemm_launches - g0
            bracket(dist)
            dt = time.perf_counter() - t0
            if step >= a.warmup:
                times.append(dt)
                conv.append(sum(ok))
                evals.extend(ev)
                launches += nl
        res[form] = dict(value=sum(conv) / sum(times), seconds_per_batch=statistics.mean(times), states=n,
                         converged_per_batch=statistics.mean(conv), evaluations_mean=statistics.mean(evals),
                         kernel_launches=launches)
    for k in kernels:
        k.close()
    return res


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


def run_gb300(a, rank, world):
    import torch

    from sosfuse2_gb300 import _abi, build, learned, synth
    from sosfuse2_gb300.solver import Solver
    from sosfuse2_gb300.state import PackedState

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
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group('nccl')
    # ---------------------------------------------------------------- plain single-state solve (kernel roofline)
    arrays, desc = workload(a.config, a.seed + rank)
    state = PackedState(arrays)
    solver = Solver(state, device=device)
    k = solver.kernel
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=k.device)
    tol = float(state.meta['tolerance'])
    max_eval = int(state.meta['max_eval'])
    for _ in range(max(a.warmup, 0)):
        solver.solve(max_eval, tol, device_out=True)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    clocks = Clocks(local)
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
    plain_ms = statistics.mean(step_ms)
    # per-class kernel times of one more solve with CUDA events around every launch (launched one by one: an event
    # pair per kernel, so this solve is not one of the timed steps)
    ncls = len(_abi.KERNEL_CLASSES)
    ms = (_abi.c_dbl * ncls)()
    cnt = (_abi.c_i64 * ncls)()
    flush.fill_(1.0)
    k.lib.sosb_set_timing(k.h, 1)
    solver.solve(max_eval, tol, device_out=True)
    k.lib.sosb_get_timing(k.h, ms, cnt, ncls)
    k.lib.sosb_set_timing(k.h, 0)
    # ---------------------------------------------------------------- batched forms on the config-0 family
    forms = None
    if a.config == 0 and not a.no_forms:
        fam = synth.config0_family()
        t0 = time.perf_counter()
        ws, report = learned.train_warm_start(fam, n_train=a.train_solves, epochs=a.epochs, seed=10000, device=device)
        report['seconds'] = time.perf_counter() - t0
        seeds = list(range(90000, 90000 + a.batch))
        forms = _time_batched(a, fam, ws, device, seeds, dist)
        forms['training'] = report
        forms['learned_vs_plain'] = forms['learned']['value'] / max(forms['plain']['value'], 1e-30)
        forms['learned_batched_vs_plain_sequential'] = (forms['learned']['value']
                                                         / max(forms['sequential']['value'], 1e-30))
        forms['precision'] = _precision_form(device)
        forms['table'] = _table_form(fam, device)
        forms['ground'] = _ground_form(fam, device)
        launches += sum(forms[f]['kernel_launches'] for f in ('plain', 'learned', 'sequential'))
    clk = clocks.stop()
    value_plain = 1e3 / plain_ms
    value = forms['learned']['value'] if forms else value_plain
    value = whole_job(value, world, dist)
    bracket(dist)
    # ---------------------------------------------------------------- end to end through the public API
    # The user's calls for states on one geometry: handles created once with the bundles (outside the timing); every
    # step uploads each state's constants from host arrays (Kernel.update), solves, and reads the fields back to the
    # host. h2d counts the constant arrays uploaded, d2h the fields read back.
    from sosfuse2_gb300.solver import Kernel

    def constant_bytes(arr):
        return sum(v.nbytes for key, v in arr.items()
                   if key != 'meta' and not key.startswith('cell_') and not key.startswith('query_'))

    e2e_ms = []
    if forms:
        from sosfuse2_gb300.synth import family_state

        seeds = list(range(90000, 90000 + a.batch))
        host = [family_state(fam, sd) for sd in seeds]
        h2d = sum(constant_bytes(arr) for arr in host)
        d2h = sum(int(np.prod(PackedState(arr).shape)) * 4 for arr in host)
        kernels = [Kernel(PackedState(host[0]), device) for _ in host]
        for kk in kernels:
            kk._check(kk.lib.sosb_set_stream(kk.h, None))
        for _ in range(max(1, min(a.steps, 2))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sts = [PackedState(arr) for arr in host]
            for kk, st in zip(kernels, sts):
                kk.update(st)
            r = learned.solve_batch(ws, kernels, sts)
            fields = [x[0].cpu().numpy() for x in r if not isinstance(x, Exception)]
            torch.cuda.synchronize()
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
            conv = len(fields)
        for kk in kernels:
            kk.close()
        e2e = dict(value=world * conv / (statistics.mean(e2e_ms) / 1e3), unit='solves/s', h2d_bytes_per_step=int(h2d),
                   d2h_bytes_per_step=int(d2h))
    else:
        h2d = constant_bytes(arrays)
        d2h = int(np.prod(state.shape)) * 4
        s2 = Solver(PackedState(arrays), device=device)
        for _ in range(max(1, min(a.steps, 3))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s2.kernel.update(PackedState(arrays))
            s2.solve(max_eval, tol)  # host output
            torch.cuda.synchronize()
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
        s2.kernel.close()
        e2e = dict(value=world / (statistics.mean(e2e_ms) / 1e3), unit='solves/s', h2d_bytes_per_step=int(h2d),
                   d2h_bytes_per_step=int(d2h))
    if rank != 0:
        return
    classes = _abi.KERNEL_CLASSES
    ncls = len(classes)
    times = {classes[i]: dict(ms=ms[i], launches=int(cnt[i]), share=ms[i] / max(sum(ms), 1e-30))
             for i in range(ncls)}
    top = max(range(ncls), key=lambda i: ms[i])
    E = statistics.mean(evaluations)
    peak, peak_kind = peaks()
    roof = None
    if classes[top] in ('transport', 'transport_table'):
        b = transport_bytes(state)
        if classes[top] == 'transport_table':
            # ground + warm + 2 observer launches per evaluation, all from node tables
            per_launch = (b['ground'] + b['warm'] + 2 * b['observer']) / 4
            name = 'transport_table_kernel' if state.W <= 4 else 'transport_table_wave_kernel'
        else:
            per_launch = b['first']
            name = 'transport_warp_kernel' if state.W <= 4 else 'transport_wave_kernel'
        mean_ms = ms[top] / max(cnt[top], 1)
        achieved = per_launch / (mean_ms / 1e3) / 1e9
        roof = dict(kernel=name, bound='hbm', achieved=achieved, peak=peak, unit='GB/s', frac=achieved / peak,
                    peak_source=peak_kind, traffic=profiled_traffic(name), bytes_per_launch=per_launch,
                    mean_launch_ms=mean_ms,
                    measured_on='CUDA events around each launch of one more plain solve of the workload below')
    cb = None
    if world == 1 and not a.no_cpu_baseline:
        cb, _ = cpu_baseline(arrays, int(round(E)))
    if forms:
        wl = (f'config-0 family batch: {a.batch} held-out seeded states (seeds 90000+) on the config-0 grid (101 '
              f'heights x 10 solar-zenith nodes, nmu 1, nphi 2, path_n 4, L=16, 550 nm, stratospheric layer), amounts '
              f'from the batched configuration ranges (AOD 0.02-0.5, g 0.5-0.8, ozone 250-400 DU, albedo 0.05-0.8); '
              f'learned start + concurrent batched solves; value counts converged solves only')
        step_ms_out = forms['learned']['seconds_per_batch'] * 1e3
    else:
        wl = desc
        step_ms_out = plain_ms
    out = dict(
        metric=METRIC, value=value, unit='solves/s', n_gpus=world, steps=a.steps, warmup=a.warmup,
        ms_per_step=step_ms_out, higher_is_better=True, scaling='weak', vs_baseline=None, dtype='f32',
        data='synthetic (seeded atmosphere on the reference geometry, sosfuse2_gb300.synth)',
        config=dict(workload=wl, plain_single_state=desc, rays=state.meta['rays'], segments=state.meta['segments'],
                    cells=state.ns, evaluations_per_plain_solve=E, plain_single_solves_per_s=value_plain,
                    l2='flushed between timed plain solves (512 MiB write outside the events); batch steps exceed L2',
                    parallelism=f'replicas x{world}'),
        forms=forms, roofline=roof, kernel_times=times, cpu_baseline=cb, e2e=e2e, gpu_launches=int(launches),
        clocks=clk)
    print(json.dumps(out), flush=True)


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
