"""The `b200` backend: a Kernel and a Solver with the reference's interface, over libsosb (C ABI, sm_103a).

`Kernel` stands where the reference's `source_solver.Kernel` stands (src/sosfuse2/solve/source_solver.py:1109-2484):
it owns the device copy of one state's constants and ray bundles and runs `launch` (phases 0, 1, 2 and first light)
and the observer `transport`. `Solver` stands where `source_iteration.Solver` stands
(src/sosfuse2/solve/source_iteration.py:100-663): `initialize`, `apply`, `boxes` and `solve(max_eval, tolerance)`
with the same return values and the same error codes (E_NONFINITE_SOURCE, E_NOT_CONVERGED).

Device buffers are torch CUDA tensors; every call runs on torch's current stream. There is no CPU path: without a
GPU or without the built library the constructor raises.
"""

import ctypes
import time

import numpy as np

from . import _abi
from .state import PackedState


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError('E_CUDA_DEVICE: no CUDA device (the b200 backend has no CPU path)')
    return torch


class Kernel:
    """Device-resident state of one packed state (constants, cell bundle, observer bundle)."""

    backend = 'b200'

    def __init__(self, state, device=None, library=None):
        torch = _torch()
        self.torch = torch
        self.state = state if isinstance(state, PackedState) else PackedState(state)
        self.device = torch.device(device or 'cuda')
        self.lib = _abi.library(library)
        st = self.state
        self.L, self.K, self.W = st.L, st.K, st.W
        self.deterministic = True
        self._dims = st.dims()
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            rc = self.lib.sosb_create(ctypes.byref(self._dims), ctypes.byref(handle))
            if rc:
                raise RuntimeError(f'E_CREATE: sosb_create returned {rc}')
            self.h = handle
            self._check(self.lib.sosb_set_stream(self.h, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
            self._check(self.lib.sosb_set_constants(self.h, ctypes.byref(st.constants())))
            self._check(self.lib.sosb_set_bundle(self.h, _abi.CELLS, ctypes.byref(st.abi_bundle('cell'))))
            self._check(self.lib.sosb_set_bundle(self.h, _abi.OBSERVER, ctypes.byref(st.abi_bundle('query'))))
        st._keep.clear()
        self.n_query = len(st['query_d'])
        self.n_rays = len(st['cell_d'])
        self.ground_rays = None    # the rays of set_ground_rays
        self.ground_optics = None  # (albedo, ext, strato_ext) of the last prepare_ground since the constants

    def update(self, state):
        """Replace the constants by those of another state with the same geometry (bundles stay on the device)."""
        st = state if isinstance(state, PackedState) else PackedState(state)
        if st.shape != self.state.shape or len(st['cell_d']) != self.n_rays:
            raise ValueError('E_SHAPE: update needs a state of the same geometry')
        self._check(self.lib.sosb_set_constants(self.h, ctypes.byref(st.constants())))
        st._keep.clear()
        self.state = st
        self.ground_optics = None  # the state's own ground arrays replaced any prepared on the device

    def set_node_tables(self, enable):
        """Store per-node geometry and attenuation at the first launch over a bundle and read them in warm launches
        (default on); off: every launch recomputes them."""
        self._check(self.lib.sosb_set_node_tables(self.h, int(bool(enable))))

    def set_projection(self, mode):
        """Projection form: 0 FP32 CUDA cores, 1 bf16x3, 2 TF32, 3 BF16 tensor cores."""
        self._check(self.lib.sosb_set_projection(self.h, int(mode)))

    def set_graphs(self, enable):
        """Replay each solve's evaluations from a captured CUDA graph (default on)."""
        self._check(self.lib.sosb_set_graphs(self.h, int(bool(enable))))

    def _check(self, rc):
        if rc:
            msg = self.lib.sosb_last_error(self.h).decode()
            if msg.startswith('E_NONFINITE_SOURCE') or msg.startswith('E_NOT_CONVERGED'):
                raise RuntimeError(msg)
            raise RuntimeError(msg or f'E_NATIVE: status {rc}')

    def close(self):
        if getattr(self, 'h', None):
            self.lib.sosb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ reference Kernel surface
    def set_ground_rays(self, rays):
        """Upload the ground-illumination rays of every cell (synth.Family.ground_rays(); the geometry of
        engine_core.Solver.prepare_ground) for sosb_prepare_ground."""
        keep = dict(cell=np.ascontiguousarray(rays['cell'], np.int32),
                    loc=np.ascontiguousarray(rays['loc'], np.float64),
                    weight=np.ascontiguousarray(rays['weight'], np.float64),
                    cols=np.ascontiguousarray(rays['cols'], np.float64),
                    cos_sun=np.ascontiguousarray(rays['cos_sun'], np.float64),
                    ok=np.ascontiguousarray(rays['ok'], np.uint8))
        g = _abi.GroundRays(n=len(keep['cell']))
        for name, ct in _abi.GroundRays._fields_[1:]:
            setattr(g, name, keep[name].ctypes.data_as(ct))
        self._check(self.lib.sosb_set_ground_rays(self.h, ctypes.byref(g)))
        self.ground_rays = keep

    def prepare_ground(self, albedo, ext, strato_ext=None):
        """Solver.prepare_ground on the device for a state's albedo and FP64 extinction ext [5, W] (and the
        stratospheric extinction [W]); replaces the ground arrays of the constants until the next `update`."""
        self._stream()
        e = np.ascontiguousarray(ext, np.float64)
        s = None if strato_ext is None else np.ascontiguousarray(strato_ext, np.float64)
        self._check(self.lib.sosb_prepare_ground(self.h, float(albedo), e.ctypes.data_as(_abi.P_f64),
                                                 None if s is None else s.ctypes.data_as(_abi.P_f64)))
        self.ground_optics = (float(albedo), e, s)

    def set_observer(self, bundle):
        """Replace the observer (phase-2) ray bundle by `bundle` (the packed-state bundle keys, without prefix); the
        cell bundle and the constants stay. Node tables and pairs of the old observer bundle are dropped."""
        arrays = {'query_' + k: v for k, v in bundle.items()}
        arrays['meta'] = dict(self.state.meta)
        st = PackedState(arrays)
        self._check(self.lib.sosb_set_bundle(self.h, _abi.OBSERVER, ctypes.byref(st.abi_bundle('query'))))
        st._keep.clear()
        self.n_query = len(bundle['d'])

    def _stream(self):
        self.lib.sosb_set_stream(self.h, ctypes.c_void_p(self.torch.cuda.current_stream(self.device).cuda_stream))

    def field(self, value=None):
        """A device field [cells, slots, W] (zeros, or a copy of `value`)."""
        if value is None:
            return self.torch.zeros(self.state.shape, dtype=self.torch.float32, device=self.device)
        return self.torch.as_tensor(np.ascontiguousarray(value, np.float32), device=self.device).contiguous()

    def _dev(self, t):
        if t is None:
            return None
        if not (t.is_cuda and t.dtype == self.torch.float32 and t.is_contiguous()):
            raise ValueError('E_LAYOUT: expected a contiguous float32 CUDA tensor')
        return ctypes.c_void_p(t.data_ptr())

    def launch(self, phase, first=False, field=None, boundary=None, radiance=False):
        """Kernel.launch: (moments [cells, 4+K, W], flux [cells, W], radiance [rays, W, 4]) for the phase; phase 0
        also returns the per-ray radiance of the cell rays when `radiance`."""
        torch = self.torch
        st = self.state
        self._stream()
        f32 = dict(dtype=torch.float32, device=self.device)
        moments = flux = rad = None
        if phase == 0:
            moments = torch.empty((st.ns, 4 + self.K, self.W), **f32)
            flux = torch.empty((st.ns, self.W), **f32)
            if radiance:
                rad = torch.empty((self.n_rays, self.W, 4), **f32)
        elif phase == 1:
            flux = torch.empty((st.nc, self.W), **f32)
        else:
            rad = torch.empty((self.n_query, self.W, 4), **f32)
        self._check(self.lib.sosb_evaluate(self.h, phase, int(bool(first)), self._dev(field), self._dev(boundary),
                                           self._dev(moments), self._dev(flux), self._dev(rad)))
        return moments, flux, rad

    def transport(self, field, first=False):
        """Observer-ray radiance [rays, W, 4] (Kernel.transport of the observer rays)."""
        return self.launch(2, first, field)[2]

    def host(self, t):
        return t.detach().cpu().numpy()

    def sync(self):
        self.torch.cuda.synchronize(self.device)

    def memory(self):
        return self.torch.cuda.max_memory_allocated(self.device)


class Solver:
    """source_iteration.Solver over the b200 Kernel."""

    def __init__(self, state, kernel=None, device=None):
        self.kernel = kernel or Kernel(state, device)
        self.state = self.kernel.state
        self.first_moments = None
        self.first_flux = None
        self.timings = dict(apply_seconds=[], setup_seconds=0.0)

    def initialize(self):
        if self.first_moments is None:
            t = time.perf_counter()
            self.first_moments, self.first_flux, _ = self.kernel.launch(0, True)
            self.timings['setup_seconds'] = time.perf_counter() - t

    def apply(self, field):
        k = self.kernel
        k._stream()
        out = k.torch.empty_like(field)
        t = time.perf_counter()
        k._check(k.lib.sosb_apply(k.h, k._dev(field), k._dev(out)))
        self.timings['apply_seconds'].append(time.perf_counter() - t)
        return out

    def boxes(self, field):
        k = self.kernel
        k._stream()
        rows = k._dims.n_monitor_rows
        out = np.empty((rows, k._dims.n_dirs, k.W), np.float64)
        k._check(k.lib.sosb_boxes(k.h, k._dev(field), out.ctypes.data_as(_abi.P_f64)))
        return out

    def solve(self, max_eval=16, tolerance=0.005, initial=None, device_out=False):
        """Solver.solve: (field, stats). The field is a host array unless device_out (then a CUDA tensor)."""
        k = self.kernel
        k._stream()
        st = self.state
        stats = _abi.Stats()
        x0 = None if initial is None else np.ascontiguousarray(initial, np.float32)
        if device_out:
            out = k.field()
            out_ptr = ctypes.c_void_p(out.data_ptr())
        else:
            out = np.empty(st.shape, np.float32)
            out_ptr = out.ctypes.data_as(ctypes.c_void_p)
        t = time.perf_counter()
        rc = k.lib.sosb_solve(k.h, int(max_eval), float(tolerance),
                              None if x0 is None else x0.ctypes.data_as(ctypes.c_void_p), out_ptr, int(device_out),
                              ctypes.byref(stats))
        seconds = time.perf_counter() - t
        self.last_stats = stats
        k._check(rc)
        W = k.W
        obs = [float(stats.observer_relative[w]) for w in range(W)]
        src = [float(stats.source_relative[w]) for w in range(W)]
        return out, dict(
            seconds=seconds,
            evaluations=int(stats.evaluations),
            tolerance=tolerance,
            converged=[bool(stats.done[w]) for w in range(W)],
            observer_relative=obs,
            source_relative=src,
            # the reference's per-evaluation history (source_iteration.py:381-391); its consumers read the last entry
            # (jobs/run_state.py:99-104, jobs/walkthrough.py:296)
            history=self.history(),
            kernel_launches=int(stats.kernel_launches),
        )

    def history(self):
        """Per-evaluation history of the last solve on this kernel: [{evaluation, observer_relative, source_relative}]."""
        k = self.kernel
        count = ctypes.c_int32()
        k._check(k.lib.sosb_history(k.h, 0, ctypes.byref(count), None, None))
        n, W = int(count.value), k.W
        obs = np.zeros((max(n, 1), W))
        src = np.zeros((max(n, 1), W))
        k._check(k.lib.sosb_history(k.h, n, ctypes.byref(count), obs.ctypes.data_as(_abi.P_f64),
                                    src.ctypes.data_as(_abi.P_f64)))
        return [dict(evaluation=e + 1, observer_relative=obs[e].tolist(), source_relative=src[e].tolist())
                for e in range(n)]


class BatchSolver:
    """Many independent states solved together (sosb_solve_batch): each state has its own handle and stream; one
    library thread enqueues every state's first evaluation and solve graph (the loop runs on the device), so the GPU
    overlaps their launches, and waits only for the streams to finish (`threads`: solves in flight, 0 all)."""

    def __init__(self, states, device=None):
        self.kernels = [Kernel(st, device) for st in states]
        for k in self.kernels:
            k._check(k.lib.sosb_set_stream(k.h, None))  # each handle on its own stream
        self.lib = self.kernels[0].lib if self.kernels else _abi.library()

    def close(self):
        for k in self.kernels:
            k.close()

    def solve(self, max_eval=64, tolerance=1e-3, initial=None, threads=0):
        """[(field, stats) or RuntimeError per state]; fields are host arrays."""
        n = len(self.kernels)
        outs = [np.empty(k.state.shape, np.float32) for k in self.kernels]
        x0 = None if initial is None else [np.ascontiguousarray(a, np.float32) for a in initial]
        handles = (ctypes.c_void_p * n)(*[k.h.value for k in self.kernels])
        out_ptrs = (ctypes.c_void_p * n)(*[o.ctypes.data for o in outs])
        x0_ptrs = None if x0 is None else (ctypes.c_void_p * n)(*[a.ctypes.data for a in x0])
        stats = (_abi.Stats * n)()
        status = (ctypes.c_int32 * n)()
        t = time.perf_counter()
        self.lib.sosb_solve_batch(handles, n, int(max_eval), float(tolerance), x0_ptrs, out_ptrs, 0, stats, status,
                                  int(threads))
        seconds = time.perf_counter() - t
        results = []
        for i, k in enumerate(self.kernels):
            if status[i]:
                results.append(RuntimeError(k.lib.sosb_last_error(k.h).decode()))
                continue
            st = stats[i]
            results.append((outs[i], dict(evaluations=int(st.evaluations), converged=[bool(st.done[w]) for w in range(k.W)],
                                          seconds=float(st.seconds), kernel_launches=int(st.kernel_launches))))
        self.seconds = seconds
        return results
