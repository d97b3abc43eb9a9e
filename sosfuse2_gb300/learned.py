"""Learned warm start: an MLP predicts the converged source from per-cell optics and the single-scattering source;
the solver starts from its prediction and the unchanged convergence test judges the result.

The network (4 hidden layers of width 512, GELU, BF16 weights and activations, FP32 accumulation and master weights)
runs forward and backward on the project's own tcgen05 GEMM (`sosb_gemm_bf16`, fused bias + GELU epilogue) and
elementwise kernels (GELU backward, transposes, bias sums, Adam, MSE) in libsosb; torch provides only device memory,
gathers and the random batch order.

Rows are (cell, wavelength) pairs. Input: the cell's height and solar zenith, the log extinctions of air, aerosol,
ozone and stratospheric aerosol at the cell and the optical depth above it, single-scattering albedo, albedo, the
mixture's first 8 phase moments, the column optical depths of the four components, the cell's single-scattering source
g1 = apply(0) divided by its norm, and that norm.
Target: (x* - g1) / |g1| over all source slots, x* the converged source, for cells with single scattering; cells in
the Earth's shadow (|g1| below 1e-8 of the largest) keep g1. The start is g1 + |g1| * prediction; if the
first evaluation from it changes the source more than the single-scattering start typically does, the solve restarts
from g1 (sosb_solve_warm's fallback).
"""

import ctypes
import math
import time

import numpy as np

from . import _abi


def _ceil(n, k):
    return (n + k - 1) // k * k


class MLP:
    """Fully connected network on libsosb's BF16 tensor-core GEMM."""

    def __init__(self, n_in, n_out, width=512, depth=4, device='cuda', seed=0):
        import torch

        self.torch = torch
        self.lib = _abi.library()
        self.device = torch.device(device)
        self.n_in, self.n_out = n_in, n_out
        self.n_in_p, self.n_out_p = _ceil(n_in, 128), _ceil(n_out, 128)
        dims = [self.n_in_p] + [width] * depth + [self.n_out_p]
        g = torch.Generator(device='cpu').manual_seed(seed)
        f32 = dict(dtype=torch.float32, device=self.device)
        self.W, self.b, self.Wb, self.Wt, self.mW, self.vW, self.mb, self.vb = ([] for _ in range(8))
        for i in range(len(dims) - 1):
            fan_in, fan_out = dims[i], dims[i + 1]
            w = (torch.randn(fan_out, fan_in, generator=g) * math.sqrt(2.0 / fan_in)).to(**f32)
            if i == len(dims) - 2:
                w *= 0.1
            self.W.append(w)
            self.b.append(torch.zeros(fan_out, **f32))
            self.Wb.append(w.to(torch.bfloat16))
            self.Wt.append(w.T.contiguous().to(torch.bfloat16))
            self.mW.append(torch.zeros_like(w))
            self.vW.append(torch.zeros_like(w))
            self.mb.append(torch.zeros(fan_out, **f32))
            self.vb.append(torch.zeros(fan_out, **f32))
        self.dims = dims
        self.step_count = 0
        self.gemm_launches = 0

    # ------------------------------------------------------------------ kernels
    def _s(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream(self.device).cuda_stream)

    @staticmethod
    def _p(t):
        return None if t is None else ctypes.c_void_p(t.data_ptr())

    def _gemm(self, A, B, bias, epilogue, C, H=None):
        M, K = A.shape
        N = B.shape[0]
        rc = self.lib.sosb_gemm_bf16(self._p(A), self._p(B), M, N, K, self._p(bias), epilogue, self._p(C), self._p(H),
                                     self._s())
        if rc:
            raise RuntimeError(self.lib.sosb_tc_last_error().decode())
        self.gemm_launches += 1

    def check(self):
        if self.lib.sosb_tc_check(self._s()):
            raise RuntimeError(self.lib.sosb_tc_last_error().decode())

    def _transpose(self, x, rows, cols):
        out = self.torch.empty((cols, rows), dtype=self.torch.bfloat16, device=self.device)
        self.lib.sosb_mlp_transpose(self._p(x), int(x.dtype == self.torch.float32), rows, cols, self._p(out),
                                    self._s())
        return out

    # ------------------------------------------------------------------ network
    def forward(self, X, keep=False):
        """X: BF16 [R, n_in_p] (R a multiple of 128) -> FP32 [R, n_out_p]."""
        torch = self.torch
        R = X.shape[0]
        H, Z = [X], []
        for i in range(len(self.W)):
            out = self.dims[i + 1]
            C = torch.empty((R, out), dtype=torch.float32, device=self.device)
            if i < len(self.W) - 1:
                Hn = torch.empty((R, out), dtype=torch.bfloat16, device=self.device)
                self._gemm(H[-1], self.Wb[i], self.b[i], 1, C, Hn)
                H.append(Hn)
                Z.append(C)
            else:
                self._gemm(H[-1], self.Wb[i], self.b[i], 2, C)
                Z.append(C)
        if keep:
            self._H, self._Z = H, Z
        return Z[-1]

    def backward(self, dOut):
        """Gradients of the kept forward pass: lists dW [out, in] and db [out] (FP32)."""
        torch = self.torch
        H, Z = self._H, self._Z
        R = dOut.shape[0]
        dW, db = [None] * len(self.W), [None] * len(self.W)
        dz_f = dOut
        dz_b = torch.empty_like(dOut, dtype=torch.bfloat16)
        self.lib.sosb_mlp_to_bf16(self._p(dOut), dOut.numel(), self._p(dz_b), self._s())
        for i in range(len(self.W) - 1, -1, -1):
            out, inn = self.dims[i + 1], self.dims[i]
            gW = torch.empty((out, inn), dtype=torch.float32, device=self.device)
            self._gemm(self._transpose(dz_b, R, out), self._transpose(H[i], R, inn), None, 0, gW)
            gb = torch.empty(out, dtype=torch.float32, device=self.device)
            self.lib.sosb_mlp_column_sum(self._p(dz_f), R, out, self._p(gb), self._s())
            dW[i], db[i] = gW, gb
            if i > 0:
                dH = torch.empty((R, inn), dtype=torch.float32, device=self.device)
                self._gemm(dz_b, self.Wt[i], None, 0, dH)
                dz_f = torch.empty_like(dH)
                dz_b = torch.empty((R, inn), dtype=torch.bfloat16, device=self.device)
                self.lib.sosb_mlp_gelu_backward(self._p(dH), self._p(Z[i - 1]), dH.numel(), self._p(dz_b),
                                                self._p(dz_f), self._s())
        return dW, db

    def adam(self, dW, db, lr, decay=0.0):
        self.step_count += 1
        for i in range(len(self.W)):
            self.lib.sosb_mlp_adam(self._p(self.W[i]), self._p(dW[i]), self._p(self.mW[i]), self._p(self.vW[i]),
                                   self.W[i].numel(), lr, 0.9, 0.999, 1e-8, self.step_count, decay,
                                   self._p(self.Wb[i]), self._s())
            self.lib.sosb_mlp_adam(self._p(self.b[i]), self._p(db[i]), self._p(self.mb[i]), self._p(self.vb[i]),
                                   self.b[i].numel(), lr, 0.9, 0.999, 1e-8, self.step_count, 0.0, None, self._s())
            out, inn = self.W[i].shape
            self.lib.sosb_mlp_transpose(self._p(self.W[i]), 1, out, inn, self._p(self.Wt[i]), self._s())

    def mse_grad(self, pred, target):
        """dLoss/dpred of the mean squared error and the loss (one float read back)."""
        torch = self.torch
        n = pred.numel()
        d = torch.empty_like(pred)
        blocks = 256
        partial = torch.empty(blocks, dtype=torch.float32, device=self.device)
        self.lib.sosb_mlp_mse(self._p(pred), self._p(target), n, 1.0 / n, self._p(d), self._p(partial), blocks,
                              self._s())
        return d, partial

    def train(self, X, Y, epochs=20, batch=4096, lr=1e-3, seed=0, log=None):
        """X BF16 [N, n_in_p], Y FP32 [N, n_out_p]; mini-batch Adam with a cosine learning-rate schedule."""
        torch = self.torch
        N = X.shape[0]
        steps = max(1, N // batch)
        total = epochs * steps
        g = torch.Generator(device=self.device).manual_seed(seed)
        losses = []
        k = 0
        for ep in range(epochs):
            perm = torch.randperm(N, generator=g, device=self.device)
            acc = torch.zeros((), device=self.device)
            for s in range(steps):
                idx = perm[s * batch:(s + 1) * batch]
                pred = self.forward(X.index_select(0, idx), keep=True)
                d, partial = self.mse_grad(pred, Y.index_select(0, idx))
                dW, db = self.backward(d)
                rate = lr * 0.5 * (1 + math.cos(math.pi * k / total))
                self.adam(dW, db, rate)
                acc += partial.sum()
                k += 1
            losses.append(float(acc) / (steps * batch * self.n_out_p))
            if log:
                log(ep, losses[-1])
        self.check()
        return losses

    def predict(self, X, rows=8192):
        torch = self.torch
        out = []
        for r0 in range(0, X.shape[0], rows):
            out.append(self.forward(X[r0:r0 + rows]))
        return torch.cat(out)

    def state_dict(self):
        return dict(W=[w.cpu().numpy() for w in self.W], b=[b.cpu().numpy() for b in self.b], dims=self.dims)


# ---------------------------------------------------------------------------------------------------- features
def cell_features(state):
    """Optics features of every (cell, wavelength) row of a packed state [ns * W, 24] (FP64 on the host)."""
    a, m = state.arrays, state.meta
    h, chi = a['h'].astype(float), a['chi'].astype(float)
    nh, nc, W = len(h), len(chi), state.W
    ext = a['ext'].astype(float)
    prof = np.stack([np.exp(-h / 8), np.exp(-h / float(m['height'])), np.interp(h, np.arange(len(a['density_table']))
                     * float(m['profile_step_km']), a['density_table'][:, 1])], -1)
    beta = np.stack([prof[:, 0, None] * ext[0], prof[:, 1, None] * ext[1], prof[:, 2, None] * ext[2]], 0)  # [3, nh, W]
    sca_air = beta[0]
    sca_aer = prof[:, 1, None] * a['asca'].astype(float)
    if state.strato:
        st = a['strato_density'].astype(float)[:, None] * a['strato_ext'].astype(float)
    else:
        st = np.zeros((nh, W))
    total = beta.sum(0) + st
    dz = np.diff(h)
    mid = 0.5 * (total[1:] + total[:-1]) * dz[:, None]
    above = np.r_[np.cumsum(mid[::-1], axis=0)[::-1], np.zeros((1, W))]
    g = float(m['g'])
    gs = float(a['strato_chi'][1, 0] / 3.0) if state.strato else 0.0
    sca = sca_air + sca_aer + st
    moments = np.stack([(sca_aer * g ** l + st * gs ** l + (sca_air * 0.1 if l == 2 else 0.0)) / np.maximum(sca, 1e-30)
                        for l in range(1, 9)], -1)  # [nh, W, 8]
    ssa = sca / np.maximum(total, 1e-30)
    # rows ordered (height, chi, wavelength)
    shp = (nh, nc, W)
    col = lambda v: np.broadcast_to(v, shp).reshape(-1)  # noqa: E731
    feats = [col((h / h[-1])[:, None, None]), col(np.cos(chi)[None, :, None]), col(np.sin(chi)[None, :, None])]
    for v in (beta[0], beta[1], beta[2], st, above, total):
        feats.append(col(np.log10(np.maximum(v, 1e-12))[:, None, :]))
    feats += [col(ssa[:, None, :]), np.full(nh * nc * W, float(m['albedo'])), np.full(nh * nc * W, g)]
    feats += [col(moments[:, None, :, l]) for l in range(8)]
    # whole-atmosphere quantities (multiple scattering at a cell depends on the whole column, not only the cell):
    # total optical depths of air, aerosol, ozone and stratospheric aerosol
    tau_air, tau_aer, tau_o3 = (np.trapezoid(beta[k], h, axis=0) for k in range(3))
    tau_st = np.trapezoid(st, h, axis=0)
    for v in (tau_air, tau_aer, tau_o3, tau_st):
        feats.append(col(np.log10(np.maximum(v, 1e-12))[None, None, :]))
    return np.stack(feats, -1)


class WarmStart:
    """Feature scaling, the network, and the warm-started solve of one state family."""

    def __init__(self, n_slots, W=1, width=512, depth=4, device='cuda', seed=0):
        self.n_slots = n_slots
        self.n_opt = 24
        self.n_in = self.n_opt + n_slots + 1
        self.mlp = MLP(self.n_in, n_slots, width, depth, device, seed)
        self.torch = self.mlp.torch
        self.device = self.mlp.device
        self.x_mean = self.x_std = self.y_mean = self.y_std = None
        self.fallback_ss = 1.0

    def rows(self, state, g1):
        """Inputs [rows, n_in] (FP32 device) and the per-row norm of g1 from a state and its g1 [ns, slots, W]."""
        torch = self.torch
        opt = torch.as_tensor(cell_features(state), dtype=torch.float32, device=self.device)
        g = g1.permute(0, 2, 1).reshape(-1, self.n_slots)  # (cell, w) rows
        norm = g.norm(dim=1, keepdim=True).clamp_min(1e-30)
        x = torch.cat([opt, g / norm, torch.log10(norm)], 1)
        return x, norm

    @staticmethod
    def lit(norm):
        """Rows with single scattering (|g1| above 1e-8 of the state's largest); cells in the Earth's shadow have
        none, so a relative correction is undefined there and their start stays g1."""
        return (norm > norm.max() * 1e-8).squeeze(1)

    @staticmethod
    def targets(g1, x_star, norm, n_slots):
        g = g1.permute(0, 2, 1).reshape(-1, n_slots)
        xs = x_star.permute(0, 2, 1).reshape(-1, n_slots)
        return (xs - g) / norm

    def fit_scaling(self, X, Y):
        self.x_mean, self.x_std = X.mean(0), X.std(0).clamp_min(1e-6)
        self.y_mean, self.y_std = Y.mean(0), Y.std(0).clamp_min(1e-6)

    def _pad_in(self, X):
        torch = self.torch
        Xs = (X - self.x_mean) / self.x_std
        R = X.shape[0]
        out = torch.zeros((_ceil(R, 128), self.mlp.n_in_p), dtype=torch.bfloat16, device=self.device)
        out[:R, :self.n_in] = Xs.to(torch.bfloat16)
        return out

    def train(self, X, Y, epochs=20, batch=4096, lr=1e-3, log=None):
        torch = self.torch
        self.fit_scaling(X, Y)
        Xp = self._pad_in(X)
        Yp = torch.zeros((Xp.shape[0], self.mlp.n_out_p), dtype=torch.float32, device=self.device)
        Yp[:Y.shape[0], :self.n_slots] = (Y - self.y_mean) / self.y_std
        n = (Y.shape[0] // batch) * batch or Y.shape[0]
        return self.mlp.train(Xp[:n], Yp[:n], epochs=epochs, batch=min(batch, n), lr=lr, log=log)

    def predict_start(self, state, g1):
        """The warm start [ns, slots, W] (device) of a state whose single-scattering source is g1."""
        X, norm = self.rows(state, g1)
        pred = self.mlp.predict(self._pad_in(X))[:X.shape[0], :self.n_slots] * self.y_std + self.y_mean
        pred = pred * self.lit(norm)[:, None]
        ns, slots, W = g1.shape
        x0 = g1.permute(0, 2, 1).reshape(-1, slots) + norm * pred
        return x0.reshape(ns, W, slots).permute(0, 2, 1).contiguous()


def solve_warm(solver, start, fallback, fallback_ss, max_eval=64, tolerance=1e-3):
    """sosb_solve_warm on a Solver whose handle holds first light (after solver.apply): (field device, stats)."""
    k = solver.kernel
    k._stream()
    out = k.field()
    stats = _abi.Stats()
    t = time.perf_counter()
    rc = k.lib.sosb_solve_warm(k.h, int(max_eval), float(tolerance), k._dev(start), float(fallback_ss),
                               k._dev(fallback), ctypes.c_void_p(out.data_ptr()), 1, ctypes.byref(stats))
    seconds = time.perf_counter() - t
    k._check(rc)
    return out, dict(seconds=seconds, evaluations=int(stats.evaluations), fallback=bool(stats.start_fallback),
                     converged=[bool(stats.done[w]) for w in range(k.W)], kernel_launches=int(stats.kernel_launches))


# ---------------------------------------------------------------------------------------------------- drivers
def generate(family, seeds, device='cuda:0', max_eval=64, tolerance=1e-3, log=None, slow=24):
    """Training data from plain solves of family states: inputs X, targets Y (FP32 device), and per state the plain
    evaluation count and the single-scattering start's first source relative change. States the plain solve does
    not converge on, or needs more than `slow` evaluations for, are skipped (generate.skipped)."""
    import torch

    from .solver import Kernel, Solver
    from .state import PackedState
    from .synth import family_state

    kernel = None
    ws_rows, ws_targets, evals, ss_single, skipped = [], [], [], [], []
    helper = None
    for i, seed in enumerate(seeds):
        st = PackedState(family_state(family, seed))
        if kernel is None:
            kernel = Kernel(st, device)
            helper = WarmStart(st.source_size, st.W, device=device)
        else:
            kernel.update(st)
        solver = Solver(st, kernel=kernel)
        g1 = solver.apply(kernel.field())
        try:
            x, stats = solver.solve(max_eval, tolerance, device_out=True)
        except RuntimeError as exc:  # states the plain iteration does not converge on teach nothing: skip them
            if not str(exc).startswith('E_NOT_CONVERGED'):
                raise
            skipped.append(seed)
            continue
        if stats['evaluations'] > slow:
            # a slowly contracting iteration stops (at the tolerance) further from its fixed point: noisy targets
            skipped.append(seed)
            continue
        g2 = solver.apply(g1)
        ss_single.append(float(((g2 - g1).abs().amax() / g2.abs().amax().clamp_min(1e-30)).item()))
        X, norm = helper.rows(st, g1)
        lit = WarmStart.lit(norm)
        ws_rows.append(X[lit])
        ws_targets.append(WarmStart.targets(g1, x, norm, st.source_size)[lit])
        evals.append(stats['evaluations'])
        if log and i % 64 == 0:
            log(i, stats['evaluations'])
    kernel.close()
    generate.skipped = skipped
    return torch.cat(ws_rows), torch.cat(ws_targets), np.asarray(evals), np.asarray(ss_single)


def train_warm_start(family, n_train=512, epochs=30, seed=10000, device='cuda:0', log=None, tolerance=1e-3, slow=24):
    """Generate n_train solves (seeds seed, seed+1, ...) and train the network; returns (WarmStart, report)."""
    from .state import PackedState
    from .synth import family_state

    t0 = time.perf_counter()
    X, Y, evals, ss1 = generate(family, range(seed, seed + n_train), device, tolerance=tolerance, slow=slow)
    t1 = time.perf_counter()
    st = PackedState(family_state(family, seed))
    ws = WarmStart(st.source_size, st.W, device=device)
    losses = ws.train(X, Y, epochs=epochs, lr=1e-3, log=log)
    t2 = time.perf_counter()
    ws.fallback_ss = float(np.quantile(ss1, 0.9))
    return ws, dict(train_solves=n_train, skipped_not_converged_or_slow=len(generate.skipped), rows=int(X.shape[0]),
                    generate_seconds=t1 - t0, train_seconds=t2 - t1,
                    plain_evaluations_mean=float(evals.mean()), loss_first=losses[0], loss_last=losses[-1],
                    fallback_ss=ws.fallback_ss, gemm_launches=ws.mlp.gemm_launches)


def evaluate(ws, family, seeds, device='cuda:0', max_eval=64, tolerance=1e-3):
    """Held-out comparison per state: plain solve vs learned start (apply(0), prediction, warm solve)."""
    import torch

    from .solver import Kernel, Solver
    from .state import PackedState
    from .synth import family_state

    kernel = None
    out = []
    for seed in seeds:
        st = PackedState(family_state(family, seed))
        if kernel is None:
            kernel = Kernel(st, device)
        else:
            kernel.update(st)
        solver = Solver(st, kernel=kernel)
        torch.cuda.synchronize()
        t = time.perf_counter()
        try:
            xp, sp = solver.solve(max_eval, tolerance, device_out=True)
        except RuntimeError as exc:
            if not str(exc).startswith('E_NOT_CONVERGED'):
                raise
            out.append(dict(seed=seed, plain_evaluations=None, error=str(exc)))
            continue
        torch.cuda.synchronize()
        tp = time.perf_counter() - t
        kernel.update(st)  # drop the plain solve's first light: the learned path computes its own
        torch.cuda.synchronize()
        t = time.perf_counter()
        g1 = solver.apply(kernel.field())
        x0 = ws.predict_start(st, g1)
        try:
            xl, sl = solve_warm(solver, x0, g1, ws.fallback_ss, max_eval, tolerance)
        except RuntimeError as exc:
            if not str(exc).startswith('E_NOT_CONVERGED'):
                raise
            out.append(dict(seed=seed, plain_evaluations=sp['evaluations'], learned_evaluations=None, error=str(exc)))
            continue
        torch.cuda.synchronize()
        tl = time.perf_counter() - t
        bp, bl = solver.boxes(xp), solver.boxes(xl)
        big = np.abs(bp) > 1e-6 * np.abs(bp).max()
        out.append(dict(seed=seed, plain_evaluations=sp['evaluations'], learned_evaluations=sl['evaluations'] + 1,
                        fallback=sl['fallback'], plain_seconds=tp, learned_seconds=tl,
                        observer_max_rel_diff=float(np.max(np.abs(bl[big] - bp[big]) / np.abs(bp[big]))),
                        source_rel_l2=float(((xl - xp).norm() / xp.norm()).item())))
    kernel.close()
    return out


def train_config3(orders=(16, 24, 32, 48), n_train=64, epochs=30, seed=10000, device='cuda:0', log=None,
                  tolerance=1e-4):
    """One network per SH order of the batched configuration (the network's input and output are the source slots,
    10 + 2K of them), each trained on n_train solves of synth.config3_training_family(L) (seeds seed, seed + 1, ...)
    to `tolerance` (solves over 40 evaluations are skipped); returns ({L: WarmStart}, {L: report})."""
    from .synth import config3_table, config3_training_family

    table = config3_table()
    nets, reports = {}, {}
    for L in orders:
        fam = config3_training_family(L, table)
        nets[L], reports[L] = train_warm_start(fam, n_train=n_train, epochs=epochs, seed=seed, device=device, log=log,
                                               tolerance=tolerance, slow=40)
    return nets, reports


def solve_batch(ws, kernels, states, max_eval=64, tolerance=1e-3, threads=0, history=True):
    """Learned-start batched solves: apply(0) on every handle concurrently, one network pass over the rows of the
    states of each SH order, then the warm-started solves concurrently (history: the pair (0, g1) of the apply(0)
    first enters each solve's Anderson history, sosb_set_warm_history). `ws`: one WarmStart, or {L: WarmStart}.
    Returns [(field, stats) or RuntimeError] per state."""
    import torch

    n = len(kernels)
    lib = kernels[0].lib
    handles = (ctypes.c_void_p * n)(*[k.h.value for k in kernels])
    zeros = [k.field() for k in kernels]
    g1 = [torch.empty_like(z) for z in zeros]
    status = (ctypes.c_int32 * n)()
    torch.cuda.synchronize()
    lib.sosb_apply_batch(handles, n, (ctypes.c_void_p * n)(*[z.data_ptr() for z in zeros]),
                         (ctypes.c_void_p * n)(*[g.data_ptr() for g in g1]), status, int(threads))
    for i in range(n):
        if status[i]:
            raise RuntimeError(lib.sosb_last_error(kernels[i].h).decode())
    nets = ws if isinstance(ws, dict) else None
    starts = [None] * n
    for L in sorted({st.L for st in states}):
        net = nets[L] if nets is not None else ws
        idx = [i for i, st in enumerate(states) if st.L == L]
        rows, norms, counts = [], [], []
        for i in idx:
            X, norm = net.rows(states[i], g1[i])
            rows.append(X)
            norms.append(norm)
            counts.append(X.shape[0])
        X = torch.cat(rows)
        pred = net.mlp.predict(net._pad_in(X))[:X.shape[0], :net.n_slots] * net.y_std + net.y_mean
        r0 = 0
        for i, norm, c in zip(idx, norms, counts):
            p = pred[r0:r0 + c] * net.lit(norm)[:, None]
            r0 += c
            ns, slots, W = g1[i].shape
            x0 = g1[i].permute(0, 2, 1).reshape(-1, slots) + norm * p
            starts[i] = x0.reshape(ns, W, slots).permute(0, 2, 1).contiguous()
    outs = [torch.empty_like(g) for g in g1]
    stats = (_abi.Stats * n)()
    torch.cuda.synchronize()
    fallback_ss = min(w.fallback_ss for w in nets.values()) if nets is not None else ws.fallback_ss
    for k in kernels:  # (0, g1) enters the Anderson history: the network's start is the second iterate
        k._check(lib.sosb_set_warm_history(k.h, int(history)))
    lib.sosb_solve_warm_batch(handles, n, int(max_eval), float(tolerance),
                              (ctypes.c_void_p * n)(*[x.data_ptr() for x in starts]), float(fallback_ss),
                              (ctypes.c_void_p * n)(*[g.data_ptr() for g in g1]),
                              (ctypes.c_void_p * n)(*[o.data_ptr() for o in outs]), 1, stats, status, int(threads))
    res = []
    for i in range(n):
        if status[i]:
            res.append(RuntimeError(lib.sosb_last_error(kernels[i].h).decode()))
        else:
            res.append((outs[i], dict(evaluations=int(stats[i].evaluations) + 1, fallback=bool(stats[i].start_fallback),
                                      kernel_launches=int(stats[i].kernel_launches))))
    return res
