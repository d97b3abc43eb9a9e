"""The `b200` backend registered with the reference at run time (the reference's files stay unchanged).

`install()` adds the backend name where the reference chooses a backend and routes its hot path to the GB300
library, so that a reference program keeps its calls:

    from sosfuse2_gb300 import b200; b200.install()
    s, scope = create_configured(out, cfg, wl, 'b200', state)        # src/sosfuse2/solve/build.py:14-118
    x, stats = Solver(s, TransientGeometry(s, scope)).solve(64, 1e-3) # src/sosfuse2/solve/source_iteration.py:309
    table, seconds = make_table(s, x, hs, el, az)                     # src/sosfuse2/outputs/radiance_table.py:167

What it changes, each time wrapping the reference's own function:
* `Kernel.__init__` (src/sosfuse2/solve/source_solver.py:1110-1114) accepts backend='b200': the kernel is built as
  the NumPy kernel (its `setup` gives the constants the state is packed from) and then reports backend 'b200';
* `Solver.solve` (source_iteration.py:309-663) of a 'b200' kernel packs the assembled state
  (reference_adapter.pack_state) and runs the whole iteration on the GPU (sosb_solve), returning the field and the
  stats dict (seconds, evaluations, tolerance, converged, history) or raising the reference's E_NOT_CONVERGED /
  E_NONFINITE_SOURCE;
* `radiance_table.make_table` (radiance_table.py:167-219) of a 'b200' state runs both phase-2 transports on the GPU
  over the reference's own view rays (reference_adapter.make_table) with the geometry of the state's last solve.
Any other backend goes through the reference's functions untouched; `uninstall()` restores them. The reference's
`flags_env.resolve_backend` (src/sosfuse2/backends/flags_env.py:149-165) already keeps a typed 'b200'; its command
lines' --backend choices (jobs/run_state.py:1267-1272, jobs/pipeline.py:220) are argparse lists that a maintainer
extends by one word.
"""

_SAVED = {}


def _modules():
    from sosfuse2.outputs import radiance_table
    from sosfuse2.solve import source_iteration, source_solver

    return source_solver, source_iteration, radiance_table


def installed():
    return bool(_SAVED)


def install(device=None, solve_fn=None):
    """Register 'b200' with the imported reference. `solve_fn(arrays, max_eval, tolerance, device)` replaces the GPU
    solve of a packed state (default: the library's, sosfuse2_gb300.reference_adapter.solve_packed)."""
    if _SAVED:
        return
    source_solver, source_iteration, radiance_table = _modules()
    from . import reference_adapter

    kernel_init = source_solver.Kernel.__init__
    solve = source_iteration.Solver.solve
    table = radiance_table.make_table
    run = solve_fn or reference_adapter.solve_packed

    def init(self, *args, backend='numpy', **kw):
        kernel_init(self, *args, backend='numpy' if backend == 'b200' else backend, **kw)
        if backend == 'b200':
            self.backend = 'b200'

    def b200_solve(self, max_eval=16, tolerance=0.005):
        if getattr(self.kernel, 'backend', None) != 'b200':
            return solve(self, max_eval, tolerance)
        scope = self.geometry.scope
        arrays = reference_adapter.pack_state(self.s, self.geometry, scope, tolerance, max_eval)
        self.s._b200_geometry = (self.geometry, scope)
        return run(arrays, max_eval, tolerance, device)

    def b200_table(s, source, hs, el, az, group=32, batch=25, log=print):
        if getattr(s.kernel, 'backend', None) != 'b200':
            return table(s, source, hs, el, az, group, batch, log)
        if not hasattr(s, '_b200_geometry'):
            raise RuntimeError('E_STATE: make_table of a b200 state needs a solve on it first (its geometry)')
        geometry, scope = s._b200_geometry
        return reference_adapter.make_table(s, source, hs, el, az, group, batch, log, geometry=geometry, scope=scope,
                                            device=device)

    _SAVED.update(kernel_init=kernel_init, solve=solve, table=table)
    source_solver.Kernel.__init__ = init
    source_iteration.Solver.solve = b200_solve
    radiance_table.make_table = b200_table


def uninstall():
    if not _SAVED:
        return
    source_solver, source_iteration, radiance_table = _modules()
    source_solver.Kernel.__init__ = _SAVED['kernel_init']
    source_iteration.Solver.solve = _SAVED['solve']
    radiance_table.make_table = _SAVED['table']
    _SAVED.clear()
