"""Fused PM engine: the whole KDK step as four device passes per force evaluation.

This is the fast path behind the reference's force chain + ``kdk_step``
(sim.py:320-327, integrator.py:100-131, bench.py:145-152). Per step it runs the
int64 fixed-point deposit on cell-sorted particles, one conversion pass that
also reduces the boundary moments, the multigrid to a relative residual
``tol`` (default 1e-6, FP64-class through the double-float finest level) with
FP64 multipole faces, and one particle pass that gathers -grad(phi) on the fly
and applies the half-kicks and the drift.

State: the engine owns SoA particle tensors in grid-origin coordinates
(node i at i*dx) and keeps them cell-sorted (re-sorted every ``sort_every``
steps; ``pid`` records the original index). Between steps the velocities are
staggered by half a step; :meth:`synchronize` closes the step.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from galaxy_collision_gb300 import _native

_FLOAT_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "m")
_INT_FIELDS = ("gid", "pid")


@dataclass
class StepResult:
    cycles: int
    converged: bool
    rel_residual: float
    diag: np.ndarray | None = None
    grid_pe_raw: float | None = None


class PMEngine:
    def __init__(self, grid_size: int, dx: float, grav: float = 1.0, *, origin=(0.0, 0.0, 0.0), tol: float = 1e-6,
                 max_cycles: int = 50, pre_sweeps: int = 2, post_sweeps: int = 2, coarse_sweeps: int = 40,
                 fixed_point_bits: int = 52, sort_every: int = 20, grad_grid: bool = True, fixed_cycles: int = 0,
                 max_particles: int = 0, deposit_next: bool = False, plain_f32: bool = False,
                 sort_ahead: float | None = None, phase_launches: bool = False,
                 coarse_level_sweeps: int | None = None):
        self.grid_size = int(grid_size)
        self.dx = float(dx)
        self.grav = float(grav)
        self.origin = np.asarray(origin, dtype=np.float64)
        self.ctx = _native.Context(self.grid_size, self.dx, self.grav)
        self.mg = _native.MGParams()
        self.mg.pre_sweeps = int(pre_sweeps)
        self.mg.post_sweeps = int(post_sweeps)
        self.mg.coarse_sweeps = int(coarse_sweeps)
        self.mg.max_cycles = int(max_cycles)
        self.mg.min_cycles = 1
        self.mg.tol = float(tol)
        if plain_f32:  # the all-FP32 method: stalls at the FP32 floor, runs to max_cycles
            self.mg.flags |= _native.GC_MG_PLAIN_F32
        if phase_launches:  # coarse levels launched phase by phase (ensembles of small runs)
            self.mg.flags |= _native.GC_MG_PHASE_LAUNCHES
        # sweeps each way below the finest level: None (the default) for pre/post_sweeps
        # on every level, as the reference; 1 for fewer latency-bound coarse phases at
        # the price of a weaker cycle (about 0.2 per cycle instead of 0.1)
        if coarse_level_sweeps is not None and int(coarse_level_sweeps) == 1:
            self.mg.flags |= _native.GC_MG_COARSE_ONE_SWEEP
        elif coarse_level_sweeps is not None and not (int(coarse_level_sweeps) == int(pre_sweeps) == int(post_sweeps)):
            raise ValueError("coarse_level_sweeps must be 1, None, or equal to pre_sweeps and post_sweeps")
        # fixed_cycles > 0: exactly that many V-cycles per solve and no host read in
        # the step (the residual stays on the device, see last_residual), which is
        # what lets a step be captured as a CUDA graph
        self.fixed_cycles = int(fixed_cycles)
        if self.fixed_cycles > 0:
            self.mg.flags |= _native.GC_MG_FIXED_CYCLES
            self.mg.max_cycles = self.fixed_cycles
            self.mg.min_cycles = self.fixed_cycles
        self.fixed_point_bits = int(fixed_point_bits)
        self.sort_every = int(sort_every)
        # the periodic sort orders the particles by their cells predicted
        # sort_ahead steps later (x + v * sort_ahead * dt; default half the sort
        # period, so that they drift from their sorted cells by half as much);
        # 0: by the current cells
        self.sort_ahead = self.sort_every / 2.0 if sort_ahead is None else float(sort_ahead)
        self.grad_grid = bool(grad_grid)  # gather from a float4 -grad(phi) grid (same results)
        # the particle pass deposits the drifted positions for the next step (same
        # density, one pass fewer); off by default: at 100M particles on GB300 the
        # fused pass (1.33 ms after a sort, 1.92 ms 20 steps later) is no faster
        # than the gather and deposit passes it replaces (1.37 / 1.86 ms)
        self.deposit_next = bool(deposit_next)
        self.n = 0
        self.state = "empty"   # empty -> synced -> open -> synced ...
        self.steps_since_sort = 0
        self.cur = None
        self.alt = None
        self.last = None
        self._graphs = {}
        if max_particles > 0:  # allocate the particle sets and sort scratch now, not in load
            self.reserve(max_particles)

    def reserve(self, n: int) -> None:
        """Allocate both particle sets for n particles and the context's sort
        scratch, so that load(n particles) allocates nothing."""
        n = int(n)
        if self.cur is None or self.cur["x"].numel() != n:
            self.cur = self._alloc(n)
            self.alt = self._alloc(n)
        self.ctx.call("gc_pm_reserve", n, what="gc_pm_reserve")
        self._side_stream()  # the copy stream of load and export

    # -- state ------------------------------------------------------------------
    @staticmethod
    def _stride(n: int) -> int:
        return (n + 63) // 64 * 64  # every array of a set starts on a 256-byte boundary

    def _alloc(self, n: int):
        """One particle set: the 9 arrays as slices of one device block (so the
        block can also stage interleaved N x 3 arrays for import and export)."""
        dev = torch.device("cuda", torch.cuda.current_device())
        st = self._stride(n)
        blk = torch.empty(9 * st, dtype=torch.float32, device=dev)
        f = {k: blk[i * st:i * st + n] for i, k in enumerate(_FLOAT_FIELDS)}
        f.update({k: blk[(7 + i) * st:(7 + i) * st + n].view(torch.int32) for i, k in enumerate(_INT_FIELDS)})
        f["_block"] = blk
        return f

    def _origin_c(self):
        return (C.c_double * 3)(*[float(v) for v in self.origin])

    def load(self, pos, vel, mass, gid=None, *, sort: bool = True, non_blocking: bool = False) -> None:
        """Load particles in the reference's layout (pos and vel N x 3 in physical
        coordinates, mass N, gid N or None; host or device arrays) into the engine.
        Host arrays are copied into the spare particle set (asynchronously when
        they are pinned) and split on the device by gc_pm_import, or with sort
        by gc_pm_import_order (keys and sort of the positions) and one
        gc_pm_import_gather per array as its copy lands, which gathers them
        straight into cell order."""
        pos_t = torch.as_tensor(pos)
        n = int(pos_t.shape[0])
        if n <= 0:
            raise ValueError("need at least one particle")
        if tuple(pos_t.shape) != (n, 3):
            raise ValueError(f"pos must be N x 3, got {tuple(pos_t.shape)}")
        self.n = n
        if self.cur is None or self.cur["x"].numel() != n:
            self.cur = self._alloc(n)
            self.alt = self._alloc(n)
        dev = self.cur["x"].device
        st = self._stride(n)
        stage = self.alt["_block"]
        origin = self._origin_c()
        if pos_t.dtype == torch.float64:  # subtract the origin in f64 first, as the reference's f64 inputs allow
            pos_t = (pos_t - torch.as_tensor(self.origin, dtype=torch.float64, device=pos_t.device)).to(torch.float32)
            origin = (C.c_double * 3)(0.0, 0.0, 0.0)

        def staged(a, off, shape, dtype):
            t = torch.as_tensor(a)
            if t.device == dev and t.dtype == dtype and t.is_contiguous():
                return t
            dst = stage[off:off + t.numel()].view(dtype).view(shape)
            if t.device.type == "cpu":
                t = t.to(dtype)
                dst.copy_(t, non_blocking=non_blocking or t.is_pinned())
            else:
                dst.copy_(t.to(dtype))
            return dst

        pos_d = staged(pos_t, 0, (n, 3), torch.float32)
        out = self._struct(self.cur)
        main = torch.cuda.current_stream()
        if sort:
            # the positions are keyed and sorted while the other arrays are still
            # being copied (on a side stream); each array is then gathered into
            # cell order as soon as its copy has landed (same result as import + sort)
            side = self._side_stream()
            side.wait_stream(main)
            landed = []
            with torch.cuda.stream(side):
                for a, off, shape, dtype in ((vel, 3 * st, (n, 3), torch.float32), (mass, 6 * st, (n,), torch.float32),
                                             (gid, 7 * st, (n,), torch.int32)):
                    if a is None:
                        landed.append((None, None))
                        continue
                    d = staged(a, off, shape, dtype)
                    ev = torch.cuda.Event()
                    ev.record(side)
                    landed.append((d, ev))
            self.ctx.call("gc_pm_import_order", pos_d.data_ptr(), origin, n, what="gc_pm_import_order")
            self.ctx.call("gc_pm_import_gather", pos_d.data_ptr(), None, None, None, origin, C.byref(out),
                          what="gc_pm_import")
            for slot, (d, ev) in enumerate(landed):
                if d is None:
                    continue
                main.wait_event(ev)
                one = [None, None, None]
                one[slot] = d.data_ptr()
                self.ctx.call("gc_pm_import_gather", None, *one, origin, C.byref(out), what="gc_pm_import")
            main.wait_stream(side)
        else:
            vel_d = staged(vel, 3 * st, (n, 3), torch.float32)
            m_d = staged(mass, 6 * st, (n,), torch.float32)
            gid_d = None if gid is None else staged(gid, 7 * st, (n,), torch.int32)
            self.ctx.call("gc_pm_import", pos_d.data_ptr(), vel_d.data_ptr(), m_d.data_ptr(),
                          None if gid_d is None else gid_d.data_ptr(), origin, C.byref(out), what="gc_pm_import")
        self.state = "synced"
        self.steps_since_sort = 0
        self._graphs = {}

    def export(self, pos=None, vel=None, mass=None, gid=None):
        """The state in the original particle order and the reference's layout:
        pos (N x 3 f32, physical coordinates), vel (N x 3 f32), mass, gid, written
        into the given tensors (host, pinned host or device); only the given ones
        are written, or all four into new host tensors when none is given.
        gc_pm_export_order inverts pid, gc_pm_export_range writes each array in
        the original order into the spare particle set (or straight into device
        outputs); host outputs are filled range by range on a side stream while
        later ranges are written, asynchronously when pinned. Velocities are
        those of the current state (staggered by half a step while the engine is
        open)."""
        n = self.n
        st = self._stride(n)
        stage = self.alt["_block"]
        dev = self.cur["x"].device
        spec = [(pos, 0, (n, 3), torch.float32), (vel, 3 * st, (n, 3), torch.float32),
                (mass, 6 * st, (n,), torch.float32), (gid, 7 * st, (n,), torch.int32)]
        want_all = all(t is None for t, _, _, _ in spec)
        outs, ptrs = [], []
        for t, off, shape, dtype in spec:
            if t is None:
                if not want_all:
                    outs.append((None, None))
                    ptrs.append(None)
                    continue
                t = torch.empty(shape, dtype=dtype)
            if tuple(t.shape) != shape or t.dtype != dtype:
                raise ValueError(f"export output must be {shape} {dtype}, got {tuple(t.shape)} {t.dtype}")
            direct = t.device == dev and t.is_contiguous()
            outs.append((t, None if direct else stage[off:off + t.numel()].view(dtype).view(shape)))
            ptrs.append(t.data_ptr() if direct else outs[-1][1].data_ptr())
        src = self._struct(self.cur)
        origin = self._origin_c()
        main = torch.cuda.current_stream()
        side = self._side_stream()
        # pid inverted once; then each array is written in the original order a
        # range at a time, and every finished range of a host output goes to
        # the host on the side stream while the next one is being written
        self.ctx.call("gc_pm_export_order", C.byref(src), what="gc_pm_export_order")
        for a, (t, stg) in enumerate(outs):
            if t is None:
                continue
            one = [None] * 4
            one[a] = ptrs[a]
            ranges = [(0, n)] if stg is None else self._export_ranges(n)
            for q0, q1 in ranges:
                self.ctx.call("gc_pm_export_range", C.byref(src), origin, *one, q0, q1, what="gc_pm_export_range")
                if stg is not None:
                    side.wait_stream(main)
                    with torch.cuda.stream(side):
                        t[q0:q1].copy_(stg[q0:q1], non_blocking=t.is_pinned())
        main.wait_stream(side)
        return tuple(t for t, _ in outs)

    @staticmethod
    def _export_ranges(n: int, per: int = 1 << 23):
        """Ranges of about `per` particles (8M: ~100 MB of positions, ~0.5 ms on
        the host link) for the overlapped export."""
        k = max(1, -(-n // per))
        b = [n * i // k for i in range(k + 1)]
        return list(zip(b[:-1], b[1:]))

    def _side_stream(self):
        if getattr(self, "_side", None) is None:
            self._side = torch.cuda.Stream()
        return self._side

    def _struct(self, f) -> _native.Particles:
        p = _native.Particles()
        for k in _FLOAT_FIELDS + _INT_FIELDS:
            setattr(p, k, f[k].data_ptr())
        p.n = self.n
        return p

    def sort(self, dt: float | None = None) -> None:
        """Stable cell-key sort of all particle arrays (ping-pong buffers), by
        the cells predicted sort_ahead steps of dt later when both are set."""
        a, b = self._struct(self.cur), self._struct(self.alt)
        tau = self.sort_ahead * float(dt) if dt else 0.0
        self.ctx.call("gc_pm_sort_ahead", C.byref(a), C.byref(b), C.c_float(tau), what="gc_pm_sort_ahead")
        self.cur, self.alt = self.alt, self.cur
        self.steps_since_sort = 0

    # -- stepping ---------------------------------------------------------------
    def _step_params(self, mode: int, dt: float, diagnostics: bool, phase_flags: int = 0) -> _native.StepParams:
        sp = _native.StepParams()
        sp.dt = float(dt)
        sp.mode = mode
        sp.warm_start = 1
        sp.diagnostics = int(bool(diagnostics))
        sp.mg = self.mg
        sp.fixed_point_bits = self.fixed_point_bits
        sp.flags = (_native.GC_STEP_GRAD_GRID if self.grad_grid else 0) | phase_flags
        if self.deposit_next:
            sp.flags |= _native.GC_STEP_DEPOSIT_NEXT
        return sp

    def _step(self, mode: int, dt: float, diagnostics: bool, phase_flags: int = 0) -> StepResult:
        sp = self._step_params(mode, dt, diagnostics, phase_flags)
        st = _native.StepStats()
        p = self._struct(self.cur)
        self.ctx.call("gc_pm_step", C.byref(p), C.byref(sp), C.byref(st), what="gc_pm_step")
        if self.fixed_cycles > 0:
            res = StepResult(int(st.mg.cycles), False, float("nan"))
        else:
            rel = st.mg.res_norm / st.mg.rhs_norm if st.mg.rhs_norm > 0 else 0.0
            res = StepResult(int(st.mg.cycles), bool(st.mg.converged), float(rel))
        if diagnostics:
            res.diag = np.array(st.diag[:], dtype=np.float64)
            res.grid_pe_raw = float(st.grid_pe_raw)
        self.last = res
        return res

    def evaluate(self, diagnostics: bool = True) -> StepResult:
        """Force evaluation (and FP64 diagnostics) of the synchronised state without
        moving it: a PRIME with dt = 0 leaves x and v unchanged."""
        if self.state != "synced":
            raise RuntimeError(f"evaluate needs synchronised state, engine is {self.state!r}")
        return self._step(_native.GC_STEP_PRIME, 0.0, diagnostics)

    def prime(self, dt: float, diagnostics: bool = False) -> StepResult:
        if self.state != "synced":
            raise RuntimeError(f"prime needs synchronised state, engine is {self.state!r}")
        r = self._step(_native.GC_STEP_PRIME, dt, diagnostics)
        self.state = "open"
        return r

    def advance(self, dt: float, diagnostics: bool = False) -> StepResult:
        if self.state != "open":
            raise RuntimeError("advance needs an open (primed) engine")
        if self.sort_every > 0 and self.steps_since_sort >= self.sort_every:
            self.sort(dt)
        r = self._step(_native.GC_STEP_ADVANCE, dt, diagnostics)
        self.steps_since_sort += 1
        return r

    def synchronize(self, dt: float, diagnostics: bool = False) -> StepResult:
        if self.state != "open":
            raise RuntimeError("synchronize needs an open engine")
        r = self._step(_native.GC_STEP_CLOSE, dt, diagnostics)
        self.state = "synced"
        return r

    def last_residual(self) -> float:
        """Relative residual of the last solve (reads the device; synchronises)."""
        r = C.c_double()
        self.ctx.call("gc_pm_last_residual", C.byref(r), what="last_residual")
        return float(r.value)

    # -- CUDA graphs ------------------------------------------------------------
    def step_kernels(self, dt: float) -> None:
        """Launch one ADVANCE step without any host synchronisation (needs
        fixed_cycles > 0). Used to capture the step into a CUDA graph; the host-side
        state does not advance, see advance_graph."""
        if self.fixed_cycles <= 0:
            raise RuntimeError("graph capture needs fixed_cycles > 0 (no host reads inside the step)")
        self._step(_native.GC_STEP_ADVANCE, dt, False)

    def solve_kernels(self, dt: float) -> None:
        """First half of an ADVANCE step (deposit and fixed-cycle solve), no host read."""
        if self.fixed_cycles <= 0:
            raise RuntimeError("split steps need fixed_cycles > 0")
        self._step(_native.GC_STEP_ADVANCE, dt, False, _native.GC_STEP_SOLVE_ONLY)

    def push_kernels(self, dt: float) -> None:
        """Second half: the particle pass on the potential of solve_kernels."""
        self._step(_native.GC_STEP_ADVANCE, dt, False, _native.GC_STEP_PUSH_ONLY)

    def residual_host(self) -> float:
        """Relative residual of the last fixed-cycle solve from the pinned host copy
        it enqueued (call after synchronising; no device access)."""
        r = C.c_double()
        _native.check(self.ctx._lib.gc_pm_residual_host(self.ctx.handle, C.byref(r)), self.ctx.handle,
                      "residual_host")
        return float(r.value)

    def refine(self) -> int:
        """More V-cycles on the pending solve until it meets the tolerance; returns
        how many were run."""
        q = _native.MGParams()
        C.pointer(q)[0] = self.mg
        q.flags &= ~_native.GC_MG_FIXED_CYCLES
        q.max_cycles, q.min_cycles = 60, 0
        n = C.c_int()
        self.ctx.call("gc_pm_refine", C.byref(q), C.byref(n), what="refine")
        return int(n.value)

    def advance_graph(self, dt: float) -> None:
        """advance() through a CUDA graph of the whole step (gc_pm_graph_create),
        captured on first use for each particle-buffer set and dt (the cell sort,
        run between replays, swaps the buffers). The adaptive solve's stopping
        rule is decided on the device, so a replay makes no host read; its
        V-cycles and residual are read with graph_stats() after a
        synchronisation. Needs an open engine that has taken at least three
        steps (complete warm-start history). Ordered after the work already
        queued on the current stream, and the current stream waits for it."""
        if self.state != "open":
            raise RuntimeError("advance_graph needs an open (primed) engine")
        if self.sort_every > 0 and self.steps_since_sort >= self.sort_every:
            self.sort(dt)
        key = (self.cur["x"].data_ptr(), float(dt))
        main = torch.cuda.current_stream()
        gs = self._graph_stream()
        gs.wait_stream(main)
        with torch.cuda.stream(gs):
            g = self._graphs.get(key)
            if g is None:
                g = _native.StepGraph(self.ctx, self._struct(self.cur), self._step_params(_native.GC_STEP_ADVANCE, dt,
                                                                                         False))
                self._graphs[key] = g
            self.ctx.bind_stream()
            g.launch()
        main.wait_stream(gs)
        self.steps_since_sort += 1
        self.last_graph = g

    def launch_graph(self, dt: float):
        """Replay the step graph of the current buffer set on this engine's graph
        stream and return that stream, without ordering it against any other
        stream (the caller does: make it wait for the work the step depends on,
        and wait for it before using the results). For many engines stepping
        concurrently; prepare_graphs first, and sort (with the usual ordering)
        before calling when a sort is due."""
        g = self._graphs[(self.cur["x"].data_ptr(), float(dt))]
        gs = self._graph_stream()
        with torch.cuda.stream(gs):
            self.ctx.bind_stream()
            g.launch()
        self.steps_since_sort += 1
        self.last_graph = g
        return gs

    def prepare_graphs(self, dt: float) -> None:
        """Capture the step graphs of both particle-buffer sets now (a capture
        runs no kernels), so that later advance_graph calls only replay. The
        engine must be open and have stepped (see advance_graph)."""
        if self.state != "open":
            raise RuntimeError("prepare_graphs needs an open (primed) engine")
        main = torch.cuda.current_stream()
        gs = self._graph_stream()
        gs.wait_stream(main)
        with torch.cuda.stream(gs):
            for f in (self.cur, self.alt):
                key = (f["x"].data_ptr(), float(dt))
                if key not in self._graphs:
                    self._graphs[key] = _native.StepGraph(self.ctx, self._struct(f),
                                                          self._step_params(_native.GC_STEP_ADVANCE, dt, False))
        main.wait_stream(gs)

    def _graph_stream(self):
        if getattr(self, "_gstream", None) is None:
            self._gstream = torch.cuda.Stream()
        return self._gstream

    def solve_counters(self, reset: bool = True) -> dict:
        """Totals of the device-decided (graph-replayed) solves since the last
        reset: solves, V-cycles and the largest relative residual (synchronises)."""
        out = (C.c_double * 3)()
        self.ctx.call("gc_pm_solve_counters", out, int(bool(reset)), what="solve_counters")
        return {"solves": int(out[0]), "cycles": int(out[1]), "max_rel_residual": float(out[2])}

    def graph_stats(self) -> StepResult:
        """V-cycles, convergence and relative residual of the last graph-replayed
        step (synchronises the device)."""
        torch.cuda.synchronize()
        c, conv, rel = C.c_int(), C.c_int(), C.c_double()
        _native.check(self.ctx._lib.gc_pm_graph_stats(self.ctx.handle, C.byref(c), C.byref(conv), C.byref(rel)),
                      self.ctx.handle, "graph_stats")
        return StepResult(int(c.value), bool(conv.value), float(rel.value))

    def run(self, steps: int, dt: float) -> None:
        """Advance ``steps`` KDK steps from a synchronised state and end synchronised."""
        if steps <= 0:
            return
        self.prime(dt)
        for _ in range(steps - 1):
            self.advance(dt)
        self.synchronize(dt)

    # -- initial guess of the solve ---------------------------------------------------
    def set_warmstart(self, mode: str = "plain", net=None, track: bool = False) -> None:
        """'plain' (previous potential, the reference's warm start), 'extrapolate'
        (previous + previous change, full resolution) or 'learned' (the
        extrapolation + the network's predicted second difference; ``net`` a
        WarmStartNet with R = G/2)."""
        modes = {"plain": _native.GC_WS_PLAIN, "learned": _native.GC_WS_LEARNED,
                 "extrapolate": _native.GC_WS_EXTRAPOLATE}
        if mode not in modes:
            raise ValueError(f"unknown warm-start mode {mode!r} (expected one of {sorted(modes)})")
        self._ws_net = net  # keep the network alive while attached
        self._graphs = {}   # captured steps embed the initial-guess kernels of the old mode
        h = net._h if net is not None else None
        self.ctx.call("gc_pm_set_warmstart", h, modes[mode], int(bool(track)), what="set_warmstart")

    def record_sample(self, out: torch.Tensor) -> None:
        """Have the next step write its network features (channels 0..3) and the
        second difference of the potential its solve produced (channel 4, the
        training target) into ``out`` (float16, shape (5, G/2, G/2, G/2))."""
        R = self.grid_size // 2
        if out.dtype != torch.float16 or tuple(out.shape) != (5, R, R, R) or not out.is_contiguous() or not out.is_cuda:
            raise ValueError(f"out must be a contiguous CUDA float16 tensor of shape (5, {R}, {R}, {R})")
        self.ctx.call("gc_pm_record_sample", C.c_void_p(out.data_ptr()), what="record_sample")

    # -- output -----------------------------------------------------------------
    def potential(self) -> torch.Tensor:
        """A copy of the current finest-level potential (f32, G^3, grid-origin frame)."""
        G = self.grid_size
        out = torch.empty((G, G, G), dtype=torch.float32, device=self.cur["x"].device)
        self.ctx.call("gc_pm_copy_potential", out.data_ptr(), what="copy potential")
        return out

    def state_arrays(self, physical: bool = True):
        """(pos (N,3), vel (N,3), mass, gid) in original particle order, on the device."""
        order = torch.argsort(self.cur["pid"].long())
        pos = torch.stack([self.cur[k][order] for k in ("x", "y", "z")], dim=1).to(torch.float64)
        if physical:
            pos = pos + torch.as_tensor(self.origin, dtype=torch.float64, device=pos.device)
        vel = torch.stack([self.cur[k][order] for k in ("vx", "vy", "vz")], dim=1)
        return pos, vel, self.cur["m"][order], self.cur["gid"][order]

    def diagnostics_physical(self, diag: np.ndarray) -> dict:
        """Reference diagnostic keys from the engine's FP64 sums (grid-origin frame -> physical)."""
        M, ke = float(diag[0]), float(diag[1])
        P = diag[2:5].copy()
        L = diag[5:8] + np.cross(self.origin, P)
        com = (diag[8:11] / M + self.origin) if M > 0 else np.zeros(3)
        return {"M": M, "kinetic": ke, "momentum": P, "ang_momentum": L, "center_of_mass": com}


__all__ = ["PMEngine", "StepResult"]
