"""The FastPM time loop on one GPU: fused steps, the one-kernel-per-op
comparison form, and a differentiable step with a hand-written adjoint.

A step is one force evaluation plus a kick and a drift (``jaxpm/ode.py:13-82``
driven on the grid ``a_i = a0 + i*dt``).  The fused step is one library
call, ``pmgb_fpm_step_f32``: paint -> R2C -> fused k-space -> batched C2R ->
gather + kick + drift in one kernel.  Positions and velocities are
``[Np, 3]`` float32 CUDA tensors updated in place.
"""
import ctypes

import numpy as np
import torch
from torch.utils.checkpoint import checkpoint

from . import _lib
from .ode import fpm_coefficients
from .painting import _mode


def _ws(nbytes, device):
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)


class FastPM:
    """Runs FastPM steps from ``a0`` to ``a1`` on a fixed mesh.

    ``paint_mode`` selects the painter of the fused step; ``plain=True``
    runs the one-kernel-per-op form instead (global-atomic paint, separate
    k-space multiplies, three gathers, separate kick and drift).
    The workspace is allocated once, for ``n_particles`` particles."""

    def __init__(self, mesh_shape, cosmo, a0, a1, n_steps, n_particles=None, paint_mode="atomic",
                 r_split=0.0, plain=False, device="cuda"):
        self.mesh_shape = tuple(int(s) for s in mesh_shape)
        self.cosmo = cosmo
        self.n_steps = int(n_steps)
        self.kick, self.drift = fpm_coefficients(cosmo, a0, a1, n_steps)
        self.mode = _mode(paint_mode)
        self.r_split = float(r_split)
        self.plain = plain
        self.n_particles = (int(np.prod(self.mesh_shape)) if n_particles is None
                            else int(n_particles))
        nx, ny, nz = self.mesh_shape
        self.ws_bytes = _lib.load().pmgb_pm_workspace_size(
            nx, ny, nz, self.n_particles, _lib.PAINT_ATOMIC if plain else self.mode)
        self.ws = _ws(self.ws_bytes, device)

    def step(self, pos, vel, i, stream=None):
        """Advances ``(pos, vel)`` in place by step ``i``."""
        n = pos.numel() // 3
        if n > self.n_particles:
            raise ValueError("more particles than the workspace was sized for")
        nx, ny, nz = self.mesh_shape
        s = _lib.stream() if stream is None else stream
        if self.plain:
            _lib.call("pmgb_fpm_step_plain_f32", _lib.ptr(pos), _lib.ptr(vel), n, nx, ny, nz,
                      float(self.kick[i]), float(self.drift[i]), self.r_split,
                      _lib.ptr(self.ws), self.ws_bytes, s)
        else:
            _lib.call("pmgb_fpm_step_f32", _lib.ptr(pos), _lib.ptr(vel), n, nx, ny, nz,
                      float(self.kick[i]), float(self.drift[i]), self.r_split, self.mode,
                      _lib.ptr(self.ws), self.ws_bytes, s)

    def run(self, pos, vel, steps=None):
        """Runs ``steps`` (default: all) steps in place and returns
        ``(pos, vel)``."""
        _lib.require_cuda(pos, vel)
        for i in range(self.n_steps if steps is None else steps):
            self.step(pos, vel, i)
        return pos, vel

    def step_vjp(self, x, gx, gv, i, stream=None):
        """Adjoint of step ``i`` taken from positions ``x`` (before the step):
        given the cotangents ``(gx, gv)`` of the step's outputs, overwrites
        them with the cotangents of its inputs.  ``u = gv + drift gx``;
        ``gx += (dF/dx)^T (kick u)``; ``gv = u``."""
        nx, ny, nz = self.mesh_shape
        n = x.numel() // 3
        s = _lib.stream() if stream is None else stream
        if not hasattr(self, "_adj"):
            self._adj = (torch.empty_like(x), torch.empty_like(x))
        ku, gpos = self._adj
        # gv <- gv + drift*gx (= u); ku <- kick*u
        _lib.call("pmgb_lpt_combine_f32", _lib.ptr(gv), _lib.ptr(gx), 3 * n, 1.0,
                  float(self.drift[i]), _lib.ptr(gv), s)
        _lib.call("pmgb_lpt_combine_f32", _lib.ptr(gv), None, 3 * n, float(self.kick[i]), 0.0,
                  _lib.ptr(ku), s)
        mode = _lib.PAINT_ATOMIC if self.plain else self.mode
        _lib.call("pmgb_pm_forces_vjp_f32", _lib.ptr(x), n, nx, ny, nz, self.r_split, mode,
                  _lib.ptr(ku), _lib.ptr(gpos), _lib.ptr(self.ws), self.ws_bytes, s)
        _lib.call("pmgb_lpt_combine_f32", _lib.ptr(gx), _lib.ptr(gpos), 3 * n, 1.0, 1.0,
                  _lib.ptr(gx), s)

    def vjp(self, pos, vel, g_pos, g_vel, store=None):
        """Forward run from ``(pos, vel)`` followed by the reverse sweep:
        returns the final state and the cotangents of the initial state for
        output cotangents ``(g_pos, g_vel)``.  The positions before every
        step are kept (``store`` preallocated ``[n_steps, Np, 3]`` buffer,
        or allocated here); the reverse sweep only needs positions."""
        n = self.n_steps
        x, v = pos.clone(), vel.clone()
        if store is None:
            store = torch.empty((n, *x.shape), dtype=x.dtype, device=x.device)
        for i in range(n):
            store[i].copy_(x)
            self.step(x, v, i)
        gx, gv = g_pos.clone(), g_vel.clone()
        for i in reversed(range(n)):
            self.step_vjp(store[i], gx, gv, i)
        return (x, v), (gx, gv)


class SortedFastPM:
    """The fast FastPM loop: particles kept physically sorted by mesh tile.

    ``load(pos, vel)`` sorts the caller's particles into internal
    double-buffered arrays; ``step(i)`` runs one ``pmgb_fpm_step_sorted_f32``
    (box paint, R2C, fused k-space kernel, batched C2R, box-staged gather +
    kick + drift, tile counting sort); ``state()`` returns positions and
    velocities in the caller's order.  ``stats`` counts the paint and gather
    particles found outside their tile (zero when the ranges are fresh)."""

    def __init__(self, mesh_shape, cosmo, a0, a1, n_steps, n_particles=None, r_split=0.0,
                 device="cuda"):
        self.mesh_shape = tuple(int(s) for s in mesh_shape)
        self.n_steps = int(n_steps)
        self.kick, self.drift = fpm_coefficients(cosmo, a0, a1, n_steps)
        self.r_split = float(r_split)
        n = int(np.prod(self.mesh_shape)) if n_particles is None else int(n_particles)
        self.n = n
        nx, ny, nz = self.mesh_shape
        lib = _lib.load()
        self.ws_bytes = lib.pmgb_pm_workspace_size(nx, ny, nz, n, _lib.PAINT_BINNED)
        self.ws = _ws(self.ws_bytes, device)
        self.sort_bytes = lib.pmgb_tile_sort_workspace_size(nx, ny, nz, n)
        self.sort_ws = _ws(self.sort_bytes, device)
        f = dict(dtype=torch.float32, device=device)
        self.pos = [torch.empty((n, 3), **f), torch.empty((n, 3), **f)]
        self.vel = [torch.empty((n, 3), **f), torch.empty((n, 3), **f)]
        self.ids = [torch.empty(n, dtype=torch.int32, device=device) for _ in range(2)]
        self.cur = 0
        self.stats_buf = torch.zeros(3, dtype=torch.int32, device=device)

    def load(self, pos, vel):
        """Sorts ``pos``/``vel`` ([Np, 3], caller's order) into the engine."""
        pos, vel = pos.contiguous(), vel.contiguous()
        _lib.require_cuda(pos, vel)
        if pos.numel() != 3 * self.n:
            raise ValueError(f"expected {self.n} particles")
        nx, ny, nz = self.mesh_shape
        self.cur = 0
        _lib.call("pmgb_tile_sort_f32", _lib.ptr(pos), _lib.ptr(vel), None, self.n, nx, ny, nz,
                  _lib.ptr(self.pos[0]), _lib.ptr(self.vel[0]), _lib.ptr(self.ids[0]),
                  _lib.ptr(self.sort_ws), self.sort_bytes, _lib.stream())
        self.stats_buf.zero_()

    def step(self, i, stream=None, pos_in=None, pos_out=None, record=None):
        """Runs step ``i``.  ``pos_in``/``pos_out`` replace the internal
        position buffers of this step; ``record = (force3, dest, offsets)``
        keeps what the reverse step needs."""
        a, b = self.cur, 1 - self.cur
        nx, ny, nz = self.mesh_shape
        s = _lib.stream() if stream is None else stream
        f3, dest, offs = record if record is not None else (None, None, None)
        _lib.call("pmgb_fpm_step_sorted_f32",
                  _lib.ptr(self.pos[a] if pos_in is None else pos_in), _lib.ptr(self.vel[a]),
                  _lib.ptr(self.ids[a]), _lib.ptr(self.pos[b] if pos_out is None else pos_out),
                  _lib.ptr(self.vel[b]), _lib.ptr(self.ids[b]), self.n, nx, ny, nz,
                  float(self.kick[i]), float(self.drift[i]), self.r_split, _lib.ptr(self.ws),
                  self.ws_bytes, _lib.ptr(self.sort_ws), self.sort_bytes, _lib.ptr(f3),
                  _lib.ptr(dest), _lib.ptr(offs), _lib.ptr(self.stats_buf), s)
        self.cur = b

    def check(self, stream=None):
        """Raises ``PmgbError`` if a wait on a TMA transfer in one of the tile
        kernels reached its spin limit since the counters were zeroed (the
        kernel then abandoned its work, so the state is invalid):
        ``pmgb_check_stats``, which waits for the stream."""
        s = _lib.stream(self.ws.device) if stream is None else stream
        _lib.call("pmgb_check_stats", _lib.ptr(self.stats_buf), s)

    def run(self, steps=None, start=0, stream=None, check=True):
        """Runs steps ``start .. start+steps-1`` (default: all remaining) with
        one ``pmgb_fpm_run_sorted_f32`` call: each step's gather also paints
        the next step's density.  With ``check`` (default) it then waits for
        the run and raises if a kernel reported a failed wait (``check()``);
        ``check=False`` returns at once (call ``check()`` later)."""
        n = (self.n_steps - start) if steps is None else int(steps)
        if n <= 0:
            return
        nx, ny, nz = self.mesh_shape
        a, b = self.cur, 1 - self.cur
        kick = np.ascontiguousarray(self.kick[start:start + n], dtype=np.float32)
        drift = np.ascontiguousarray(self.drift[start:start + n], dtype=np.float32)
        fp = ctypes.POINTER(ctypes.c_float)
        s = _lib.stream() if stream is None else stream
        _lib.call("pmgb_fpm_run_sorted_f32", _lib.ptr(self.pos[a]), _lib.ptr(self.vel[a]),
                  _lib.ptr(self.ids[a]), _lib.ptr(self.pos[b]), _lib.ptr(self.vel[b]),
                  _lib.ptr(self.ids[b]), self.n, nx, ny, nz, n, kick.ctypes.data_as(fp),
                  drift.ctypes.data_as(fp), self.r_split, _lib.ptr(self.ws), self.ws_bytes,
                  _lib.ptr(self.sort_ws), self.sort_bytes, _lib.ptr(self.stats_buf), s)
        self.cur = a if n % 2 == 0 else b
        if check:
            self.check(s)

    @property
    def positions(self):
        """Current positions in tile order (for order-independent uses such
        as painting the density)."""
        return self.pos[self.cur]

    @property
    def ids_current(self):
        return self.ids[self.cur]

    def run_host(self, hpos, hvel, steps=None, chunks=16, start=0, check=True,
                 paint_mode="binned"):
        """Steps a state that lives in pinned host memory: ``hpos``/``hvel``
        ([Np, 3] float32, caller's order) are updated in place after each of
        steps ``start .. start+steps-1`` (default: all remaining; a range
        past the engine's steps raises before any work is queued); every
        step copies them up, steps them and copies them back, in ``chunks``
        pieces on two copy streams.

        Where the potential pipeline serves the mesh the step is streamed
        through the host link: the position pieces go up first and each is
        painted (``pmgb_cic_paint_f32``, ``paint_mode``, accumulating) as
        soon as it has landed; the velocity pieces follow and are in flight
        while the forces are evaluated after the last position piece
        (``pmgb_mesh_forces_f32``: the potential and its order-1 gradient
        stencil); each piece is then gathered, kicked and drifted
        (``pmgb_read3_kick_drift_f32``) and goes back down, positions
        before velocities, and piece c of the next step's positions
        (velocities) goes up as soon as piece c of this step's positions
        (velocities) is down.  The link then carries both directions
        through the whole step.  Otherwise each step sorts the state by tile
        (``pmgb_tile_sort_f32``), runs the composite step
        (``pmgb_fpm_step_sorted_f32``) and returns it to the caller's order
        (``pmgb_unpermute3_f32``) before copying it back.

        After the call the engine holds the last state, sorted by tile.
        With ``check`` (default) it waits for the steps and raises if a
        kernel reported a failed wait; otherwise it returns when the last
        copy has been issued (ordered before later work on the current
        stream)."""
        if not (hpos.is_pinned() and hvel.is_pinned()):
            raise ValueError("run_host needs pinned host tensors")
        start = int(start)
        n = (self.n_steps - start) if steps is None else int(steps)
        if start < 0 or n < 0 or start + n > self.n_steps:
            raise ValueError(f"steps {start}..{start + n - 1} outside the engine's "
                             f"{self.n_steps} steps")
        if paint_mode not in ("atomic", "binned", "deterministic"):
            raise ValueError(f"unknown paint_mode {paint_mode!r}")
        nx, ny, nz = self.mesh_shape
        dev = self.ws.device
        stream = torch.cuda.current_stream(dev)
        s = _lib.stream(dev)
        if not hasattr(self, "_host_bufs"):
            f = dict(dtype=torch.float32, device=dev)
            self._host_bufs = (torch.empty((self.n, 3), **f), torch.empty((self.n, 3), **f),
                               torch.cuda.Stream(dev), torch.cuda.Stream(dev))
        dx, dv, up, down = self._host_bufs
        lib = _lib.load()
        streamed = (bool(lib.pmgb_fft3_supported(nx, ny, nz)) and lib.pmgb_fft_path() != 0 and
                    nz % 4 == 0)
        bounds = np.linspace(0, self.n, int(chunks) + 1).astype(np.int64)
        parts = [slice(int(a), int(b)) for a, b in zip(bounds[:-1], bounds[1:])]
        came_down = [torch.cuda.Event() for _ in parts]
        ready = [torch.cuda.Event() for _ in parts]
        went_up = [torch.cuda.Event() for _ in parts]
        # the streamed schedule's positions and velocities, piece by piece
        pos_down = [torch.cuda.Event() for _ in parts]
        vel_down = [torch.cuda.Event() for _ in parts]
        pos_up = [torch.cuda.Event() for _ in parts]
        vel_up = [torch.cuda.Event() for _ in parts]
        up.wait_stream(stream)

        def upload(i, c, sl):
            with torch.cuda.stream(up):
                if i > 0:
                    up.wait_event(came_down[c])
                dx[sl].copy_(hpos[sl], non_blocking=True)
                dv[sl].copy_(hvel[sl], non_blocking=True)
                went_up[c].record(up)

        def download(c, sl):
            with torch.cuda.stream(down):
                down.wait_event(ready[c])
                hpos[sl].copy_(dx[sl], non_blocking=True)
                hvel[sl].copy_(dv[sl], non_blocking=True)
                came_down[c].record(down)

        if streamed:
            from .painting import MODES
            mode = MODES[paint_mode]
            big = max(sl.stop - sl.start for sl in parts)
            key = (paint_mode, big)
            if getattr(self, "_stream_key", None) != key:
                mb = lib.pmgb_mesh_forces_workspace_size(nx, ny, nz)
                pb = max(int(lib.pmgb_cic_paint_workspace_size(nx, ny, nz, big, mode)), 1)
                f = dict(dtype=torch.float32, device=dev)
                self._stream_bufs = (torch.empty((nx, ny, nz), **f),
                                     torch.empty((3, nx, ny, nz), **f),
                                     torch.empty(mb, dtype=torch.uint8, device=dev), mb,
                                     torch.empty(pb, dtype=torch.uint8, device=dev), pb)
                self._stream_key = key
            mesh, f3, mws, mb, pws, pb = self._stream_bufs
            cs = nx * ny * nz
            for i in range(n):
                kick, drift = float(self.kick[start + i]), float(self.drift[start + i])
                # the density, piece by piece as the position pieces land
                for c, sl in enumerate(parts):
                    with torch.cuda.stream(up):
                        if i > 0:
                            up.wait_event(pos_down[c])
                        dx[sl].copy_(hpos[sl], non_blocking=True)
                        pos_up[c].record(up)
                    stream.wait_event(pos_up[c])
                    _lib.call("pmgb_cic_paint_f32", _lib.ptr(mesh), nx, ny, nz, _lib.ptr(dx[sl]),
                              sl.stop - sl.start, None, 1.0, mode, 1 if c else 0, _lib.ptr(pws),
                              pb, s)
                # the velocities go up while the forces are evaluated
                with torch.cuda.stream(up):
                    for c, sl in enumerate(parts):
                        if i > 0:
                            up.wait_event(vel_down[c])
                        dv[sl].copy_(hvel[sl], non_blocking=True)
                        vel_up[c].record(up)
                _lib.call("pmgb_mesh_forces_f32", _lib.ptr(mesh), _lib.ptr(f3), nx, ny, nz,
                          self.r_split, _lib.ptr(mws), mb, s)
                # gather + kick + drift piece by piece; positions down first
                for c, sl in enumerate(parts):
                    stream.wait_event(vel_up[c])
                    _lib.call("pmgb_read3_kick_drift_f32", _lib.ptr(f3), cs, nx, ny, nz,
                              _lib.ptr(dx[sl]), _lib.ptr(dv[sl]), sl.stop - sl.start, kick,
                              drift, None, s)
                    ready[c].record(stream)
                    with torch.cuda.stream(down):
                        down.wait_event(ready[c])
                        hpos[sl].copy_(dx[sl], non_blocking=True)
                        pos_down[c].record(down)
                with torch.cuda.stream(down):
                    for c, sl in enumerate(parts):
                        hvel[sl].copy_(dv[sl], non_blocking=True)
                        vel_down[c].record(down)
        else:
            for i in range(n):
                kick, drift = float(self.kick[start + i]), float(self.drift[start + i])
                for c, sl in enumerate(parts):
                    upload(i, c, sl)
                for ev in went_up:
                    stream.wait_event(ev)
                _lib.call("pmgb_tile_sort_f32", _lib.ptr(dx), _lib.ptr(dv), None, self.n, nx, ny,
                          nz, _lib.ptr(self.pos[0]), _lib.ptr(self.vel[0]),
                          _lib.ptr(self.ids[0]), _lib.ptr(self.sort_ws), self.sort_bytes, s)
                _lib.call("pmgb_fpm_step_sorted_f32", _lib.ptr(self.pos[0]),
                          _lib.ptr(self.vel[0]), _lib.ptr(self.ids[0]), _lib.ptr(self.pos[1]),
                          _lib.ptr(self.vel[1]), _lib.ptr(self.ids[1]), self.n, nx, ny, nz, kick,
                          drift, self.r_split, _lib.ptr(self.ws), self.ws_bytes,
                          _lib.ptr(self.sort_ws), self.sort_bytes, None, None, None,
                          _lib.ptr(self.stats_buf), s)
                _lib.call("pmgb_unpermute3_f32", _lib.ptr(self.pos[1]), _lib.ptr(self.ids[1]),
                          self.n, _lib.ptr(dx), s)
                _lib.call("pmgb_unpermute3_f32", _lib.ptr(self.vel[1]), _lib.ptr(self.ids[1]),
                          self.n, _lib.ptr(dv), s)
                for c, sl in enumerate(parts):
                    ready[c].record(stream)
                    download(c, sl)
        stream.wait_stream(down)
        if n > 0:  # the engine's buffers: the last state, sorted by tile
            _lib.call("pmgb_tile_sort_f32", _lib.ptr(dx), _lib.ptr(dv), None, self.n, nx, ny, nz,
                      _lib.ptr(self.pos[0]), _lib.ptr(self.vel[0]), _lib.ptr(self.ids[0]),
                      _lib.ptr(self.sort_ws), self.sort_bytes, s)
            self.cur = 0
        if check:
            self.check(s)

    def state(self):
        """``(pos, vel)`` in the caller's order (new tensors)."""
        out_p = torch.empty_like(self.pos[self.cur])
        out_v = torch.empty_like(self.vel[self.cur])
        s = _lib.stream()
        for src, dst in ((self.pos[self.cur], out_p), (self.vel[self.cur], out_v)):
            _lib.call("pmgb_unpermute3_f32", _lib.ptr(src), _lib.ptr(self.ids[self.cur]), self.n,
                      _lib.ptr(dst), s)
        return out_p, out_v

    @property
    def stats(self):
        """Particles found outside their tile by the paint and the gather
        (0 unless the tile ranges were stale)."""
        c = self.stats_buf.cpu().tolist()
        return {"paint": c[0], "gather": c[1], "tma_wait_timeout": c[2]}

    def alloc_store(self, potential=None):
        """Buffers of what the forward run records for the reverse sweep:
        ``(positions [n,Np,3], meshes, dest [n,Np], tile ranges [n,keys+1])``
        with ``meshes`` each step's three force meshes ``[n,3,nx,ny,nz]``
        or, with ``potential``, its potential ``[n,nx,ny,nz]`` (a third of
        the mesh bytes; the reverse gather then derives each tile's forces
        from the potential, 0.8 ms per step slower at 512^3).  The default
        (None) records force meshes unless they would not fit in the free
        device memory and the potential pipeline serves the mesh shape."""
        n, dev = self.n_steps, self.ws.device
        nx, ny, nz = self.mesh_shape
        lib = _lib.load()
        if potential is None:
            free = torch.cuda.mem_get_info(dev)[0]
            f3_bytes = 4 * n * (3 * self.n + 3 * nx * ny * nz + self.n)
            potential = f3_bytes > 0.9 * free and bool(lib.pmgb_fft3_supported(nx, ny, nz))
        keys = lib.pmgb_tile_key_count(nx, ny, nz)
        meshes = (n, nx, ny, nz) if potential else (n, 3, nx, ny, nz)
        return (torch.empty((n, self.n, 3), dtype=torch.float32, device=dev),
                torch.empty(meshes, dtype=torch.float32, device=dev),
                torch.empty((n, self.n), dtype=torch.int32, device=dev),
                torch.empty((n, keys + 1), dtype=torch.int32, device=dev))

    def vjp(self, pos, vel, g_pos, g_vel, store=None, check=True, coef_grads=False):
        """Forward run from ``(pos, vel)`` (caller's order) then the reverse
        sweep; returns the final state and the cotangents of the initial
        state, all in the caller's order.  With ``check`` (default) it waits
        for the sweep and raises if a kernel reported a failed wait.

        With ``coef_grads`` it also returns the cotangents of every step's
        coefficients (float64 arrays): ``<u_i, F_i(x_i)>`` for the kick
        (``u_i`` the velocity cotangent the reverse step returns, ``F_i``
        read from the recorded force meshes at the recorded positions) and
        ``<g_x(i+1), v'_i>`` for the drift (``v'_i`` from the positions the
        step started and ended with, ``(x_{i+1} - x_i) / drift``); it needs
        the store of force meshes.

        Each forward step records the positions it starts from, its
        potential (or its force meshes, by the store's layout), where each
        particle moved in the re-sort and the tile ranges (``store`` from
        ``alloc_store()``, or allocated here).  The reverse
        sweep then runs in tile order throughout: the cotangents are put in
        the final tile order once, each ``pmgb_fpm_step_sorted_vjp_f32``
        pulls them one re-sort back, and the result is returned to the
        caller's order once."""
        n = self.n_steps
        nx, ny, nz = self.mesh_shape
        if store is None:
            store = self.alloc_store()
        xs, f3s, dests, offs = store
        pot = f3s.dim() == 4  # [n, nx, ny, nz]: the potentials
        if coef_grads and pot:
            raise ValueError("coef_grads needs the store of force meshes")
        record = "pmgb_fpm_run_sorted_record_pot_f32" if pot else "pmgb_fpm_run_sorted_record_f32"
        reverse = "pmgb_fpm_step_sorted_vjp_pot_f32" if pot else "pmgb_fpm_step_sorted_vjp_f32"
        self.load(pos, vel)
        ids0 = self.ids[self.cur].clone()
        if n:
            # the recording forward as one run (pmgb_fpm_run_sorted_record_f32)
            xs[0].copy_(self.pos[self.cur])
            a, b = self.cur, 1 - self.cur
            last = a if n % 2 == 0 else b
            kick = np.ascontiguousarray(self.kick[:n], dtype=np.float32)
            drift = np.ascontiguousarray(self.drift[:n], dtype=np.float32)
            fp = ctypes.POINTER(ctypes.c_float)
            _lib.call(record, _lib.ptr(xs), _lib.ptr(self.vel[a]),
                      _lib.ptr(self.ids[a]), _lib.ptr(self.vel[b]), _lib.ptr(self.ids[b]),
                      _lib.ptr(self.pos[last]), self.n, nx, ny, nz, n, kick.ctypes.data_as(fp),
                      drift.ctypes.data_as(fp), self.r_split, _lib.ptr(self.ws), self.ws_bytes,
                      _lib.ptr(self.sort_ws), self.sort_bytes, _lib.ptr(f3s), _lib.ptr(dests),
                      _lib.ptr(offs), _lib.ptr(self.stats_buf), _lib.stream())
            self.cur = last
        final = self.state()
        if not hasattr(self, "_adj"):
            e = lambda: torch.empty((self.n, 3), dtype=torch.float32, device=self.ws.device)  # noqa
            self._adj = (e(), e(), e(), e())
        gxa, gva, gxb, gvb = self._adj
        s = _lib.stream()
        idn = self.ids[self.cur]
        _lib.call("pmgb_permute3_f32", _lib.ptr(g_pos.contiguous()), _lib.ptr(idn), self.n,
                  _lib.ptr(gxa), s)
        _lib.call("pmgb_permute3_f32", _lib.ptr(g_vel.contiguous()), _lib.ptr(idn), self.n,
                  _lib.ptr(gva), s)
        # per step: <u_i, F_i(x_i)> and <g_x(i+1), x(i+1) - x_i>, summed on the
        # device (pmgb_fpm_coef_cotangents_f32) and read back once
        coef = torch.zeros((n, 2), dtype=torch.float64, device=gxa.device) if coef_grads \
            else None
        for i in reversed(range(n)):
            _lib.call(reverse, _lib.ptr(xs[i]), _lib.ptr(f3s[i]),
                      _lib.ptr(dests[i]), _lib.ptr(offs[i]), _lib.ptr(gxa), _lib.ptr(gva),
                      _lib.ptr(gxb), _lib.ptr(gvb), self.n, nx, ny, nz, float(self.kick[i]),
                      float(self.drift[i]), self.r_split, _lib.ptr(self.ws), self.ws_bytes,
                      _lib.ptr(self.stats_buf), s)
            gxa, gxb, gva, gvb = gxb, gxa, gvb, gva
            if coef_grads:
                # u_i is now in gva; the step's output cotangents stay in gxb
                x_next = xs[i + 1] if i + 1 < n else self.pos[self.cur]
                _lib.call("pmgb_fpm_coef_cotangents_f32", _lib.ptr(xs[i]), _lib.ptr(x_next),
                          _lib.ptr(dests[i]), _lib.ptr(f3s[i]), nx * ny * nz, nx, ny, nz,
                          _lib.ptr(gxb), _lib.ptr(gva), self.n, _lib.ptr(coef[i]), s)
        gx, gv = torch.empty_like(gxa), torch.empty_like(gva)
        _lib.call("pmgb_unpermute3_f32", _lib.ptr(gxa), _lib.ptr(ids0), self.n, _lib.ptr(gx), s)
        _lib.call("pmgb_unpermute3_f32", _lib.ptr(gva), _lib.ptr(ids0), self.n, _lib.ptr(gv), s)
        if check:
            self.check(s)
        if coef_grads:
            c = coef.cpu().numpy()
            return final, (gx, gv), (c[:, 0].copy(), c[:, 1] / np.asarray(self.drift[:n]))
        return final, (gx, gv)


def _combine(x, y, cx, cy):
    out = torch.empty_like(x)
    _lib.call("pmgb_lpt_combine_f32", _lib.ptr(x), _lib.ptr(y), x.numel(), float(cx), float(cy),
              _lib.ptr(out), _lib.stream())
    return out


class _Step(torch.autograd.Function):
    """One FastPM step ``(x, v) -> (x', v')`` with
    ``v' = v + kick F(x)``, ``x' = x + drift v'``.

    Backward, given ``(gx', gv')``: ``u = gv' + drift gx'``,
    ``gx = gx' + (dF/dx)^T (kick u)`` (one ``pmgb_pm_forces_vjp_f32``),
    ``gv = u``.  ``kick`` and ``drift`` may be 0-dim tensors that require
    grad (coefficients that depend on the cosmology): their cotangents are
    ``<u, F(x)>`` (one more force evaluation) and ``<gx', v'>``."""

    @staticmethod
    def forward(ctx, x, v, mesh_shape, kick, drift, mode, r_split):
        nx, ny, nz = mesh_shape
        n = x.numel() // 3
        xo, vo = x.clone(), v.clone()
        wsb = _lib.load().pmgb_pm_workspace_size(nx, ny, nz, n, mode)
        ws = _ws(wsb, x.device)
        _lib.call("pmgb_fpm_step_f32", _lib.ptr(xo), _lib.ptr(vo), n, nx, ny, nz, float(kick),
                  float(drift), float(r_split), mode, _lib.ptr(ws), wsb, _lib.stream())
        coef_grad = torch.is_tensor(drift) and drift.requires_grad
        ctx.save_for_backward(x, vo if coef_grad else None)
        ctx.coef = (kick if torch.is_tensor(kick) else None,
                    drift if torch.is_tensor(drift) else None)
        ctx.args = (mesh_shape, float(kick), float(drift), mode, float(r_split))
        return xo, vo

    @staticmethod
    def backward(ctx, gx, gv):
        x, vo = ctx.saved_tensors
        (nx, ny, nz), kick, drift, mode, r_split = ctx.args
        gx = torch.zeros_like(x) if gx is None else gx.contiguous()
        gv = torch.zeros_like(x) if gv is None else gv.contiguous()
        u = _combine(gv, gx, 1.0, drift)
        ku = _combine(u, None, kick, 0.0)
        n = x.numel() // 3
        wsb = _lib.load().pmgb_pm_workspace_size(nx, ny, nz, n, mode)
        ws = _ws(wsb, x.device)
        gpos = torch.empty_like(x)
        _lib.call("pmgb_pm_forces_vjp_f32", _lib.ptr(x), n, nx, ny, nz, r_split, mode,
                  _lib.ptr(ku), _lib.ptr(gpos), _lib.ptr(ws), wsb, _lib.stream())
        g_kick = g_drift = None
        kt, dt = ctx.coef
        if kt is not None and ctx.needs_input_grad[3]:
            F = torch.empty_like(x)
            _lib.call("pmgb_pm_forces_f32", _lib.ptr(x), n, nx, ny, nz, r_split, mode,
                      _lib.ptr(F), _lib.ptr(ws), wsb, _lib.stream())
            g_kick = (u.double() * F.double()).sum().to(kt.dtype).to(kt.device)
        if dt is not None and ctx.needs_input_grad[4] and vo is not None:
            g_drift = (gx.double() * vo.double()).sum().to(dt.dtype).to(dt.device)
        return _combine(gx, gpos, 1.0, 1.0), u, None, g_kick, g_drift, None, None


def fpm_step(x, v, mesh_shape, kick, drift, paint_mode="atomic", r_split=0.0):
    """Differentiable fused FastPM step (new tensors; inputs unchanged)."""
    x, v = x.contiguous(), v.contiguous()
    _lib.require_cuda(x, v)
    return _Step.apply(x, v, tuple(mesh_shape), kick, drift, _mode(paint_mode), r_split)


# segment engines of the sorted differentiable path, one per (device, mesh,
# particle count, segment length, r_split): their workspaces outlive a call.
# The two most recently used are kept; release_segment_engines() drops all.
_SEGMENT_ENGINES = {}
_SEGMENT_KEEP = 2


def release_segment_engines():
    """Frees the device memory the sorted differentiable path keeps between
    calls (its engines' buffers and recording stores)."""
    _SEGMENT_ENGINES.clear()


def _segment_engine(mesh_shape, n, steps, r_split, device):
    key = (str(device), tuple(mesh_shape), int(n), int(steps), float(r_split))
    eng = _SEGMENT_ENGINES.pop(key, None)
    if eng is None:
        from .cosmology import Planck15
        while len(_SEGMENT_ENGINES) >= _SEGMENT_KEEP:
            _SEGMENT_ENGINES.pop(next(iter(_SEGMENT_ENGINES)))
        # the coefficients are replaced by the segment's before every use;
        # the recording store is made by the first backward pass
        eng = SortedFastPM(mesh_shape, Planck15(), 0.1, 1.0, steps, n_particles=n,
                           r_split=r_split, device=device)
        eng.store = None
    _SEGMENT_ENGINES[key] = eng  # most recently used last
    return eng


class _SortedSegment(torch.autograd.Function):
    """``len(kick)`` FastPM steps ``(x, v) -> (x', v')`` on the tile-sorted
    engine.  Forward: the run loop (``pmgb_fpm_run_sorted_f32``), nothing
    kept but the segment's first state.  Backward: the recording forward
    run from that state and the reverse sweep
    (``pmgb_fpm_step_sorted_vjp_f32`` per step), which also yields the
    cotangents of the per-step coefficients ``kick`` and ``drift`` (1-D
    tensors that may require grad)."""

    @staticmethod
    def forward(ctx, x, v, kick, drift, mesh_shape, r_split):
        n = x.numel() // 3
        eng = _segment_engine(mesh_shape, n, kick.numel(), r_split, x.device)
        eng.kick = kick.detach().double().cpu().numpy().copy()
        eng.drift = drift.detach().double().cpu().numpy().copy()
        eng.load(x.contiguous(), v.contiguous())
        eng.run()
        xo, vo = eng.state()
        ctx.save_for_backward(x, v, kick, drift)
        ctx.args = (mesh_shape, r_split)
        return xo, vo

    @staticmethod
    def backward(ctx, gx, gv):
        x, v, kick, drift = ctx.saved_tensors
        mesh_shape, r_split = ctx.args
        eng = _segment_engine(mesh_shape, x.numel() // 3, kick.numel(), r_split, x.device)
        eng.kick = kick.detach().double().cpu().numpy().copy()
        eng.drift = drift.detach().double().cpu().numpy().copy()
        gx = torch.zeros_like(x) if gx is None else gx.contiguous()
        gv = torch.zeros_like(x) if gv is None else gv.contiguous()
        need_coef = ctx.needs_input_grad[2] or ctx.needs_input_grad[3]
        if eng.store is None:
            eng.store = eng.alloc_store(potential=False)
        out = eng.vjp(x.contiguous(), v.contiguous(), gx, gv, store=eng.store,
                      coef_grads=need_coef)
        g_x, g_v = out[1]
        g_kick = g_drift = None
        if need_coef:
            gk, gd = out[2]
            g_kick = torch.as_tensor(gk, dtype=kick.dtype, device=kick.device)
            g_drift = torch.as_tensor(gd, dtype=drift.dtype, device=drift.device)
        return g_x.reshape(x.shape), g_v.reshape(v.shape), g_kick, g_drift, None, None


def _sorted_supported(mesh_shape, n):
    """The tile-sorted engine's limits: 32-bit particle slots, at most 256
    tiles (2048 cells) per axis."""
    return n < (1 << 32) - 1 and max(int(a) for a in mesh_shape) <= 2048


def nbody(pos, vel, cosmo, mesh_shape, a0, a1, n_steps, paint_mode="atomic", r_split=0.0,
          checkpoint_every=0, coefficients=None, engine="lattice"):
    """Differentiable FastPM integration from ``a0`` to ``a1`` in
    ``n_steps`` steps; returns the final ``(pos, vel)``.  With
    ``checkpoint_every = k > 0`` only every k-th state is kept for the
    backward pass and the steps in between are recomputed.
    ``coefficients`` (optional): the per-step ``(kick, drift)`` as 1-D
    tensors, which may require grad (see ``forward_model``); by default
    they are computed from ``cosmo``.

    ``engine="sorted"`` runs each segment of ``checkpoint_every`` steps
    (the whole run when it is 0) on the tile-sorted engine: the run loop
    forward, the recording forward and the reverse sweep backward
    (``_SortedSegment``); it keeps the recorded force meshes of one
    segment at a time, and paints with the engine's own fixed-point tile
    boxes whatever ``paint_mode`` says.  ``"lattice"`` differentiates step by step
    (``fpm_step``), painting with ``paint_mode``."""
    if coefficients is None:
        kick, drift = fpm_coefficients(cosmo, a0, a1, n_steps)
    else:
        kick, drift = coefficients
    if engine not in ("lattice", "sorted"):
        raise ValueError(f"unknown engine {engine!r}")
    if engine == "sorted" and _sorted_supported(mesh_shape, pos.numel() // 3):
        k = checkpoint_every if checkpoint_every and checkpoint_every > 0 else n_steps
        kt = kick if torch.is_tensor(kick) else torch.as_tensor(np.asarray(kick), dtype=torch.float64)
        dt = drift if torch.is_tensor(drift) else torch.as_tensor(np.asarray(drift),
                                                                   dtype=torch.float64)
        x, v = pos, vel
        for lo in range(0, n_steps, k):
            hi = min(n_steps, lo + k)
            x, v = _SortedSegment.apply(x, v, kt[lo:hi], dt[lo:hi], tuple(mesh_shape),
                                        float(r_split))
        return x, v

    def segment(x, v, lo, hi):
        for i in range(lo, hi):
            x, v = fpm_step(x, v, mesh_shape, kick[i], drift[i], paint_mode, r_split)
        return x, v

    if checkpoint_every and checkpoint_every > 0:
        for lo in range(0, n_steps, checkpoint_every):
            hi = min(n_steps, lo + checkpoint_every)
            pos, vel = checkpoint(segment, pos, vel, lo, hi, use_reentrant=False)
        return pos, vel
    return segment(pos, vel, 0, n_steps)
