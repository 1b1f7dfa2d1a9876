"""Batched simulations: many independent FastPM runs, each with its own mesh
shape, cosmology and seed, advanced with one launch per phase for the whole
batch.

The reference batches independent simulations with ``jax.vmap`` over its
step (``README.md:29``; ``tests/test_distributed_pm.py:335-409``).  Here the
batch is a table of ``pmgb_sim`` entries (mesh shape, particle count); the
particle arrays are the concatenation, in table order, of every
simulation's ``[np, 3]`` array, and every step is one
``pmgb_fpm_step_batched_f32`` call: one paint launch over all particles,
one batched cuFFT R2C per mesh shape, one k-space launch, one batched C2R
per mesh shape and one gather + kick + drift launch.  Each simulation has
its own kick/drift coefficients (its own cosmology), held on the device as
an ``[n_steps, n_sims]`` table, so a whole run can be captured in one CUDA
graph and replayed.
"""
import numpy as np
import torch

from . import _lib
from .ode import fpm_coefficients


class BatchedFastPM:
    """FastPM steps from ``a0`` to ``a1`` for a batch of simulations.

    ``mesh_shapes[s]`` and ``cosmos[s]`` give simulation ``s``'s mesh and
    cosmology; ``n_particles[s]`` its particle count (default: one particle
    per cell).  Positions and velocities are ``[sum np, 3]`` float32 CUDA
    tensors in each simulation's cell units, updated in place."""

    def __init__(self, mesh_shapes, cosmos, a0, a1, n_steps, n_particles=None, r_split=0.0,
                 device="cuda"):
        self.shapes = [tuple(int(v) for v in s) for s in mesh_shapes]
        if len(cosmos) != len(self.shapes):
            raise ValueError("one cosmology per simulation is required")
        self._setup = (list(cosmos), float(a0), float(a1))
        self.n_sims = len(self.shapes)
        self.counts = ([int(np.prod(s)) for s in self.shapes] if n_particles is None
                       else [int(n) for n in n_particles])
        self.offsets = np.concatenate([[0], np.cumsum(self.counts)]).astype(np.int64)
        self.n = int(self.offsets[-1])
        self.n_steps = int(n_steps)
        self.r_split = float(r_split)
        self.device = torch.device(device)
        self.table = _lib.sim_table(self.shapes, self.counts)
        coef = [fpm_coefficients(c, a0, a1, n_steps) for c in cosmos]
        f = dict(dtype=torch.float32, device=self.device)
        self.kick = torch.tensor(np.stack([k for k, _ in coef], axis=1), **f)
        self.drift = torch.tensor(np.stack([d for _, d in coef], axis=1), **f)
        lib = _lib.load()
        self.ws_bytes = int(lib.pmgb_batch_workspace_size(self.table, self.n_sims))
        if self.ws_bytes == 0:
            _lib.call("pmgb_batch_counts", self.table, self.n_sims, None, None)
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=self.device)
        _lib.call("pmgb_batch_init", self.table, self.n_sims, _lib.ptr(self.ws), self.ws_bytes,
                  _lib.stream(self.device))
        self._lib = lib

    def __del__(self):
        lib = getattr(self, "_lib", None)
        if lib is not None and getattr(self, "ws", None) is not None:
            lib.pmgb_batch_release(_lib.ptr(self.ws))

    def _args(self):
        return self.table, self.n_sims

    def _check(self, *ts):
        _lib.require_cuda(*ts)
        for t in ts:
            if t is not None and t.numel() != 3 * self.n:
                raise ValueError(f"expected [{self.n}, 3] particles, got {tuple(t.shape)}")

    def split(self, a):
        """Per-simulation views of a concatenated ``[sum np, ...]`` array."""
        return [a[self.offsets[s]:self.offsets[s + 1]] for s in range(self.n_sims)]

    def cat(self, parts):
        """Concatenates per-simulation arrays in table order."""
        return torch.cat([p.reshape(-1, 3) for p in parts]).contiguous()

    def step(self, pos, vel, i, pos_before=None, stream=None):
        """Advances every simulation by step ``i`` (``pos_before`` optional:
        receives the positions before the step)."""
        s = _lib.stream(self.device) if stream is None else stream
        _lib.call("pmgb_fpm_step_batched_f32", *self._args(), _lib.ptr(pos), _lib.ptr(vel),
                  _lib.ptr(self.kick[i]), _lib.ptr(self.drift[i]), self.r_split,
                  _lib.ptr(pos_before), _lib.ptr(self.ws), self.ws_bytes, s)

    def run(self, pos, vel, steps=None, start=0):
        """Runs ``steps`` steps (default: all) in place from step ``start``."""
        self._check(pos, vel)
        for i in range(start, start + (self.n_steps - start if steps is None else steps)):
            self.step(pos, vel, i)
        return pos, vel

    def run_host(self, hpos, hvel, steps=None, start=0, groups=4):
        """Steps a batch whose state lives in pinned host memory (``[sum np,
        3]`` float32, table order, updated in place after each step): every
        step copies the particles up, steps them and copies them back.  The
        simulations are split into ``groups`` runs of about equal particle
        counts, each stepped by its own table (``pmgb_fpm_step_batched_f32``
        on the group's simulations): group g's upload, step and read-back
        follow one another, and since the simulations are independent the
        groups overlap, so the host link carries both directions while the
        groups compute.  Group g of the next step goes up as soon as group g
        of this one is down.  Returns when the last copy has been issued
        (ordered before later work on the current stream)."""
        if not (hpos.is_pinned() and hvel.is_pinned()):
            raise ValueError("run_host needs pinned host tensors")
        if hpos.numel() != 3 * self.n or hvel.numel() != 3 * self.n:
            raise ValueError(f"expected [{self.n}, 3] particles")
        start = int(start)
        n = (self.n_steps - start) if steps is None else int(steps)
        if start < 0 or n < 0 or start + n > self.n_steps:
            raise ValueError(f"steps {start}..{start + n - 1} outside the engine's "
                             f"{self.n_steps} steps")
        groups = max(1, min(int(groups), self.n_sims))
        if getattr(self, "_groups_key", None) != groups:
            # cut the table where the running particle count passes g/groups
            cum = self.offsets[1:]
            cuts = [0]
            for g in range(1, groups):
                c = int(np.searchsorted(cum, self.n * g / groups)) + 1
                if cuts[-1] < c < self.n_sims:
                    cuts.append(c)
            cuts.append(self.n_sims)
            cosmos, a0, a1 = self._setup
            self._subs = [(BatchedFastPM(self.shapes[a:b], cosmos[a:b], a0, a1, self.n_steps,
                                         n_particles=self.counts[a:b], r_split=self.r_split,
                                         device=self.device),
                           slice(int(self.offsets[a]), int(self.offsets[b])))
                          for a, b in zip(cuts[:-1], cuts[1:])]
            f = dict(dtype=torch.float32, device=self.device)
            self._host_bufs = (torch.empty((self.n, 3), **f), torch.empty((self.n, 3), **f),
                               torch.cuda.Stream(self.device), torch.cuda.Stream(self.device))
            self._groups_key = groups
        dx, dv, up, down = self._host_bufs
        stream = torch.cuda.current_stream(self.device)
        s = _lib.stream(self.device)
        hp, hv = hpos.reshape(-1, 3), hvel.reshape(-1, 3)
        went_up = [torch.cuda.Event() for _ in self._subs]
        ready = [torch.cuda.Event() for _ in self._subs]
        came_down = [torch.cuda.Event() for _ in self._subs]
        up.wait_stream(stream)
        for i in range(n):
            for g, (eng, sl) in enumerate(self._subs):
                with torch.cuda.stream(up):
                    if i > 0:
                        up.wait_event(came_down[g])
                    dx[sl].copy_(hp[sl], non_blocking=True)
                    dv[sl].copy_(hv[sl], non_blocking=True)
                    went_up[g].record(up)
                stream.wait_event(went_up[g])
                eng.step(dx[sl], dv[sl], start + i, stream=s)
                ready[g].record(stream)
                with torch.cuda.stream(down):
                    down.wait_event(ready[g])
                    hp[sl].copy_(dx[sl], non_blocking=True)
                    hv[sl].copy_(dv[sl], non_blocking=True)
                    came_down[g].record(down)
        stream.wait_stream(down)

    def capture(self, pos, vel):
        """A CUDA graph of the whole run on the buffers ``pos`` / ``vel``
        (updated in place on each replay).  The buffers' contents are left
        as they were."""
        self._check(pos, vel)
        x0, v0 = pos.clone(), vel.clone()
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):  # warm-up outside capture (module loading)
            self.step(pos, vel, 0)
        torch.cuda.current_stream(self.device).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for i in range(self.n_steps):
                self.step(pos, vel, i)
        pos.copy_(x0)
        vel.copy_(v0)
        return g

    def forces(self, pos):
        """``pm_forces`` of every simulation at its particles (``[sum np, 3]``)."""
        self._check(pos)
        out = torch.empty_like(pos)
        _lib.call("pmgb_pm_forces_batched_f32", *self._args(), _lib.ptr(pos), _lib.ptr(out),
                  self.r_split, _lib.ptr(self.ws), self.ws_bytes, _lib.stream(self.device))
        return out

    def paint(self, pos):
        """Unit-mass CIC density of every simulation: a list of meshes."""
        self._check(pos)
        cells = [int(np.prod(s)) for s in self.shapes]
        flat = torch.empty(sum(cells), dtype=torch.float32, device=self.device)
        _lib.call("pmgb_cic_paint_batched_f32", *self._args(), _lib.ptr(flat), _lib.ptr(pos),
                  _lib.ptr(self.ws), self.ws_bytes, _lib.stream(self.device))
        out, o = [], 0
        for sh, c in zip(self.shapes, cells):
            out.append(flat[o:o + c].view(sh))
            o += c
        return out

    def step_vjp(self, x, gx, gv, i, stream=None):
        """Adjoint of step ``i`` taken from positions ``x``: overwrites the
        output cotangents ``(gx, gv)`` with the input cotangents."""
        s = _lib.stream(self.device) if stream is None else stream
        _lib.call("pmgb_fpm_step_batched_vjp_f32", *self._args(), _lib.ptr(x), _lib.ptr(gx),
                  _lib.ptr(gv), _lib.ptr(self.kick[i]), _lib.ptr(self.drift[i]), self.r_split,
                  _lib.ptr(self.ws), self.ws_bytes, s)

    def alloc_store(self):
        """The ``[n_steps, sum np, 3]`` record of positions of ``vjp``."""
        return torch.empty((self.n_steps, self.n, 3), dtype=torch.float32, device=self.device)

    def vjp(self, pos, vel, g_pos, g_vel, store=None):
        """Forward run from ``(pos, vel)`` (recording every step's starting
        positions) and the reverse sweep: returns the final state and the
        cotangents of the initial state for output cotangents
        ``(g_pos, g_vel)``."""
        self._check(pos, vel, g_pos, g_vel)
        x, v = pos.clone(), vel.clone()
        if store is None:
            store = self.alloc_store()
        for i in range(self.n_steps):
            self.step(x, v, i, pos_before=store[i])
        gx, gv = g_pos.clone(), g_vel.clone()
        for i in reversed(range(self.n_steps)):
            self.step_vjp(store[i], gx, gv, i)
        return (x, v), (gx, gv)


def initial_conditions(mesh_shapes, box_sizes, cosmos, seeds, a=0.1, order=2, device="cuda"):
    """Per-simulation LPT particles at scale factor ``a`` from seeded
    Gaussian fields (``pm.linear_field`` + ``pm.lpt`` for each simulation),
    concatenated in table order: ``(pos, vel)`` each ``[sum np, 3]``."""
    from . import distributed, pm
    xs, vs = [], []
    with torch.no_grad():
        for sh, box, c, seed in zip(mesh_shapes, box_sizes, cosmos, seeds):
            sh = tuple(int(v) for v in sh)
            ic = pm.linear_field(sh, list(box), pm.pk_table(c), seed=int(seed), device=device)
            lat = distributed.uniform_particles(sh, device=device).reshape(-1, 3)
            dx, p, _ = pm.lpt(c, ic, lat, a=a, order=order)
            xs.append((lat + dx).contiguous())
            vs.append(p.contiguous())
            del ic, lat, dx
    return torch.cat(xs).contiguous(), torch.cat(vs).contiguous()
