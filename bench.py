"""Benchmark of the FastPM particle-mesh step on GB300.

Workload: 512^3 particles on a 512^3 mesh (FP32 positions and
velocities), box 512 Mpc/h, Planck15 cosmology, initial conditions from a
seeded Gaussian random field (NumPy PCG64 white noise coloured by the
Eisenstein-Hu linear power spectrum), 2LPT to a = 0.1, then K FastPM steps
(K = --steps, 20 by default) linear in a up to a = 1.  One step is one
force evaluation (paint, R2C, fused k-space kernel, batched C2R) plus the
fused gather + kick + drift over all particles.

Metric: particle-steps per second (Np * K / time of the K timed steps).
The JSON line also carries: the forward+adjoint rate (hand-written
adjoint, positions stored every step), the one-kernel-per-op GPU form,
the end-to-end rate through the C ABI with host buffers, per-phase times,
the roofline of the dominant kernel, the CPU baseline (the NumPy oracle on
the host cores) and the SM clocks sampled during the timed region.

``--impl reference`` times the reference's algorithm on the CPU instead
(the NumPy restatement in ``oracle/``; JAX is not available), printing
the same metric.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

# chunks of the end-to-end leg's host copies (see the e2e leg)
E2E_CHUNKS = 16
# groups of simulations of the batched workload's end-to-end leg
E2E_GROUPS = 4

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 512
BOX_PER_CELL = 1.0  # box 512 Mpc/h on 512^3


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--workload", default="step", choices=["step", "batched", "paint", "grad"],
                    help="step: the 512^3 FastPM step (headline); batched: 64 simulations "
                         "of 64^3-128^3; paint: cic_paint/cic_read microbenchmarks; grad: "
                         "gradients w.r.t. noise and cosmology")
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 40 for the 512^3 step, the large "
                         "configuration's step count; 20 for the others)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mesh", type=int, default=N_DEFAULT)
    ap.add_argument("--engine", default="sorted", choices=["sorted", "lattice"])
    ap.add_argument("--paint-mode", default="atomic", help="painter of the lattice engine")
    ap.add_argument("--skip", default="", help="comma list of legs to skip: "
                    "adjoint,plain,e2e,cpu,clocks,paint,1024,tune")
    ap.add_argument("--phases-only", action="store_true")
    ap.add_argument("--repeats", type=int, default=5,
                    help="timed repetitions of each K-step run (the median is reported)")
    ap.add_argument("--tuning", default=None,
                    help="JSON object of run-loop tuning fields to set instead of autotuning")
    ap.add_argument("--fft", default=None, choices=["cufft", "fused", "own"],
                    help="FFT path of the force evaluation (library default if omitted)")
    return ap.parse_args()


class nvtx:
    """An NVTX range (for `ncu --nvtx --nvtx-include <name>/`)."""

    def __init__(self, name):
        self.name = name

    def __enter__(self):
        import torch
        torch.cuda.nvtx.range_push(self.name)

    def __exit__(self, *exc):
        import torch
        torch.cuda.nvtx.range_pop()


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


def max_over_ranks(value, world):
    """Maximum of a per-rank value (the slowest replica's time)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(particles_per_rank, steps, ms_max, world):
    """Whole-job particle-steps/s of `world` independent replicas, timed by
    the slowest one."""
    return world * particles_per_rank * steps / (ms_max / 1e3)


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        rows = [r.split(",") for r in out.strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if "Active" in v and
                          "Not" not in v})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def initial_state(n, cosmo, device, seed=0):
    """2LPT particles at a = 0.1 from a seeded Gaussian random field."""
    import torch
    from jaxpm_gb300 import distributed, pm
    box = [n * BOX_PER_CELL] * 3
    ic = pm.linear_field((n,) * 3, box, pm.pk_table(cosmo), seed=seed, device=device)
    lat = distributed.uniform_particles((n,) * 3, device=device).reshape(-1, 3)
    with torch.no_grad():
        dx, p, _ = pm.lpt(cosmo, ic, lat, a=0.1, order=2)
        x = (lat + dx).contiguous()
        v = p.contiguous()
    del ic, lat, dx
    return x, v


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def link_rates(ha, hb, dev):
    """GB/s of the host link for the pinned arrays ha, hb (the same size):
    ha up alone, ha down alone, and ha up while hb goes down (two streams),
    each the median of 3 copies timed with CUDA events."""
    import torch
    da, db = torch.empty_like(ha, device=dev), torch.empty_like(hb, device=dev)
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    cur = torch.cuda.current_stream(dev)
    nb = ha.numel() * ha.element_size()

    def timed(fn, nbytes):
        out = []
        for _ in range(3):
            torch.cuda.synchronize(dev)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(cur)
            fn()
            b.record(cur)
            torch.cuda.synchronize(dev)
            out.append(a.elapsed_time(b))
        return nbytes / (float(np.median(out)) / 1e3) / 1e9

    def both():
        s1.wait_stream(cur)
        s2.wait_stream(cur)
        with torch.cuda.stream(s1):
            da.copy_(ha, non_blocking=True)
        with torch.cuda.stream(s2):
            hb.copy_(db, non_blocking=True)
        cur.wait_stream(s1)
        cur.wait_stream(s2)

    rates = {"up": timed(lambda: da.copy_(ha, non_blocking=True), nb),
             "down": timed(lambda: ha.copy_(da, non_blocking=True), nb),
             "both": timed(both, 2 * nb)}
    del da, db
    return rates


def profile_traffic():
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu
    summary (``profiles/traffic.md``: lines ``kernel: bytes_per_particle``),
    scaled to this run's particle count by the caller."""
    path = os.path.join(ROOT, "profiles", "traffic.md")
    out = {}
    try:
        for line in open(path):
            if line.startswith("traffic_per_particle "):
                _, k, v = line.split()
                out[k] = float(v)
    except OSError:
        pass
    return out


def run_gb300(args):
    import torch
    from jaxpm_gb300 import _lib, cosmology, painting, simulate, utils

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    lib = _lib.load()
    if args.fft is not None:
        from jaxpm_gb300 import distributed
        distributed.set_fft_path(args.fft)
    skip = set(filter(None, args.skip.split(",")))
    n = args.mesh
    Np = n**3
    K, W = args.steps, args.warmup
    cosmo = cosmology.Planck15()
    engine = args.engine
    mode = _lib.PAINT_BINNED if engine == "sorted" else painting._mode(args.paint_mode)

    x0, v0 = initial_state(n, cosmo, dev)
    stream = torch.cuda.current_stream(dev)
    s = _lib.stream(dev)
    nx = ny = nz = n
    ncell = n**3
    mf_bytes = lib.pmgb_mesh_forces_workspace_size(nx, ny, nz)
    fft_path = lib.pmgb_fft_path() if lib.pmgb_fft3_supported(nx, ny, nz) else 0
    # buffers of the phase-by-phase step: the same C-ABI calls the composite
    # step makes, issued separately so that each phase is timed on the stream
    buf = {"mesh": torch.empty(ncell, dtype=torch.float32, device=dev),
           "mfws": torch.empty(mf_bytes, dtype=torch.uint8, device=dev),
           "f3": torch.empty(3 * ncell, dtype=torch.float32, device=dev),
           "det": torch.empty(ncell * 8 if mode == _lib.PAINT_DETERMINISTIC else 1,
                              dtype=torch.uint8, device=dev),
           "perm": torch.empty((2, Np if engine == "sorted" else 1), dtype=torch.int32,
                               device=dev)}
    perms = buf["perm"]
    perm_cur = [0]
    P = lambda name: _lib.ptr(buf[name])  # noqa: E731
    det_bytes = ncell * 8 if mode == _lib.PAINT_DETERMINISTIC else 0

    # the sorted run loop takes the forces from the potential where the
    # spectral pipeline serves the mesh (pmgb_fpm_run_sorted_f32); the phase
    # pass issues the same kernels
    use_pot = engine == "sorted" and fft_path != 0
    if engine == "sorted":
        eng = simulate.SortedFastPM((n,) * 3, cosmo, 0.1, 1.0, K, device=dev)
        kick, drift = eng.kick, eng.drift
        phase_names = ["paint", "forces", "read_kick_drift", "sort"]
    else:
        eng = simulate.FastPM((n,) * 3, cosmo, 0.1, 1.0, K, paint_mode=mode, device=dev)
        kick, drift = eng.kick, eng.drift
        x, v = x0.clone(), v0.clone()
        phase_names = ["paint", "forces", "read_kick_drift"]
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(len(phase_names) + 1)]
              for _ in range(K)]

    # sorted loop: every step's gather also paints the next step's density
    # (pmgb_read3_kick_drift_paint_binned_f32), so only the first step of a
    # run has a paint phase
    density_ready = [False]
    permuted = [False]  # the engine's particles are read through buf["perm"]

    def reset():
        density_ready[0] = False
        permuted[0] = False
        if engine == "sorted":
            eng.load(x0, v0)
        else:
            x.copy_(x0)
            v.copy_(v0)

    def current_positions():
        return eng.positions if engine == "sorted" else x

    def step_phased(i, ev=None):
        rec = (lambda j: ev[j].record(stream)) if ev is not None else (lambda j: None)
        if engine == "sorted":
            a, b = eng.cur, 1 - eng.cur
            px, pv = eng.pos[a], eng.vel[a]
        else:
            px, pv = x, v
        rec(0)
        if engine == "sorted":
            if not density_ready[0]:
                _lib.call("pmgb_cic_paint_sorted_f32", P("mesh"), nx, ny, nz, _lib.ptr(px), Np,
                          _lib.ptr(eng.sort_ws), eng.sort_bytes, _lib.ptr(eng.stats_buf), s)
        else:
            _lib.call("pmgb_cic_paint_f32", P("mesh"), nx, ny, nz, _lib.ptr(px), Np, None, 1.0,
                      mode, 0, P("det"), det_bytes, s)
        rec(1)
        if use_pot:
            # density -> potential (the run loop's one inverse transform)
            _lib.call("pmgb_mesh_potential_f32", P("mesh"), P("f3"), nx, ny, nz, 0.0, P("mfws"),
                      mf_bytes, s)
        else:
            # density -> three force meshes (fused FFT pipeline, or cuFFT)
            _lib.call("pmgb_mesh_forces_f32", P("mesh"), P("f3"), nx, ny, nz, 0.0, P("mfws"),
                      mf_bytes, s)
        rec(2)
        if engine == "sorted" and use_pot:
            # the run loop's permuted gather: slot p is read from index perm[p]
            # (in place, without perm, on the first step after a sort) and
            # written to index p of the other buffer, with its new tile key
            last = i + 1 == K
            out = a if not permuted[0] else b
            pc = perm_cur[0]
            _lib.call("pmgb_read_potential_kick_drift_paint_perm_f32", P("f3"), nx, ny, nz,
                      _lib.ptr(px), _lib.ptr(pv), _lib.ptr(perms[pc]) if permuted[0] else None,
                      _lib.ptr(eng.pos[out]), _lib.ptr(eng.vel[out]), Np, float(kick[i]),
                      float(drift[i]), None if last else P("mesh"), _lib.ptr(eng.sort_ws),
                      eng.sort_bytes, _lib.ptr(eng.stats_buf), s)
            density_ready[0] = not last
            rec(3)
            if last:  # the ids follow the gather, then the run's one full sort
                if permuted[0]:
                    _lib.call("pmgb_gather_u32", _lib.ptr(eng.ids[a]), _lib.ptr(perms[pc]), Np,
                              _lib.ptr(eng.ids[out]), s)
                _lib.call("pmgb_tile_scatter_f32", _lib.ptr(eng.pos[out]),
                          _lib.ptr(eng.vel[out]), _lib.ptr(eng.ids[out]), Np, nx, ny, nz,
                          _lib.ptr(eng.pos[1 - out]), _lib.ptr(eng.vel[1 - out]),
                          _lib.ptr(eng.ids[1 - out]), None, _lib.ptr(eng.sort_ws),
                          eng.sort_bytes, s)
                eng.cur = 1 - out
                permuted[0] = False
            else:  # the re-sort of the permutation (the ids follow it)
                _lib.call("pmgb_tile_resort_index", Np, nx, ny, nz,
                          _lib.ptr(perms[pc]) if permuted[0] else None, _lib.ptr(perms[1 - pc]),
                          _lib.ptr(eng.ids[a]), _lib.ptr(eng.ids[out]), _lib.ptr(eng.sort_ws),
                          eng.sort_bytes, s)
                perm_cur[0] = 1 - pc
                eng.cur = out
                permuted[0] = True
            rec(4)
        elif engine == "sorted":
            if i + 1 < K:  # gather + kick + drift + paint of the next density
                _lib.call("pmgb_read3_kick_drift_paint_binned_f32", P("f3"), ncell, nx, ny, nz,
                          _lib.ptr(px), _lib.ptr(pv), Np, float(kick[i]), float(drift[i]),
                          P("mesh"), _lib.ptr(eng.sort_ws), eng.sort_bytes,
                          _lib.ptr(eng.stats_buf), s)
            else:
                _lib.call("pmgb_read3_kick_drift_binned_f32", P("f3"), ncell, nx, ny, nz,
                          _lib.ptr(px), _lib.ptr(pv), Np, float(kick[i]), float(drift[i]),
                          _lib.ptr(eng.sort_ws), eng.sort_bytes, _lib.ptr(eng.stats_buf), s)
            density_ready[0] = i + 1 < K
            rec(3)
            _lib.call("pmgb_tile_scatter_f32", _lib.ptr(px), _lib.ptr(pv), _lib.ptr(eng.ids[a]),
                      Np, nx, ny, nz, _lib.ptr(eng.pos[b]), _lib.ptr(eng.vel[b]),
                      _lib.ptr(eng.ids[b]), None, _lib.ptr(eng.sort_ws), eng.sort_bytes, s)
            rec(4)
            eng.cur = b
        else:
            _lib.call("pmgb_read3_kick_drift_f32", P("f3"), ncell, nx, ny, nz, _lib.ptr(px),
                      _lib.ptr(pv), Np, float(kick[i]), float(drift[i]), None, s)
            rec(3)

    # warm-up on the initial state, then reset
    reset()
    for i in range(W):
        step_phased(i % K)
    reset()
    torch.cuda.synchronize(dev)
    # launch configuration of the run loop, tuned on this workload (untimed;
    # cached per mesh, particle count, step count and GPU)
    tuning = None
    if args.tuning is not None:
        fields = _lib.get_tuning()
        fields.update(json.loads(args.tuning))
        _lib.set_tuning(**fields)
        tuning = {"choice": fields, "set_by": "--tuning"}
    elif engine == "sorted" and "tune" not in skip:
        from jaxpm_gb300 import autotune
        choice, report = autotune.tune_run(eng, x0, v0, steps=K)
        tuning = {"choice": choice, "ms_per_step_by_candidate": report,
                  "default": autotune.DEFAULT}
        reset()
        torch.cuda.synchronize(dev)

    if engine == "sorted":
        eng.stats_buf.zero_()
        # the phase breakdown: the step's C-ABI calls one by one, with events
        # between them (serialised; the timed run below overlaps the sort
        # with the next force evaluation)
        for i in range(K):
            step_phased(i, events[i])
        torch.cuda.synchronize(dev)
        reset()
        eng.run(steps=min(W, K))  # warm-up of the run call itself
        reset()
        torch.cuda.synchronize(dev)

    R = max(1, args.repeats)
    clocks = ClockSampler(local) if "clocks" not in skip else None
    if clocks:
        clocks.start()
        time.sleep(0.3)

    in_run = []  # the run loop's own per-launch phase times of each timed run

    def timed_run():
        """One timed K-step run from the initial state: (ms, own launches)."""
        reset()
        torch.cuda.synchronize(dev)
        barrier(world)
        torch.cuda.synchronize(dev)
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        launches0 = lib.pmgb_launch_count()
        t0.record(stream)
        with nvtx("timed"):
            if engine == "sorted":
                eng.run()  # pmgb_fpm_run_sorted_f32: the K steps in one call
            else:
                for i in range(K):
                    step_phased(i, events[i])
        t1.record(stream)
        launches = lib.pmgb_launch_count() - launches0
        torch.cuda.synchronize(dev)
        if engine == "sorted":
            in_run.append(_lib.run_timing())
        barrier(world)
        return max_over_ranks(t0.elapsed_time(t1), world), launches

    if engine == "sorted":
        # CUDA events on the run loop's own streams around each gather, force
        # evaluation and re-sort of the timed runs (pmgb_set_run_timing)
        _lib.set_run_timing(True)
    try:
        runs = [timed_run() for _ in range(R)]
    finally:
        if engine == "sorted":
            _lib.set_run_timing(False)
    clk = clocks.stop() if clocks else None
    run_ms = [r[0] for r in runs]
    ms_max = float(np.median(run_ms))
    value = world * Np * K / (ms_max / 1e3)
    phase_ms = {name: float(np.mean([events[i][j].elapsed_time(events[i][j + 1])
                                     for i in range(K)])) for j, name in enumerate(phase_names)}

    # sanity: mass of the final density equals the particle count
    rho = painting.paint(torch.zeros((n,) * 3, device=dev), current_positions(),
                         mode="deterministic")
    mass_err = abs(rho.double().sum().item() - Np) / Np
    # P(k) of the final density (GPU R2C + binned |delta_k|^2): against the
    # oracle's run of the same workload (below) and the one-kernel-per-op path
    _, pk_run = utils.power_spectrum(rho, box_shape=[n * BOX_PER_CELL] * 3)
    del rho
    # own kernels launched in one timed run, counted by the library (cuFFT's
    # kernels are not counted)
    gpu_launches = int(runs[-1][1])

    result = {"metric": "particle-steps/s (FastPM PM step, 512^3 particles on 512^3 mesh)",
              "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": K,
              "warmup": W, "ms_per_step": ms_max / K, "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None, "dtype": "f32",
              "data": "synthetic: seeded Gaussian random field (NumPy PCG64 noise, "
                      "Eisenstein-Hu P(k)), 2LPT to a=0.1",
              "config": {"workload": f"FastPM {n}^3 particles on {n}^3 mesh, box {n} Mpc/h, "
                                     f"2LPT a=0.1, {K} steps to a=1",
                         "particles": Np, "mesh": [n, n, n], "box_mpc_h": n * BOX_PER_CELL,
                         "engine": engine, "fft": ["cufft", "fused", "own"][fft_path],
                         "forces": ("potential, order-1 gradient as a stencil in the gather"
                                    if use_pot else "three force meshes"),
                         "paint_mode": {0: "atomic", 1: "binned",
                                                          2: "deterministic"}[mode],
                         "parallelism": "replicas" if world > 1 else "single",
                         "l2": "inputs larger than L2 (positions+velocities 3.2 GB, "
                               "meshes 0.54 GB each)"},
              "repeats": {"n": R, "ms_per_step": [m / K for m in run_ms],
                          "median_ms_per_step": ms_max / K,
                          "spread": (max(run_ms) - min(run_ms)) / ms_max,
                          "note": "value is the median of the repeated K-step runs, each "
                                  "from the same initial state"},
              "phases_ms": phase_ms, "mass_rel_err": mass_err,
              "gpu_launches": gpu_launches}
    if tuning is not None:
        result["config"]["tuning"] = tuning["choice"]
        result["autotune"] = tuning
    if engine == "sorted":
        result["particles_outside_tile"] = eng.stats
        if eng.stats.get("tma_wait_timeout"):
            raise RuntimeError("a TMA wait of the gather timed out: the run is invalid")
    result["parity"] = parity_vs_oracle(n, K, pk_run, eng.state() if engine == "sorted"
                                        else (x, v))

    # roofline of the dominant own kernel
    peak, peak_kind = peaks()
    # algorithmic bytes per particle (Np = mesh cells): paint 12 read + 4
    # write; forces 4 read + 12 write + the half spectra in and out of each
    # of its three passes (4 + 4, 4 + 12, 12 + 12 at nz/2+1 of nz); gather
    # 12 force + 24 read + 24 write, + 4 for the sorted loop's paint of the
    # next density (its paint phase runs once per run, so it has no per-step
    # roofline)
    if use_pot:
        # the potential pipeline: plane R2C 4 + 4, x pass 4 + 4, plane C2R
        # 4 + 4.  The run loop's permuted gather: the potential 4, positions
        # and velocities 24 read through the permutation (4) and 24 written,
        # the (new tile key, stayer rank) pair 8, the next density 4.  The
        # re-sort: the pairs 8, the new permutation 4, the ids following the
        # old one 4 + 4 + 4.
        alg = {"forces": 24.0, "read_kick_drift": 68.0, "sort": 24.0}
    elif engine == "sorted":
        alg = {"forces": 48.0, "read_kick_drift": 64.0}
    else:
        alg = {"paint": 16.0, "forces": 48.0, "read_kick_drift": 60.0}
    # per-launch times: measured inside the timed runs where the run loop
    # records them, else from the phase pass
    launch_ms = dict(phase_ms)
    if in_run:
        for k in ("read_kick_drift", "forces", "sort"):
            launch_ms[k] = float(np.median([t[k] for t in in_run]))
        result["phases_in_timed_run_ms"] = {
            k: launch_ms[k] for k in ("read_kick_drift", "forces", "sort")}
        result["phases_in_timed_run_ms"]["how"] = (
            "mean per launch over each timed run (CUDA events the run loop records on the "
            "streams it launches on: gathers and force evaluations on the caller's stream, "
            "re-sorts on the second stream), median over the repeats")
    own = {k: launch_ms[k] for k in alg}
    dom = max(own, key=own.get)
    achieved = alg[dom] * Np / (launch_ms[dom] / 1e3) / 1e9
    tr = profile_traffic().get(dom)
    result["roofline"] = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak,
                          "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                          "algorithmic_bytes_per_particle": alg[dom],
                          "launch_ms": launch_ms[dom],
                          "launch_ms_from": ("the timed runs" if in_run else
                                             "the serialised phase pass"),
                          "traffic": (tr * Np if tr is not None else None)}
    result["kernels_frac_of_peak"] = {k: alg[k] * Np / (launch_ms[k] / 1e3) / 1e9 / peak
                                      for k in alg}
    # the same from the phase pass, each phase alone on the GPU
    result["kernels_frac_of_peak_alone"] = {
        k: alg[k] * Np / (phase_ms[k] / 1e3) / 1e9 / peak for k in alg}
    if args.phases_only:
        print(json.dumps(result))
        return

    def repeated(fn, reps):
        """Median and spread of `reps` timed calls of fn (CUDA events on the
        stream, max over ranks); fn(prepare=True) runs untimed first."""
        out = []
        for _ in range(reps):
            fn(True)
            torch.cuda.synchronize(dev)
            barrier(world)
            a0 = torch.cuda.Event(enable_timing=True)
            a1 = torch.cuda.Event(enable_timing=True)
            a0.record(stream)
            fn(False)
            a1.record(stream)
            torch.cuda.synchronize(dev)
            out.append(max_over_ranks(a0.elapsed_time(a1), world))
        med = float(np.median(out))
        return med, {"n": reps, "ms_per_step": [m / K for m in out],
                     "spread": (max(out) - min(out)) / med}

    # forward + adjoint (hand-written adjoint; positions stored before every
    # step, and for the sorted loop also its force meshes and re-sort map)
    if "adjoint" not in skip:
        gx = torch.ones_like(x0) * 1e-3
        gv = torch.zeros_like(v0)
        if engine == "sorted":
            store = eng.alloc_store()
        else:
            store = torch.empty((K, Np, 3), dtype=torch.float32, device=dev)
        eng.vjp(x0, v0, gx, gv, store=store)  # warm-up (plans, buffers)

        def adj(prepare):
            if not prepare:
                with nvtx("adjoint"):
                    eng.vjp(x0, v0, gx, gv, store=store)
        ams, rep = repeated(adj, R)
        result["fwd_adjoint"] = {"value": world * Np * K / (ams / 1e3),
                                 "unit": "particle-steps/s", "ms_per_step": ams / K,
                                 "cost_vs_forward": ams / ms_max, "repeats": rep}
        del store

    # one-kernel-per-op GPU form
    if "plain" not in skip:
        plain = simulate.FastPM((n,) * 3, cosmo, 0.1, 1.0, K, plain=True, device=dev)
        xp, vp = x0.clone(), v0.clone()
        plain.step(xp, vp, 0)

        def plain_run(prepare):
            if prepare:
                xp.copy_(x0)
                vp.copy_(v0)
            else:
                plain.run(xp, vp)
        pms, rep = repeated(plain_run, R)
        result["plain_gpu"] = {"value": world * Np * K / (pms / 1e3), "unit": "particle-steps/s",
                               "ms_per_step": pms / K, "fused_speedup": pms / ms_max,
                               "repeats": rep}
        # the two GPU forms from the same state: final P(k) of the
        # one-kernel-per-op path (atomic paint, three force meshes through
        # cuFFT, separate gather / kick / drift) against the timed run's
        rho_p = painting.paint(torch.zeros((n,) * 3, device=dev), xp, mode="deterministic")
        _, pk_plain = utils.power_spectrum(rho_p, box_shape=[n * BOX_PER_CELL] * 3)
        del rho_p
        rel = np.abs(pk_run / pk_plain - 1.0)
        rel = rel[np.isfinite(rel)]
        result["plain_gpu"]["pk_vs_timed_run"] = {
            "max_rel_dev_per_bin": float(rel.max()), "bins": int(rel.size)}
        result["plain_gpu"]["parity"] = parity_vs_oracle(n, K, pk_plain, None)
        del plain, xp, vp

    # end to end with the state in pinned host memory (SortedFastPM.run_host):
    # every step copies positions and velocities (caller's order) up in
    # E2E_CHUNKS pieces, paints each piece as it lands, evaluates the forces,
    # gathers + kicks + drifts each piece and copies it back as soon as it is
    # done; piece c of step i+1 goes up as soon as piece c of step i is down
    if "e2e" not in skip:
        hx = x0.cpu().pin_memory()
        hv = v0.cpu().pin_memory()
        E = eng if engine == "sorted" else simulate.SortedFastPM((n,) * 3, cosmo, 0.1, 1.0, K,
                                                                device=dev)

        def e2e(prepare):
            if prepare:  # the caller's state back to the initial one (untimed)
                hx.copy_(x0.cpu())
                hv.copy_(v0.cpu())
            else:
                E.run_host(hx, hv, steps=K, chunks=E2E_CHUNKS)
        # warm-up (untimed): the first call allocates the streamed schedule's
        # mesh, force meshes and workspaces
        for _ in range(max(1, min(W, 2))):
            e2e(True)
            E.run_host(hx, hv, steps=1, chunks=E2E_CHUNKS)
        ems, rep = repeated(e2e, R)
        nbytes = 2 * Np * 12
        # the state that came back: its P(k) against the timed run's
        rho_e = painting.paint(torch.zeros((n,) * 3, device=dev), hx.to(dev),
                               mode="deterministic")
        _, pk_e2e = utils.power_spectrum(rho_e, box_shape=[n * BOX_PER_CELL] * 3)
        del rho_e
        rel = np.abs(pk_e2e / pk_run - 1.0)
        rel = rel[np.isfinite(rel)]
        result["e2e"] = {"value": world * Np * K / (ems / 1e3), "unit": "particle-steps/s",
                         "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                         "ms_per_step": ems / K, "repeats": rep,
                         "api": "SortedFastPM.run_host: per step and piece "
                                "pmgb_cic_paint_f32 (binned, accumulating) as the piece "
                                "lands, pmgb_mesh_forces_f32, per piece "
                                "pmgb_read3_kick_drift_f32 then its copy down (C ABI); "
                                f"pinned host buffers, {E2E_CHUNKS} pieces on two copy "
                                "streams, piece c of the next step up as soon as piece c "
                                "of this one is down",
                         "pk_vs_timed_run": {"max_rel_dev_per_bin": float(rel.max()),
                                             "bins": int(rel.size)}}
        # the host link's own rates (copy engines, pinned memory, the same
        # buffers): the e2e leg's roofline is its bytes per step over the
        # two-direction rate
        link = link_rates(hx, hv, dev)
        moved = 2.0 * nbytes * K / (ems / 1e3) / 1e9
        result["e2e"]["link"] = dict(link, unit="GB/s",
                                     note="copy-engine rates of the pinned buffers: up alone, "
                                          "down alone, both directions at once")
        result["e2e"]["link_frac"] = {"achieved_gbs": moved, "peak_gbs": link["both"],
                                      "frac": moved / link["both"]}
        del hx, hv

    # paint / read microbenchmarks (16.7M uniform and clustered particles on
    # 256^3) and the paint-only case: the timed run's a=1 particles on 1024^3
    if "paint" not in skip and rank == 0 and n == 512:
        big = None
        if "1024" not in skip:
            reset()
            eng.run()
            big = (eng.state()[0] * 2.0).contiguous()  # cell units of the 1024^3 mesh
        torch.cuda.empty_cache()
        suite, _ = paint_read_suite(dev, max(W, 3), max(R, 5), big, skip)
        del big
        torch.cuda.empty_cache()
        result["paint_read"] = suite

    if clk is not None:
        result["clocks"] = clk

    if rank == 0 and "cpu" not in skip:
        result["cpu_baseline"] = cpu_baseline_sample(cosmo)
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def parity_vs_oracle(n, K, pk, state):
    """The final density's P(k) (and, with ``state`` = (pos, vel) in the
    caller's order, a fixed sample of particles) against the oracle's
    float32 and float64 runs of the same workload (``tests/golden/
    large_<n>_<K>.npz``, made by ``tests/golden/make_large_golden.py``),
    when a fixture exists for this mesh and step count."""
    path = os.path.join(ROOT, "tests", "golden", f"large_{n}_{K}.npz")
    if not os.path.exists(path):
        return {"fixture": None, "note": f"no oracle fixture for {n}^3 and {K} steps"}
    d = np.load(path)
    out = {"fixture": os.path.relpath(path, ROOT), "tolerance_per_bin": 1e-3}
    for tag in ("32", "64"):
        rel = np.abs(pk / d[f"pk1_{tag}"] - 1.0)
        out[f"pk_vs_oracle_f{tag}"] = {"max_rel_dev_per_bin": float(rel.max()),
                                       "bins": int(rel.size)}
    out["oracle_f32_vs_f64"] = float(np.abs(d["pk1_32"] / d["pk1_64"] - 1.0).max())
    out["within"] = bool(out["pk_vs_oracle_f32"]["max_rel_dev_per_bin"] < 1e-3)
    if state is not None:
        import torch
        idx = torch.from_numpy(d["sample"]).to(state[0].device)
        x = state[0][idx].double().cpu().numpy()
        v = state[1][idx].double().cpu().numpy()
        i = d["sample"].astype(np.int64)
        lat = np.stack([i // (n * n), (i // n) % n, i % n], -1)
        for tag in ("32", "64"):
            dx = x - d[f"x1_{tag}"]
            dx -= n * np.round(dx / n)
            out[f"displacement_vs_oracle_f{tag}"] = float(
                np.linalg.norm(dx) / np.linalg.norm(d[f"x1_{tag}"] - lat))
            out[f"velocity_vs_oracle_f{tag}"] = float(
                np.linalg.norm(v - d[f"v1_{tag}"]) / np.linalg.norm(d[f"v1_{tag}"]))
    return out


# ---------------------------------------------------------------------------
# batched workload: 64 independent simulations of 64^3, 96^3 or 128^3
# ---------------------------------------------------------------------------
BATCH_SIMS = 64
BATCH_MESHES = (64, 96, 128)


def batched_table(seed):
    """Mesh sizes, Omega_c ~ U[0.2, 0.35] and sigma8 ~ U[0.6, 1.0] of the
    64 simulations (NumPy PCG64 with `seed`); box 2N Mpc/h."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ns = [int(n) for n in rng.choice(BATCH_MESHES, size=BATCH_SIMS)]
    return ns, rng.uniform(0.2, 0.35, BATCH_SIMS), rng.uniform(0.6, 1.0, BATCH_SIMS)


def run_batched(args):
    import torch
    from jaxpm_gb300 import batched, cosmology

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    skip = set(filter(None, args.skip.split(",")))
    K, W = args.steps, args.warmup
    # replicas: every rank runs its own 64 simulations (seeds offset by rank)
    ns, ocs, s8s = batched_table(seed=rank)
    shapes = [(n,) * 3 for n in ns]
    cosmos = [cosmology.Planck15(Omega_c=float(a), sigma8=float(b)) for a, b in zip(ocs, s8s)]
    x0, v0 = batched.initial_conditions(shapes, [[2.0 * n] * 3 for n in ns], cosmos,
                                        [BATCH_SIMS * rank + i for i in range(BATCH_SIMS)],
                                        device=dev)
    eng = batched.BatchedFastPM(shapes, cosmos, 0.1, 1.0, K, device=dev)
    Np = eng.n
    stream = torch.cuda.current_stream(dev)
    x, v = x0.clone(), v0.clone()
    for i in range(W):
        eng.step(x, v, i % K)
    launches0 = batched._lib.load().pmgb_launch_count()
    graph = eng.capture(x, v)  # the K steps as one CUDA graph
    # own kernels recorded in the graph (the warm-up step of capture() included)
    graph_launches = batched._lib.load().pmgb_launch_count() - launches0
    x.copy_(x0)
    v.copy_(v0)
    graph.replay()  # warm-up of the graph itself
    x.copy_(x0)
    v.copy_(v0)
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local) if "clocks" not in skip else None
    if clocks:
        clocks.start()
        time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize(dev)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    with nvtx("timed"):
        graph.replay()
    t1.record(stream)
    torch.cuda.synchronize(dev)
    barrier(world)
    clk = clocks.stop() if clocks else None
    ms = max_over_ranks(t0.elapsed_time(t1), world)
    value = world * Np * K / (ms / 1e3)
    masses = [float(m.double().sum()) for m in eng.paint(x)]
    mass_err = max(abs(m - c) / c for m, c in zip(masses, eng.counts))
    peak, peak_kind = peaks()
    achieved = 124.0 * Np / (ms / K / 1e3) / 1e9
    counts = {n: ns.count(n) for n in BATCH_MESHES}
    result = {"metric": "particle-steps/s (batched FastPM: 64 simulations of 64^3-128^3)",
              "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": K,
              "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
              "vs_baseline": None, "dtype": "f32", "impl": "gb300",
              "data": "synthetic: per simulation a seeded Gaussian random field (NumPy PCG64 "
                      "noise, Eisenstein-Hu P(k)), 2LPT to a=0.1",
              "config": {"workload": f"64 independent FastPM simulations, N in {{64, 96, 128}} "
                                     f"({counts[64]} x 64^3, {counts[96]} x 96^3, "
                                     f"{counts[128]} x 128^3), particles = cells, box 2N Mpc/h, "
                                     f"Omega_c ~ U[0.2,0.35], sigma8 ~ U[0.6,1.0], own seeds, "
                                     f"{K} steps a=0.1 -> 1, the run captured as one CUDA graph",
                         "particles": Np, "parallelism": "replicas" if world > 1 else "single",
                         "l2": f"inputs larger than L2 (positions+velocities "
                               f"{Np * 24 / 1e9:.1f} GB)"},
              "mass_rel_err": mass_err,
              # own kernels of one replay (the K steps; the FFTs are cuFFT's):
              # the library's count at capture minus capture()'s warm-up step
              "gpu_launches": int(graph_launches * K // (K + 1)),
              "roofline": {"kernel": "whole step", "bound": "hbm", "achieved": achieved,
                           "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                           "peak_kind": peak_kind, "algorithmic_bytes_per_particle": 124.0,
                           "traffic": None}}
    if "adjoint" not in skip:
        store = eng.alloc_store()
        gx = torch.ones_like(x0) * 1e-3
        gv = torch.zeros_like(v0)
        eng.vjp(x0, v0, gx, gv, store=store)
        torch.cuda.synchronize(dev)
        barrier(world)
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        with nvtx("adjoint"):
            eng.vjp(x0, v0, gx, gv, store=store)
        a1.record(stream)
        torch.cuda.synchronize(dev)
        ams = max_over_ranks(a0.elapsed_time(a1), world)
        result["fwd_adjoint"] = {"value": world * Np * K / (ams / 1e3),
                                 "unit": "particle-steps/s", "ms_per_step": ams / K,
                                 "cost_vs_forward": ams / ms}
        del store
    # end to end with host buffers (BatchedFastPM.run_host): the simulations
    # go through the host link in E2E_GROUPS groups, each group's upload,
    # step and read-back chained, the groups overlapping one another
    if "e2e" not in skip:
        hx, hv = x0.cpu().pin_memory(), v0.cpu().pin_memory()
        # warm-up (untimed): the first call makes the groups' tables and FFT plans
        eng.run_host(hx, hv, steps=1, groups=E2E_GROUPS)
        hx.copy_(x0.cpu())
        hv.copy_(v0.cpu())
        torch.cuda.synchronize(dev)
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.run_host(hx, hv, steps=K, groups=E2E_GROUPS)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ems = max_over_ranks(e0.elapsed_time(e1), world)
        # the state that came back against the timed run's final state
        dx_ = hx.to(dev)
        disp_dev = float(((dx_ - x).double().norm() / (x - x0).double().norm()).item())
        del dx_
        result["e2e"] = {"value": world * Np * K / (ems / 1e3), "unit": "particle-steps/s",
                         "h2d_bytes_per_step": 2 * Np * 12, "d2h_bytes_per_step": 2 * Np * 12,
                         "ms_per_step": ems / K,
                         "api": "BatchedFastPM.run_host: pmgb_fpm_step_batched_f32 (C ABI) "
                                f"per group of simulations, {E2E_GROUPS} groups of about "
                                "equal particle counts, each group's copy up, step and copy "
                                "down chained on three streams, the groups overlapping",
                         "final_displacement_rel_dev_vs_timed_run": disp_dev}
    if clk is not None:
        result["clocks"] = clk
    if rank == 0 and "cpu" not in skip:
        result["cpu_baseline"] = cpu_batched_sample(ns, ocs, s8s, K)
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def cpu_batched_sample(ns, ocs, s8s, K):
    """One oracle FastPM step of the table's first 64^3 simulation."""
    from oracle import cic, cosmology as oc, nbody as onb
    i = ns.index(64) if 64 in ns else 0
    n = ns[i]
    c = oc.Cosmology(Omega_c=float(ocs[i]), sigma8=float(s8s[i]))
    k = np.logspace(-4, 1, 128)
    noise = np.random.Generator(np.random.PCG64(i)).standard_normal((n,) * 3, dtype=np.float32)
    ic = onb.linear_field(noise, [2.0 * n] * 3, k, oc.linear_matter_power(c, k))
    lat = cic.lattice((n,) * 3).reshape(-1, 3).astype(np.float32)
    dx, p, _ = onb.lpt(c, ic, lat, a=0.1, order=2)
    kc, dc = onb.fpm_coefficients(c, 0.1, 1.0, K)
    t = time.perf_counter()
    onb.fpm_step(lat + dx, p, (n,) * 3, kc[0], dc[0])
    dt = time.perf_counter() - t
    return {"value": n**3 / dt, "unit": "particle-steps/s", "cores": host_threads(),
            "kind": "port",
            "sample": f"one FastPM step of the NumPy oracle on one {n}^3 simulation of the table "
                      f"({dt:.2f} s)"}


# ---------------------------------------------------------------------------
# paint / read microbenchmarks
# ---------------------------------------------------------------------------
def paint_read_suite(dev, W, K, big=None, skip=()):
    """The cic_paint / cic_read microbenchmarks on 16,777,216 particles on a
    256^3 mesh: (i) uniform U[0,256)^3 positions (PCG64 seed 1) and (ii) the
    a = 1 positions of the 256^3 run (2LPT to a = 0.1, 20 steps), in the
    caller's (lattice) order; each painter (atomic, binned, sort + box) and
    the one- and three-component reads, median of K launches after W
    warm-up launches, with the fraction of the measured HBM peak.  With
    ``big`` (positions in cell units of a 1024^3 mesh) also the paint-only
    case on 1024^3.  Returns ``(results, launches)``."""
    import torch
    from jaxpm_gb300 import _lib, cosmology, simulate

    lib = _lib.load()
    stream = torch.cuda.current_stream(dev)
    s = _lib.stream(dev)
    peak, _ = peaks()
    n = 256
    Np = n**3
    cosmo = cosmology.Planck15()
    uni = torch.from_numpy(np.random.Generator(np.random.PCG64(1)).uniform(
        0.0, n, (Np, 3)).astype(np.float32)).to(dev)
    x0, v0 = initial_state(n, cosmo, dev)
    sim = simulate.SortedFastPM((n,) * 3, cosmo, 0.1, 1.0, 20, device=dev)
    sim.load(x0, v0)
    sim.run()
    clustered = sim.state()[0].contiguous()
    del sim, x0, v0

    launches = {}

    def timed(fn, tag=None):
        for _ in range(W):
            fn()
        l0 = lib.pmgb_launch_count()
        ts = []
        for _ in range(K):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize(dev)
            ts.append(a.elapsed_time(b))
        if tag is not None:
            launches[tag] = (lib.pmgb_launch_count() - l0) // K
        return float(np.median(ts))

    def paint_ops(pos, shape, tag):
        nx, ny, nz = shape
        npart = pos.shape[0]
        mesh = torch.empty(shape, dtype=torch.float32, device=dev)
        ops = {}
        for name, mode in [("atomic", _lib.PAINT_ATOMIC), ("binned", _lib.PAINT_BINNED)]:
            wsb = lib.pmgb_cic_paint_workspace_size(nx, ny, nz, npart, mode)
            ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=dev)
            ops[name] = (lambda m=mode, w=ws, b=wsb: _lib.call(
                "pmgb_cic_paint_f32", _lib.ptr(mesh), nx, ny, nz, _lib.ptr(pos), npart, None,
                1.0, m, 0, _lib.ptr(w), b, s))
        # sort by tile, then the shared-memory box paint
        sb = lib.pmgb_tile_sort_workspace_size(nx, ny, nz, npart)
        sws = torch.empty(sb, dtype=torch.uint8, device=dev)
        spos = torch.empty_like(pos)
        sid = torch.empty(npart, dtype=torch.int32, device=dev)

        def sorted_paint():
            _lib.call("pmgb_tile_sort_f32", _lib.ptr(pos), None, None, npart, nx, ny, nz,
                      _lib.ptr(spos), None, _lib.ptr(sid), _lib.ptr(sws), sb, s)
            _lib.call("pmgb_cic_paint_sorted_f32", _lib.ptr(mesh), nx, ny, nz, _lib.ptr(spos),
                      npart, _lib.ptr(sws), sb, None, s)
        ops["sort+box"] = sorted_paint
        alg = 12.0 * npart + 4.0 * nx * ny * nz
        out = {}
        for name, fn in ops.items():
            with nvtx(f"paint_{tag}_{name}"):
                ms = timed(fn, f"paint_{tag}_{name}")
            total = float(mesh.double().sum())
            out[name] = {"ms": ms, "particles_per_s": npart / (ms / 1e3),
                         "achieved_gbs": alg / (ms / 1e3) / 1e9,
                         "frac": alg / (ms / 1e3) / 1e9 / peak,
                         "mass_rel_err": abs(total - npart) / npart}
        del mesh, sws, spos, sid
        best = max(out, key=lambda k: out[k]["particles_per_s"])
        out["best"] = best
        return out

    def read_ops(pos, shape, tag):
        nx, ny, nz = shape
        npart = pos.shape[0]
        g = torch.Generator(device=dev).manual_seed(3)
        mesh3 = torch.rand((3,) + tuple(shape), generator=g, device=dev)
        out1 = torch.empty(npart, dtype=torch.float32, device=dev)
        out3 = torch.empty((npart, 3), dtype=torch.float32, device=dev)
        ncell = nx * ny * nz
        res = {}
        with nvtx(f"read_{tag}"):
            ms = timed(lambda: _lib.call("pmgb_cic_read_f32", _lib.ptr(mesh3), nx, ny, nz,
                                         _lib.ptr(pos), npart, _lib.ptr(out1), s),
                       f"read_{tag}")
        alg = 16.0 * npart + 4.0 * ncell  # positions + output + the mesh once
        res["read"] = {"ms": ms, "particles_per_s": npart / (ms / 1e3),
                       "achieved_gbs": alg / (ms / 1e3) / 1e9,
                       "frac": alg / (ms / 1e3) / 1e9 / peak}
        with nvtx(f"read3_{tag}"):
            ms = timed(lambda: _lib.call("pmgb_cic_read3_f32", _lib.ptr(mesh3), ncell, nx, ny,
                                         nz, _lib.ptr(pos), npart, _lib.ptr(out3), s),
                       f"read3_{tag}")
        alg = 24.0 * npart + 12.0 * ncell
        res["read3"] = {"ms": ms, "particles_per_s": npart / (ms / 1e3),
                        "achieved_gbs": alg / (ms / 1e3) / 1e9,
                        "frac": alg / (ms / 1e3) / 1e9 / peak}
        del mesh3, out1, out3
        return res

    # the L2-resident mesh makes these kernels L2-bound, not HBM-bound: the
    # library's rates of random atomics and random gathers on a buffer of the
    # mesh's size (torch's index_add_ / index_select, uniform random indices,
    # as many as the CIC paint's contributions), against which each paint and
    # read reports its rate of CIC contributions as a ratio (not a ceiling:
    # the paint pairs z-neighbours into one vector reduction)
    cells = n**3
    m = 8 * Np
    gidx = torch.randint(0, cells, (m,), device=dev,
                         generator=torch.Generator(device=dev).manual_seed(5))
    ones = torch.ones(m, dtype=torch.float32, device=dev)
    buf = torch.zeros(cells, dtype=torch.float32, device=dev)
    t_add = timed(lambda: buf.index_add_(0, gidx, ones))
    t_get = timed(lambda: torch.index_select(buf, 0, gidx))
    del gidx, ones, buf
    l2 = {"atomic_adds_per_s": m / (t_add / 1e3), "gathers_per_s": m / (t_get / 1e3),
          "buffer_bytes": 4 * cells,
          "how": "torch index_add_ / index_select of 8 x 16,777,216 uniform random "
                 "indices into a float32 buffer of the 256^3 mesh's size"}

    results = {"l2_reference": l2}
    for dname, pos in [("uniform", uni), ("clustered_a1", clustered)]:
        results[dname] = {"paint": paint_ops(pos, (n,) * 3, dname),
                          "read": read_ops(pos, (n,) * 3, dname)}
        # each CIC contribution is one atomic (paint) or one load (read)
        for name, r in results[dname]["paint"].items():
            if isinstance(r, dict):
                r["x_library_atomics"] = 8 * Np / (r["ms"] / 1e3) / l2["atomic_adds_per_s"]
        rd = results[dname]["read"]
        rd["read"]["x_library_gathers"] = 8 * Np / (rd["read"]["ms"] / 1e3) / l2["gathers_per_s"]
        rd["read3"]["x_library_gathers"] = (24 * Np / (rd["read3"]["ms"] / 1e3)
                                             / l2["gathers_per_s"])
    del uni, clustered
    if big is not None and "1024" not in skip:
        torch.cuda.empty_cache()
        results["paint_only_1024"] = paint_ops(big, (1024,) * 3, "1024")
        torch.cuda.empty_cache()
    results["accounting"] = ("paint 12 B/particle read + 4 B/cell written; read 12 B/particle "
                             "positions + 4 B/particle out + the mesh once; read3 12 + 12 B/"
                             "particle + three meshes once; frac: of the measured HBM copy "
                             "bandwidth; x_library_*: 8 CIC contributions per particle (24 "
                             "for read3) per second over l2_reference's random-index rates")
    return results, launches


def run_paint(args):
    import torch
    from jaxpm_gb300 import cosmology, simulate

    rank, world, local = dist_env()
    if rank != 0:
        return
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    skip = set(filter(None, args.skip.split(",")))
    K, W = max(args.steps, 5), max(args.warmup, 3)
    peak, peak_kind = peaks()
    big = None
    if "1024" not in skip:
        # paint-only: the 512^3 run's a=1 particles on a 1024^3 mesh
        cosmo = cosmology.Planck15()
        x5, v5 = initial_state(512, cosmo, dev)
        sim = simulate.SortedFastPM((512,) * 3, cosmo, 0.1, 1.0, 40, device=dev)
        sim.load(x5, v5)
        del x5, v5
        sim.run()
        big = (sim.state()[0] * 2.0).contiguous()  # cell units of the 1024^3 mesh
        del sim
        torch.cuda.empty_cache()
    results, launches = paint_read_suite(dev, W, K, big, skip)
    del big
    head = results["clustered_a1"]["paint"]
    best = head["best"]
    result = {"metric": "particles/s (cic_paint, 16.7M clustered a=1 particles on 256^3 mesh)",
              "value": head[best]["particles_per_s"], "unit": "particles/s", "n_gpus": 1,
              "steps": K, "warmup": W, "ms_per_step": head[best]["ms"],
              "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
              "impl": "gb300",
              "data": "synthetic: (i) uniform U[0,256)^3 positions, NumPy PCG64 seed 1; (ii) "
                      "a=1 positions of the 256^3 run (2LPT a=0.1 + 20 FastPM steps) in "
                      "lattice order",
              "config": {"workload": "cic_paint / cic_read microbenchmarks: 16,777,216 "
                                     "particles on a 256^3 mesh, uniform and clustered; "
                                     "paint-only of the 512^3 run's a=1 particles on 1024^3",
                         "paint_path": best,
                         "l2": "positions (201 MB) larger than L2; median of K launches"},
              "results": results,
              "roofline": {"kernel": f"paint ({best})", "bound": "hbm",
                           "achieved": head[best]["achieved_gbs"], "peak": peak, "unit": "GB/s",
                           "frac": head[best]["frac"], "peak_kind": peak_kind,
                           "algorithmic_bytes_per_particle": 16.0, "traffic": None},
              "gpu_launches": int(launches[f"paint_clustered_a1_{best}"])}
    print(json.dumps(result))


# ---------------------------------------------------------------------------
# gradient workload: d loss / d (noise, Omega_c, sigma8) through LPT + FastPM
# ---------------------------------------------------------------------------
def grad_case(n, steps, checkpoint_every, dev, fd_eps=1e-3, engine="sorted"):
    """Forward model at n^3 (box 2n Mpc/h, 2LPT a=0.1, `steps` steps to a=1,
    a checkpoint every `checkpoint_every` steps, the steps on `engine`), MSE
    of the a=1 density against the seed-2 target; times forward and
    forward+backward and checks the gradients against central differences
    (eps = fd_eps)."""
    import torch
    from jaxpm_gb300 import _lib, distributed, forward_model as fm, painting

    shape, box = (n,) * 3, (2.0 * n,) * 3
    theta0 = torch.tensor([0.2589, 0.8159], dtype=torch.float64)
    noise = distributed.normal_field(1, shape, device=dev)
    with torch.no_grad():
        xt, _ = fm.lpt_nbody(distributed.normal_field(2, shape, device=dev), theta0, shape, box,
                             n_steps=steps, checkpoint_every=0)
        target = painting.cic_paint(torch.zeros(shape, device=dev), xt)
        del xt

    def loss(nz, th):
        x, _ = fm.lpt_nbody(nz, th, shape, box, n_steps=steps, checkpoint_every=checkpoint_every,
                            engine=engine)
        return fm.density_mse(x, target)

    from jaxpm_gb300 import growth
    stream = torch.cuda.current_stream(dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    # warm-up forward and backward (FFT plans, k-space tables), then drop the
    # host growth tables so that the timed pass pays the host scalar work of
    # a new cosmology
    nzw = noise.clone().requires_grad_(True)
    thw = theta0.clone().requires_grad_(True)
    loss(nzw, thw).backward()
    del nzw, thw
    growth._CACHE.clear()
    torch.cuda.synchronize(dev)
    a, b = ev(), ev()
    a.record(stream)
    with torch.no_grad():
        loss0 = loss(noise, theta0)
    b.record(stream)
    torch.cuda.synchronize(dev)
    fwd_ms = a.elapsed_time(b)
    nz = noise.clone().requires_grad_(True)
    th = theta0.clone().requires_grad_(True)
    growth._CACHE.clear()
    torch.cuda.synchronize(dev)
    lib = _lib.load()
    l0 = lib.pmgb_launch_count()
    a, b = ev(), ev()
    a.record(stream)
    loss(nz, th).backward()
    b.record(stream)
    torch.cuda.synchronize(dev)
    grad_ms = a.elapsed_time(b)
    launches = lib.pmgb_launch_count() - l0
    d = torch.randn(shape, generator=torch.Generator(device=dev).manual_seed(5), device=dev)
    checks = {}
    with torch.no_grad():
        for j, name in enumerate(["Omega_c", "sigma8"]):
            tp, tm = theta0.clone(), theta0.clone()
            tp[j] += fd_eps
            tm[j] -= fd_eps
            fd = (float(loss(noise, tp)) - float(loss(noise, tm))) / (2 * fd_eps)
            an = float(th.grad[j])
            checks[name] = {"adjoint": an, "finite_difference": fd,
                            "rel_err": abs(an - fd) / max(abs(fd), 1e-30)}
        fd = (float(loss(noise + fd_eps * d, theta0)) -
              float(loss(noise - fd_eps * d, theta0))) / (2 * fd_eps)
        an = float((nz.grad.double() * d.double()).sum())
        checks["noise_direction"] = {"adjoint": an, "finite_difference": fd,
                                     "rel_err": abs(an - fd) / max(abs(fd), 1e-30)}
    return {"mesh": n, "steps": steps, "checkpoint_every": checkpoint_every, "engine": engine,
            "loss": float(loss0), "forward_ms": fwd_ms, "forward_backward_ms": grad_ms,
            "backward_vs_forward": (grad_ms - fwd_ms) / fwd_ms, "gpu_launches": int(launches),
            "grad_check_eps": fd_eps, "grad_check": checks}


def run_grad(args):
    import torch

    rank, world, local = dist_env()
    if rank != 0:
        return
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    skip = set(filter(None, args.skip.split(",")))
    K = args.steps if args.steps_given else 32
    clocks = ClockSampler(local) if "clocks" not in skip else None
    if clocks:
        clocks.start()
    main = grad_case(128, K, 4, dev, engine=args.engine)
    clk = clocks.stop() if clocks else None
    Np = 128**3
    value = Np * K / (main["forward_backward_ms"] / 1e3)
    result = {"metric": "particle-steps/s (forward+gradient: 2LPT + FastPM, 128^3, d loss / "
                        "d (noise, Omega_c, sigma8))",
              "value": value, "unit": "particle-steps/s", "n_gpus": 1, "steps": K, "warmup": 1,
              "ms_per_step": main["forward_backward_ms"] / K, "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "gb300",
              "data": "synthetic: NumPy PCG64 white noise seeds 1 (model) and 2 (target), "
                      "Eisenstein-Hu P(k)",
              "config": {"workload": f"MSE between the a=1 CIC density of 128^3 particles on a "
                                     f"128^3 mesh (box 256 Mpc/h, 2LPT a=0.1, {K} steps, "
                                     f"checkpoints every 4) and a seed-2 target; gradient w.r.t. "
                                     f"the white noise and (Omega_c, sigma8)",
                         "engine": args.engine,
                         "l2": "one timed pass; working set above L2 at 512^3"},
              "cases": [main],
              "gpu_launches": main["gpu_launches"]}
    # the other engine on the same 128^3 case, for comparison
    other = "lattice" if args.engine == "sorted" else "sorted"
    result["cases"].append(grad_case(128, K, 4, dev, engine=other))
    if "512" not in skip:
        result["cases"].append(grad_case(512, 64, 4, dev, engine=args.engine))
    if clk is not None:
        result["clocks"] = clk
    print(json.dumps(result))


# ---------------------------------------------------------------------------
# CPU: the oracle (NumPy restatement of the reference's algorithm)
# ---------------------------------------------------------------------------
def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def oracle_state(n, seed=0):
    from oracle import cic, cosmology as oc, nbody as onb
    cosmo = oc.Cosmology()
    k = np.logspace(-4, 1, 128)
    pk = oc.linear_matter_power(cosmo, k)
    noise = np.random.Generator(np.random.PCG64(seed)).standard_normal((n,) * 3,
                                                                        dtype=np.float32)
    ic = onb.linear_field(noise, [n * BOX_PER_CELL] * 3, k, pk)
    lat = cic.lattice((n,) * 3).reshape(-1, 3).astype(np.float32)
    dx, p, _ = onb.lpt(cosmo, ic, lat, a=0.1, order=2)
    return cosmo, lat + dx, p


def oracle_threads():
    """Host threads the oracle's step uses: its C paint/read (OpenMP) and
    scipy.fft (all workers)."""
    from oracle import native
    return max(native.threads(), host_threads()) if native.lib() is not None else \
        host_threads()


def oracle_kind():
    from oracle import native
    return ("C paint/read (OpenMP) + scipy.fft" if native.lib() is not None
            else "NumPy paint/read + scipy.fft")


def cpu_baseline_sample(cosmo_unused=None, n=256):
    """One oracle FastPM step (paint, C2C FFTs, k-space, three reads, kick,
    drift) on a 256^3 sub-problem, timed on the host cores."""
    from oracle import nbody as onb
    cosmo, x, v = oracle_state(n)
    kc, dc = onb.fpm_coefficients(cosmo, 0.1, 1.0, 20)
    t = time.perf_counter()
    onb.fpm_step(x, v, (n,) * 3, kc[0], dc[0])
    dt = time.perf_counter() - t
    return {"value": n**3 / dt, "unit": "particle-steps/s", "cores": oracle_threads(),
            "kind": "port",
            "sample": f"one FastPM step of the oracle on a {n}^3-particle/{n}^3-mesh sub-problem "
                      f"of the workload ({dt:.1f} s; {oracle_kind()}, all host threads)"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    if args.workload == "batched":
        return run_reference_batched(args)
    if args.workload == "paint":
        return run_reference_paint(args)
    if args.workload == "grad":
        return run_reference_grad(args)
    # the same workload as the GPU arm: n^3 particles on an n^3 mesh, 2LPT to
    # a = 0.1, K steps to a = 1 (one oracle step at 512^3 takes seconds on
    # the host cores, so the warm-up is one step)
    n = args.mesh
    K, W = args.steps, args.warmup
    w_run = min(W, 1)
    from oracle import nbody as onb
    cosmo, x0, v0 = oracle_state(n)
    kc, dc = onb.fpm_coefficients(cosmo, 0.1, 1.0, K)
    x, v = x0, v0
    for i in range(w_run):
        x, v = onb.fpm_step(x, v, (n,) * 3, kc[i % K], dc[i % K])
    x, v = x0, v0
    t = time.perf_counter()
    for i in range(K):
        x, v = onb.fpm_step(x, v, (n,) * 3, kc[i], dc[i])
    dt = time.perf_counter() - t
    value = n**3 * K / dt
    out = {"metric": "particle-steps/s (FastPM PM step, 512^3 particles on 512^3 mesh)",
           "value": value, "unit": "particle-steps/s", "n_gpus": 0, "steps": K,
           "warmup": w_run, "ms_per_step": dt / K * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
           "data": "synthetic: seeded Gaussian random field (NumPy PCG64 noise, Eisenstein-Hu "
                   "P(k)), 2LPT to a=0.1",
           "config": {"workload": f"FastPM {n}^3 particles on {n}^3 mesh, box {n} Mpc/h, "
                                  f"2LPT a=0.1, {K} steps to a=1",
                      "particles": n**3, "mesh": [n] * 3, "box_mpc_h": float(n)},
           "cpu_baseline": {"value": value, "unit": "particle-steps/s",
                            "cores": oracle_threads(), "kind": "port",
                            "sample": f"every step of the {n}^3 workload, {K} steps timed "
                                      f"after {w_run} warm-up step(s): the oracle (the "
                                      f"reference's algorithm restated: {oracle_kind()}; JAX "
                                      f"is not installed)"},
           "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_reference_batched(args):
    """The oracle on the host cores: each timed step is one FastPM step of
    one 64^3 simulation of the batch table (a bounded sample of the 64)."""
    from oracle import cic, cosmology as oc, nbody as onb
    K, W = args.steps, args.warmup
    ns, ocs, s8s = batched_table(seed=0)
    i = ns.index(64) if 64 in ns else 0
    n = ns[i]
    c = oc.Cosmology(Omega_c=float(ocs[i]), sigma8=float(s8s[i]))
    k = np.logspace(-4, 1, 128)
    noise = np.random.Generator(np.random.PCG64(i)).standard_normal((n,) * 3, dtype=np.float32)
    ic = onb.linear_field(noise, [2.0 * n] * 3, k, oc.linear_matter_power(c, k))
    lat = cic.lattice((n,) * 3).reshape(-1, 3).astype(np.float32)
    dx, p, _ = onb.lpt(c, ic, lat, a=0.1, order=2)
    kc, dc = onb.fpm_coefficients(c, 0.1, 1.0, K)
    x, v = lat + dx, p
    for j in range(W):
        onb.fpm_step(x, v, (n,) * 3, kc[j % K], dc[j % K])
    t = time.perf_counter()
    for j in range(K):
        x, v = onb.fpm_step(x, v, (n,) * 3, kc[j], dc[j])
    dt = time.perf_counter() - t
    value = n**3 * K / dt
    out = {"metric": "particle-steps/s (batched FastPM: 64 simulations of 64^3-128^3)",
           "value": value, "unit": "particle-steps/s", "n_gpus": 0, "steps": K, "warmup": W,
           "ms_per_step": dt / K * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "impl": "reference",
           "data": "synthetic: seeded Gaussian random field, 2LPT to a=0.1",
           "config": {"workload": "64 independent FastPM simulations, N in {64, 96, 128}, box "
                                  "2N Mpc/h"},
           "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": host_threads(),
                            "kind": "port",
                            "sample": f"each timed step is one FastPM step of the NumPy oracle "
                                      f"on one {n}^3 simulation of the table"},
           "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_reference_paint(args):
    """The oracle's cic_paint (np.bincount scatter) on the host: each timed
    step paints a 2M-particle sample of the uniform distribution."""
    from oracle import cic
    K, W = args.steps, args.warmup
    n, m = 256, 1 << 21
    pos = np.random.Generator(np.random.PCG64(1)).uniform(0.0, n, (m, 3)).astype(np.float32)
    for _ in range(min(W, 1)):
        cic.cic_paint(np.zeros((n,) * 3, np.float32), pos)
    t = time.perf_counter()
    steps = min(K, 5)
    for _ in range(steps):
        cic.cic_paint(np.zeros((n,) * 3, np.float32), pos)
    dt = time.perf_counter() - t
    value = m * steps / dt
    out = {"metric": "particles/s (cic_paint, 16.7M clustered a=1 particles on 256^3 mesh)",
           "value": value, "unit": "particles/s", "n_gpus": 0, "steps": steps, "warmup": W,
           "ms_per_step": dt / steps * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "impl": "reference",
           "data": "synthetic: uniform U[0,256)^3 positions, NumPy PCG64 seed 1",
           "config": {"workload": "cic_paint of 2,097,152 particles on a 256^3 mesh"},
           "cpu_baseline": {"value": value, "unit": "particles/s", "cores": 1, "kind": "port",
                            "sample": "each timed step is the NumPy oracle's cic_paint of a "
                                      "2,097,152-particle uniform sample (single-threaded "
                                      "bincount)"},
           "e2e": {"value": value, "unit": "particles/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_reference_grad(args):
    """The oracle on the host: forward FastPM steps and their reverse sweep
    (float64 NumPy) on a 32^3 sample of the 128^3 problem."""
    from oracle import nbody as onb
    K = args.steps if args.steps_given else 32
    n = 32
    cosmo, x0, v0 = oracle_state(n)
    kc, dc = onb.fpm_coefficients(cosmo, 0.1, 1.0, K)
    rng = np.random.default_rng(0)
    gx, gv = rng.standard_normal(x0.shape), rng.standard_normal(x0.shape)
    t = time.perf_counter()
    onb.fpm_run_vjp(x0, v0, (n,) * 3, kc, dc, gx, gv)
    dt = time.perf_counter() - t
    value = n**3 * K / dt
    out = {"metric": "particle-steps/s (forward+gradient: 2LPT + FastPM, 128^3, d loss / "
                     "d (noise, Omega_c, sigma8))",
           "value": value, "unit": "particle-steps/s", "n_gpus": 0, "steps": K, "warmup": 0,
           "ms_per_step": dt / K * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "impl": "reference",
           "data": "synthetic: seeded Gaussian random field, 2LPT to a=0.1",
           "config": {"workload": f"forward FastPM run and its reverse sweep, {K} steps"},
           "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": host_threads(),
                            "kind": "port",
                            "sample": f"the NumPy oracle's forward run + reverse sweep of {K} "
                                      f"FastPM steps on a {n}^3 sub-problem (float64)"},
           "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    args = parse()
    args.steps_given = args.steps is not None
    if args.steps is None:
        args.steps = 40 if args.workload == "step" else 20
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "paint":
        run_paint(args)
    elif args.workload == "grad":
        run_grad(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
