"""Autotuner of the tile-sorted run loop's launch choices.

The fastest schedule of the gather depends on how clustered the particles
are and how far they move per step: a schedule that deals most tiles to the
CTAs statically keeps the particles leaving their tiles spread over the mesh
(their global reductions then collide less), while a dynamic one absorbs the
uneven particle counts of late, clustered steps.  ``tune_run`` times the
candidates on the caller's own workload (an engine with its state loaded,
run over all its steps once per candidate) and keeps the fastest; results
are cached in a JSON file keyed by mesh, particle count, step count, GPU
and library version, so a workload is tuned once per machine.

The knobs (``pmgb_set_tuning``): the quarters of the tiles the gather deals
statically (0-4), and the CTAs per SM of the gather and of the re-sort (0:
as many as fit).  The reference has no counterpart: XLA picks the launch
shapes of its scatter and gather (``jaxpm/painting.py:43-44``, ``:104-106``).
"""
import itertools
import json
import os
import threading

import torch

from . import _lib

DEFAULT = {"gather_static_quarters": 3, "gather_ctas_per_sm": 0, "resort_ctas_per_sm": 0,
           "resort_priority": 0}

# Measured at 512^3 (40 steps) before narrowing: a fourth static quarter and
# 3 gather CTAs per SM were never faster (0.5 ms per step slower); 1-4
# re-sort CTAs per SM leave it latency-bound (6.3-8.3 ms per step against
# 6.27 with a full wave), 5-7 let the force evaluation run beside it (6.19
# at 6); the default stream priority for the re-sort was no faster there
# (6.27-6.32) but stays a candidate.
CANDIDATES = {"gather_static_quarters": (2, 3), "gather_ctas_per_sm": (0,),
              "resort_ctas_per_sm": (0, 5, 6, 7), "resort_priority": (0, 1)}

_LOCK = threading.Lock()


def cache_path():
    """The cache file: $PMGB_TUNE_CACHE, else ~/.cache/jaxpm_gb300/tuning.json."""
    return os.environ.get("PMGB_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "jaxpm_gb300",
                                       "tuning.json"))


def _key(eng, steps):
    dev = eng.ws.device
    name = torch.cuda.get_device_name(dev)
    return (f"{'x'.join(str(v) for v in eng.mesh_shape)}|np={eng.n}|steps={steps}|{name}|"
            f"abi={_lib.load().pmgb_version()}")


def _read_cache(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _write_cache(path, data):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def candidates():
    names = list(CANDIDATES)
    for values in itertools.product(*(CANDIDATES[n] for n in names)):
        yield dict(zip(names, values))


def _time_run(eng, pos, vel, steps, repeats):
    """Milliseconds of eng.run over `steps` steps from (pos, vel): the best
    of `repeats` runs after one warm-up run."""
    stream = torch.cuda.current_stream(eng.ws.device)
    best = float("inf")
    for r in range(repeats + 1):
        eng.load(pos, vel)
        torch.cuda.synchronize(eng.ws.device)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.run(steps=steps, check=False)
        b.record(stream)
        torch.cuda.synchronize(eng.ws.device)
        eng.check()
        if r > 0:
            best = min(best, a.elapsed_time(b))
    return best


def tune_run(eng, pos, vel, steps=None, repeats=1, use_cache=True, apply=True):
    """Tunes the run loop of ``eng`` (a ``simulate.SortedFastPM``) on the
    state ``(pos, vel)`` (caller's order; reloaded before every trial, so the
    engine's own state is replaced).  Returns ``(choice, report)``: the
    fastest candidate and, per candidate, its time in ms per step (empty
    when the choice came from the cache).  With ``apply`` the choice is set
    for the process (``pmgb_set_tuning``)."""
    steps = eng.n_steps if steps is None else int(steps)
    path = cache_path()
    key = _key(eng, steps)
    with _LOCK:
        if use_cache:
            hit = _read_cache(path).get(key)
            if hit is not None:
                if apply:
                    _lib.set_tuning(**hit)
                return hit, {}
        previous = _lib.get_tuning()
        report = {}
        try:
            for cand in candidates():
                _lib.set_tuning(**cand)
                ms = _time_run(eng, pos, vel, steps, repeats)
                report[json.dumps(cand, sort_keys=True)] = ms / steps
        finally:
            _lib.set_tuning(**previous)
        best = min(report, key=report.get)
        choice = json.loads(best)
        if use_cache:
            data = _read_cache(path)
            data[key] = choice
            _write_cache(path, data)
        if apply:
            _lib.set_tuning(**choice)
        return choice, report
