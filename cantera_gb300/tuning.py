"""Empirical launch-shape autotuner of the batched integrator.

The engine's automatic launch shape is a rule (Newton matrices in shared memory while a block
of 8 reactors fits, otherwise in an L2-resident global slot per warp).  ``autotune`` measures
instead: it advances a strided sample of the caller's reactors with each candidate shape
(matrix placement x reactors per block) and returns the options of the fastest, so that the
choice follows the mechanism size and the GPU.  Each candidate's sample is a whole number of
waves of its own resident capacity (blocks x reactors per block), and candidates are compared
by time per reactor: a sample of a fixed size would favour the shape whose capacity happens
to divide it well (the tail of a partial wave dominates a short run).  Within ``margin`` of
the fastest, the shape with more resident reactors wins (more latency hiding on the long
runs the tuner stands in for).  Results are cached per (mechanism, options) in the process
and persisted in a JSON file keyed by the mechanism's content, the GPU and the options
(``GBCHEM_TUNING_CACHE`` names the file; default ``~/.cache/cantera_gb300/launch_shapes.json``;
an empty value turns the file off), so a later process on the same kind of GPU skips the
measurement.
"""
import hashlib
import json
import os
import time

from . import ReactorNet

_cache = {}


def cache_path():
    p = os.environ.get("GBCHEM_TUNING_CACHE")
    if p is None:
        p = os.path.join(os.path.expanduser("~"), ".cache", "cantera_gb300", "launch_shapes.json")
    return p or None


def mechanism_key(solution):
    """Content hash of the mechanism: its file, phase and structure counts (which also cover
    species and reactions drawn from other files)."""
    h = hashlib.sha256()
    path, phase = getattr(solution, "source", ("", ""))
    try:
        with open(path, "rb") as f:
            h.update(f.read())
    except OSError:
        h.update(path.encode())
    h.update(phase.encode())
    h.update(json.dumps(solution.structure(), sort_keys=True).encode())
    return h.hexdigest()[:24]


def gpu_key():
    try:
        import torch
        d = torch.cuda.current_device()
        p = torch.cuda.get_device_properties(d)
        return "%s|sm%d%d|%dSM" % (p.name, p.major, p.minor, p.multi_processor_count)
    except Exception:
        return "unknown-gpu"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, key, value):
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        data = _load(path)
        data[key] = value
        tmp = "%s.%d.tmp" % (path, os.getpid())
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def candidates(max_warps=8):
    for placement in (1, 2):
        for wpb in (2, 4, 6, max_warps):
            yield {"matrix_placement": placement, "warps_per_block": wpb}


def _subset(T, P, Y, idx_stride, count):
    Ts, Ps, Ys = T[::idx_stride][:count], P[::idx_stride][:count], Y[:, ::idx_stride][:, :count]
    if hasattr(Ys, "contiguous"):
        return Ts.contiguous(), Ps.contiguous(), Ys.contiguous()
    import numpy as np
    return np.ascontiguousarray(Ts), np.ascontiguousarray(Ps), np.ascontiguousarray(Ys)


def autotune(solution, T, P, Y, t_probe, waves=3, pool=8192, rtol=1e-8, atol=1e-15, lu_precision=64,
             repeat=1, margin=0.03, use_cache=True, linear_solver="DENSE"):
    """Options dict (matrix_placement, warps_per_block) of the fastest launch shape for
    advancing these reactors (host or device arrays; Y species-major [K, n]) to t_probe with
    the given linear solver ("DENSE" or "GMRES", the Krylov path).  Each candidate advances
    `waves` full waves of its resident capacity, drawn with a stride from the caller's
    reactors (at most `pool` of them).  Also returns every candidate's timing (seconds per
    reactor)."""
    linear_solver = str(linear_solver).upper()
    key = (solution._h, lu_precision, waves, pool, float(t_probe), rtol, atol, linear_solver)
    if use_cache and key in _cache:
        return _cache[key]
    path = cache_path() if use_cache else None
    pkey = "|".join([mechanism_key(solution), gpu_key(), "lu%d" % lu_precision, "w%d" % waves, "p%d" % pool,
                     "t%.6g" % t_probe, "r%.3g" % rtol, "a%.3g" % atol]
                    + ([] if linear_solver == "DENSE" else [linear_solver]))
    if path:
        hit = _load(path).get(pkey)
        if hit:
            result = (dict(hit["pick"]), hit["log"])
            _cache[key] = result
            return result
    n = T.shape[0]
    npool = min(n, pool)
    Tp, Pp, Yp = _subset(T, P, Y, max(1, n // npool), npool)
    timings = []
    seen = set()
    for c in candidates():
        probe = ReactorNet(solution, Tp, Pp, Yp, rtol=rtol, atol=atol, lu_precision=lu_precision,
                           linear_solver=linear_solver, **c)
        info = probe.launch_info
        del probe
        shape = tuple(sorted(info.items()))
        if shape in seen:          # the engine capped this request to a shape already timed
            continue
        seen.add(shape)
        m = min(npool, waves * info["blocks"] * info["warps_per_block"])
        Ts, Ps, Ys = _subset(Tp, Pp, Yp, max(1, npool // m), m)
        net = ReactorNet(solution, Ts, Ps, Ys, rtol=rtol, atol=atol, lu_precision=lu_precision,
                         linear_solver=linear_solver, **c)
        net.advance(t_probe)       # warm-up (module load, first launch)
        best = float("inf")
        for _ in range(repeat):
            net.set_state(Ts, Ps, Ys)
            t0 = time.perf_counter()
            net.advance(t_probe)
            best = min(best, time.perf_counter() - t0)
        timings.append((best / m, c, dict(shape)))
        del net
    timings.sort(key=lambda x: x[0])
    fastest = timings[0][0]
    near = [t for t in timings if t[0] <= fastest * (1 + margin)]
    pick = max(near, key=lambda t: t[2]["blocks"] * t[2]["warps_per_block"])
    result = (dict(pick[1]), [{"seconds": t, "options": c, "shape": s} for t, c, s in timings])
    _cache[key] = result
    if path:
        _store(path, pkey, {"pick": result[0], "log": result[1], "measured": time.strftime("%Y-%m-%d %H:%M:%S")})
    return result
