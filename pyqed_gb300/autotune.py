"""Project-written autotuner for the propagator's schedule and tuning options.

The library picks a schedule by rule (instances that fit one CTA run on the
CTA-resident / tensor-core kernels, larger ones on the grid-wide GEMM
schedule) and exposes tuning options (``lgb_plan_set_option``: two
instances per CTA on the tensor cores for NP <= 32; for the GEMM schedule
the RK4 steps per captured CUDA graph, and for its split precisions one or
two waves of split-K CTAs and a cap on the split-K factor).  ``tune`` times every
valid candidate on the caller's own operators for a few RK4 steps (CUDA
events, after one untimed run) and returns the fastest; results are cached
per problem signature and GPU in a JSON file (``$PYQED_GB300_TUNE_CACHE``,
default ``~/.cache/pyqed_gb300/tune.json``).  Tuning never changes what is
computed beyond the precision's tolerance, only how it is scheduled (see
``candidates`` for the one schedule kept out for that reason).
"""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

__all__ = ["candidates", "signature", "tune", "cache_path"]

# the GEMM schedule handles instances one after another; beyond this many it
# is never a contender and is not timed
_GEMM_MAX_INST = 16


def cache_path():
    return os.environ.get("PYQED_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "pyqed_gb300", "tune.json"))


def signature(dims, n_cops, cops_kind, n_eops, n_drive, precision, device_name):
    """Stable key of a problem shape (the multiset of dimensions, operator
    counts and kinds, precision, GPU name)."""
    d = np.sort(np.asarray(dims, dtype=np.int64))
    key = dict(dims=hashlib.sha256(d.tobytes()).hexdigest()[:16], n_inst=int(d.size),
               n_cops=int(n_cops), cops_kind=str(cops_kind), n_eops=int(n_eops),
               n_drive=int(n_drive), precision=str(precision), device=str(device_name))
    return json.dumps(key, sort_keys=True)


def candidates(dims, precision, cops_kind, n_cops, n_drive=0):
    """Configurations worth timing for this problem shape.

    Every candidate computes the same result to the precision's tolerance.
    The 3xBF16 GEMM schedule keeps the diagonal of A inside the BF16 split
    products, which the tensor-core CTA kernel applies in FP32 (that term
    carries most of the BF16 error on Hamiltonians with order-one site
    energies), so for 3xBF16 the GEMM schedule is only a candidate when some
    instance does not fit the tensor-core kernel.
    """
    dims = np.asarray(dims)
    split = precision in ("3xtf32", "3xbf16")
    dense = cops_kind == "dense" and n_cops > 0
    out = [dict(schedule="auto", options={})]
    if split and not dense and np.any(dims <= 32):
        out.append(dict(schedule="auto", options={"tc_pairs": 0}))
    fits_tc = not dense and bool(np.all((dims <= 64) | ((dims == 65) & (n_drive == 0))))
    if precision == "3xbf16" and fits_tc:
        return out
    if dims.size <= _GEMM_MAX_INST:
        # the GEMM schedule: steps per captured CUDA graph, and for the split
        # precisions the split-K shape (waves of CTAs, a cap on the factor).
        # Split-precision static instances with 64 < N <= 256 run on the
        # persistent kernel by default, which these options do not shape: the
        # graph-replayed variants are timed with it switched off.
        persist = split and n_drive == 0 and bool(np.any((dims > 64) & (dims <= 256)))
        off = {"gemm_persist": 0} if persist else {}
        if persist:
            out.append(dict(schedule="gemm", options={}))
        for gs in (16, 32):
            base = dict(off) if gs == 16 else dict(off, graph_steps=gs)
            out.append(dict(schedule="gemm", options=dict(base)))
            if split:
                out.append(dict(schedule="gemm", options=dict(base, gemm_waves=2)))
                for cap in (4, 8):
                    out.append(dict(schedule="gemm", options=dict(base, gemm_ksplit=cap)))
    return out


def _load_cache(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store_cache(path, cache):
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def _time_candidate(cand, make_prop, operators, rho0, drive, reps):
    import torch
    from . import _capi as C
    try:
        prop = make_prop(cand)
    except C.LindbladError as e:
        if e.status == 2:  # LGB_ERR_UNSUPPORTED: not a valid schedule for this problem
            return None
        raise
    try:
        for k, v in cand["options"].items():
            prop.set_option(k, v)
        prop.set_operators(*operators)
        r0 = prop.to_device(rho0)
        d = torch.from_numpy(np.ascontiguousarray(drive).ravel()).to(prop.device) if drive is not None else None
        out = prop.alloc_outputs(want_obs=True, want_rho=False)
        prop.propagate_device(r0, d, out)
        torch.cuda.synchronize(prop.device)
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            prop.propagate_device(r0, d, out)
            e1.record()
            torch.cuda.synchronize(prop.device)
            t = e0.elapsed_time(e1)
            best = t if best is None else min(best, t)
        prop.check_errors()
        return best
    finally:
        prop.close()


def tune(bi, *, dt, precision, obs_t0=False, drive=None, drive_shared=True, device=None,
         nt_probe=6, reps=2, use_cache=True, timer=None):
    """Best (schedule, options) for the prepared batch ``bi``
    (``pyqed_gb300.batch.prepare_batch``).

    Returns dict(schedule, options, timings_ms, cached).  ``timer`` replaces
    the GPU timing (callable(candidate) -> milliseconds or None), for tests.
    """
    dev_name = "cpu"
    if timer is None:
        import torch
        dev = torch.device(device if device is not None else "cuda")
        dev_name = torch.cuda.get_device_name(dev)
    key = signature(bi.dims, bi.n_cops, bi.cops_kind, bi.n_eops, bi.n_drive, precision, dev_name)
    path = cache_path()
    cache = _load_cache(path) if use_cache else {}
    if key in cache:
        hit = dict(cache[key])
        hit["cached"] = True
        return hit
    cands = candidates(bi.dims, precision, bi.cops_kind, bi.n_cops, bi.n_drive)
    if timer is None:
        from .engine import Propagator

        def probe_steps(c):
            # GEMM candidates run two captured graphs' worth of steps, so that
            # the graph length is part of what is timed
            return max(nt_probe, 2 * c["options"].get("graph_steps", 16)) if c["schedule"] == "gemm" else nt_probe

        def make_prop(c):
            return Propagator(bi.dims, nt=probe_steps(c), dt=dt, n_cops=bi.n_cops, cops_kind=bi.cops_kind,
                              n_eops=bi.n_eops, n_drive=bi.n_drive, obs_t0=obs_t0,
                              precision=precision, schedule=c["schedule"], drive_shared=drive_shared,
                              device=device)

        def drive_for(nsteps):
            if not bi.n_drive:
                return None
            d = np.asarray(drive, dtype=np.float64)
            return d[..., :nsteps] if d.shape[-1] >= nsteps else \
                np.pad(d, [(0, 0)] * (d.ndim - 1) + [(0, nsteps - d.shape[-1])])
        ops = (bi.H, bi.cops, bi.eops, bi.dops)

        def timer(c):  # noqa: F811
            ms = _time_candidate(c, make_prop, ops, bi.rho0, drive_for(probe_steps(c)), reps)
            # per probe step, so that candidates with different probe lengths compare
            return None if ms is None else ms / probe_steps(c)
    timings = []
    for c in cands:
        t = timer(c)
        if t is not None:
            timings.append((t, c))
    if not timings:
        raise RuntimeError("no valid schedule for this problem")
    t_best, best = min(timings, key=lambda x: x[0])
    res = dict(schedule=best["schedule"], options=dict(best["options"]),
               timings_ms=[dict(schedule=c["schedule"], options=c["options"], ms=t) for t, c in timings],
               cached=False)
    if use_cache:
        cache[key] = {k: v for k, v in res.items() if k != "cached"}
        _store_cache(path, cache)
    return res
