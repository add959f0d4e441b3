"""Benchmark: Lindblad RK4 instance-steps/s on one GB300.

Default workload ``exciton4096``: 4096 Frenkel-exciton aggregates with
N = n + 1, n ~ U{8..64}, pure dephasing (diagonal collapse operators),
rho(0) = mu rho_g, dt = 0.05, 4000 RK4 steps, output C(t) = Tr[mu rho(t)]
for every instance and step (the reference's ``correlation_2op_1t``,
``pyqed/oqs.py:717-791``, over a batch).  One bench step = one full
propagation of the batch (4096 x 4000 instance-steps).

  python bench.py [--gpus 1] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload exciton4096|driven256|jc16] [--n-inst N] [--nt T]

Prints one JSON line.  ``value`` is the chosen path (``--precision``, by
default 3xBF16 with the diagonal of A applied in FP32) with inputs resident in
HBM (device-timed with CUDA events on the launch stream, L2 flushed between
steps); ``e2e`` times the public batched API including the host->device copy
of every input from pinned memory and the device->host read of C(t).
``plain`` is the FP32 CUDA-core path on the same inputs, ``alternatives``
the 3xTF32 path; ``accuracy`` checks each against the complex128 oracle;
``cpu_baseline`` is the oracle port of the reference's dense algorithm on the
host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Lindblad RK4 instance-steps/s: chosen vs plain on GB300 at |drho|<=1e-5; bwd/fwd"
UNIT = "instance-steps/s"


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def make_workload(name, n_inst=None, nt=None, shard=None):
    """The bench workloads.  ``shard=(rank, world)`` keeps this rank's share of
    the instances (``pyqed_gb300.shard.partition``: greedy balance of N^3);
    ``desc`` still describes the whole job."""
    from pyqed_gb300 import workloads as W
    from pyqed_gb300.batch import prepare_batch
    from pyqed_gb300.shard import shard_indices
    if name == "exciton4096":
        n_inst = n_inst or 4096
        idx = None if shard is None else shard_indices(W.exciton_dims(n_inst=n_inst), *shard)
        ex = W.exciton_batch(n_inst=n_inst, indices=idx)
        nt = nt or ex["nt"]
        cops = [[np.diag(c) for c in cd] for cd in ex["c_diag"]]
        seeds = [m @ r for m, r in zip(ex["mu"], ex["rho_g"])]
        bi = prepare_batch(ex["H"], cops, seeds, [[m] for m in ex["mu"]])
        desc = dict(workload=name, n_inst=n_inst, nt=nt, dt=ex["dt"],
                    N_range=[int(bi.dims.min()), int(bi.dims.max())],
                    collapse_ops="diagonal (n dephasing projectors)",
                    output="C(t)=Tr[mu rho(t)], (n_inst, nt) complex")
        flops = int(64 * np.sum(bi.dims.astype(np.int64) ** 3))
        return dict(bi=bi, nt=nt, dt=ex["dt"], obs_t0=False, drive=None, desc=desc,
                    flops_per_step=flops, ex=ex, n_total=n_inst)
    if name == "driven256":
        n_inst = n_inst or 256
        d = W.driven_batch(n_inst=n_inst, nt=nt or 2000)
        nt = d["nt"]
        sel = list(range(n_inst)) if shard is None else [int(b) for b in shard_indices(np.full(n_inst, 64), *shard)]
        cops = [[np.sqrt(d["gamma"][b][k]) * d["L"][b][k] for k in range(2)] for b in sel]
        bi = prepare_batch([d["H0"][b] for b in sel], cops, [d["rho0"][b] for b in sel],
                           [[d["O"][b]] for b in sel], drive_ops=[[d["mu"][b]] for b in sel])
        desc = dict(workload=name, n_inst=n_inst, nt=nt, dt=d["dt"], N=64, K=2,
                    drive="H(t)=H0-E(t)mu, shared GP pulse")
        flops = int(64 * 3 * np.sum(bi.dims.astype(np.int64) ** 3))
        return dict(bi=bi, nt=nt, dt=d["dt"], obs_t0=False, drive=d["E"][None, :].copy(),
                    desc=desc, flops_per_step=flops, n_total=n_inst)
    if name == "jc16":
        jc = W.jaynes_cummings()
        nt = nt or jc["nt"]
        bi = prepare_batch([jc["H"]], [jc["c_ops"]], [jc["rho0"]], [jc["e_ops"]])
        desc = dict(workload=name, n_inst=1, nt=nt, dt=jc["dt"], N=16, K=2)
        # one instance: every rank runs a replica
        return dict(bi=bi, nt=nt, dt=jc["dt"], obs_t0=True, drive=None, desc=desc,
                    flops_per_step=int(64 * 3 * 16 ** 3),
                    n_total=1 if shard is None else shard[1])
    raise SystemExit("unknown workload %s" % name)


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return dict(sm_mhz=None, sm_max_mhz=None, reasons=["nvidia-smi unavailable"])
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return dict(sm_mhz=float(np.median(sm)) if sm else None, sm_max_mhz=smax,
                    samples=len(sm), reasons=sorted(reasons))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def measure_tf32_peak(dev, n=8192, reps=5):
    """Dense TF32 tensor-core rate on this GPU: cuBLAS FP32 GEMM with TF32
    math (torch.matmul, 2 n^3 flops), best of ``reps``, TFLOP/s."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        a = torch.randn(n, n, device=dev)
        b = torch.randn(n, n, device=dev)
        c = a @ b
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1) / 1e3
            best = t if best is None else min(best, t)
        del a, b, c
        return 2.0 * n ** 3 / best / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def dist_context():
    """One rank per GPU under torchrun (WORLD_SIZE > 1): the NCCL process group
    serves only the barriers and the max-over-ranks of the timings; the
    instances shard with no exchange on the data path."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return dict(rank=rank, world=world, local=local)


def _max_over_ranks(ctx, values, dev):
    """Element-wise max over ranks of a list of floats (identity on one GPU)."""
    if ctx is None:
        return list(values)
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(values), dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.cpu().tolist()


def _barrier(ctx):
    if ctx is not None:
        import torch.distributed as dist
        dist.barrier()


def run_gpu(args, ctx=None):
    import torch
    from pyqed_gb300.build import build
    from pyqed_gb300.engine import Propagator
    build()
    dev = torch.device("cuda", 0 if ctx is None else ctx["local"])
    torch.cuda.set_device(dev)
    world = 1 if ctx is None else ctx["world"]
    rank0 = ctx is None or ctx["rank"] == 0
    wl = make_workload(args.workload, args.n_inst, args.nt,
                       shard=None if ctx is None else (ctx["rank"], world))
    bi, nt, dt = wl["bi"], wl["nt"], wl["dt"]
    n_inst = int(bi.dims.size)        # this rank's instances
    n_total = int(wl.get("n_total", n_inst))  # the whole job's
    chosen = args.precision
    paths = [chosen] + ([] if args.no_plain or chosen == "fp32" or ctx is not None else ["fp32"])
    if chosen == "3xbf16" and not args.no_plain and ctx is None:
        paths.append("3xtf32")  # the other split precision, timed and checked beside it
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    drive_shared = wl["drive"] is None or wl["drive"].ndim == 2

    def new_prop(prec):
        return Propagator(bi.dims, nt=nt, dt=dt, n_cops=bi.n_cops, cops_kind=bi.cops_kind,
                          n_eops=bi.n_eops, n_drive=bi.n_drive, obs_t0=wl["obs_t0"],
                          precision=prec, drive_shared=drive_shared, device=dev)

    results = {}
    rho0_dev = None
    drive_dev = torch.from_numpy(wl["drive"].ravel()).to(dev) if wl["drive"] is not None else None
    for prec in paths:
        prop = new_prop(prec)
        prop.set_operators(bi.H, bi.cops, bi.eops, bi.dops)
        rho0_dev = prop.to_device(bi.rho0)
        out = prop.alloc_outputs(want_obs=True, want_rho=True)
        stream = torch.cuda.current_stream(dev)
        for _ in range(args.warmup):
            prop.propagate_device(rho0_dev, drive_dev, out)
        torch.cuda.synchronize()
        prop.check_errors()
        clocks = ClockSampler(dev.index)
        if prec == chosen:
            clocks.start()
        times = []
        t_wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1.0)  # evict L2 between timed steps (untimed)
            torch.cuda.synchronize()
            _barrier(ctx)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            prop.propagate_device(rho0_dev, drive_dev, out)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        wall = time.perf_counter() - t_wall0
        times = _max_over_ranks(ctx, times, dev)
        clk = clocks.stop() if prec == chosen else None
        prop.check_errors()
        info = prop.info()
        t = float(np.mean(times))
        results[prec] = dict(sec_per_step=t, times=times, wall=wall, info=info, clocks=clk,
                             obs=prop.unpack_obs(out[0]) if out[0] is not None else None,
                             rho=out[1].cpu().numpy(), off=prop.off)
        prop.close()

    # ---- end to end through the public batched API (host buffers) ---------------
    prop = new_prop(chosen)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory() if a is not None else None  # noqa: E731
    host = [pin(x) for x in (bi.H, bi.cops, bi.eops, bi.dops, bi.rho0)]
    host_drive = pin(wl["drive"].ravel()) if wl["drive"] is not None else None
    out = prop.alloc_outputs(want_obs=True, want_rho=False)
    obs_host = torch.empty(out[0].numel(), dtype=torch.complex128).pin_memory()
    h2d = sum(x.numel() * x.element_size() for x in host if x is not None)
    h2d += host_drive.numel() * 8 if host_drive is not None else 0
    d2h = obs_host.numel() * obs_host.element_size()
    stream = torch.cuda.current_stream(dev)

    def e2e_step():
        dv = [x.to(dev, non_blocking=True) if x is not None else None for x in host]
        drv = host_drive.to(dev, non_blocking=True) if host_drive is not None else None
        prop.set_operators(dv[0], dv[1], dv[2], dv[3])
        prop.propagate_device(dv[4], drv, out)
        obs_host.copy_(out[0], non_blocking=True)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    e2e_times = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        _barrier(ctx)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        e2e_step()
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_times.append(e0.elapsed_time(e1) / 1e3)
    prop.check_errors()
    prop.close()
    e2e_times = _max_over_ranks(ctx, e2e_times, dev)
    e2e_t = float(np.mean(e2e_times))
    if ctx is not None:
        import torch.distributed as dist
        t = torch.tensor([float(h2d), float(d2h)], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)  # bytes copied by all ranks
        h2d, d2h = t.cpu().tolist()
    if not rank0:
        return

    inst_steps = n_total * nt
    ch = results[chosen]
    flops_launch = wl["flops_per_step"] * nt
    achieved = flops_launch / ch["sec_per_step"] / 1e12
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    line = dict(
        metric=METRIC, value=inst_steps / ch["sec_per_step"], unit=UNIT, n_gpus=world,
        steps=args.steps, warmup=args.warmup, ms_per_step=ch["sec_per_step"] * 1e3,
        higher_is_better=True, scaling="weak", vs_baseline=None,
        dtype={"fp32": "c64 (fp32)", "fp64": "c128 (fp64)", "3xtf32": "c64 via 3xTF32",
               "3xbf16": "c64 via 3xBF16"}[chosen],
        data="synthetic (seeded generators, pyqed_gb300/workloads.py)",
        config=dict(wl["desc"], path=chosen, schedule=ch["info"]["schedule"],
                    l2="flushed between timed steps (256 MB write)",
                    parallelism="single GPU" if ctx is None else
                    "%d GPUs, instances sharded by N^3 (LPT), no exchange; max over ranks" % world),
        gpu_launches=args.steps * ch["info"]["launches"] * world,
    )
    # roofline of the dominant kernel (the propagate launch)
    tf32_peak = measure_tf32_peak(dev) if ("3xtf32" in results) else None
    if chosen in ("3xtf32", "3xbf16"):
        pk = peaks.get("bf16_tflops", 1900.0)
        if chosen == "3xtf32":
            pk = tf32_peak
        traffic = None
        if args.workload == "exciton4096":
            # DRAM bytes per launch: operator/rho0 reads measured by ncu on a
            # small case (3xTF32: 304 mixed instances, 23.1 MB against 24.3 MB
            # algorithmic; 3xBF16: 152 instances of N = 64, 25.53 MB against
            # 25.37 MB) scaled by the algorithmic read bytes, plus the
            # algorithmic writes (C(t), rho)
            d64 = bi.dims.astype(np.int64)
            npd = np.where(d64 <= 64, (d64 + 15) // 16 * 16, (d64 + 3) // 4 * 4)
            reads = int((npd * (npd + 2) * 8 * (2 + bi.n_eops)).sum() + (d64 ** 2 * 16).sum())
            writes = int(n_inst * nt * bi.n_eops * 16 + (d64 ** 2 * 16).sum())
            traffic = int(reads * ((23.10 / 24.30) if chosen == "3xtf32" else (25.53 / 25.37))) + writes
        line["roofline"] = dict(bound="tensor", achieved=achieved, peak=pk, unit="TFLOP/s",
                                frac=achieved / pk, traffic=traffic,
                                # the split product runs three MMA products per algorithmic one
                                executed=3.0 * achieved, executed_frac=3.0 * achieved / pk,
                                traffic_note="bytes per launch: ncu-measured reads scaled to the "
                                             "full batch + algorithmic writes (profiles/)",
                                note="algorithmic 64*N^3 flops per instance-step; peak = "
                                     + ("the TF32 rate measured here (cuBLAS TF32 GEMM 8192^3)"
                                        if chosen == "3xtf32" else "measured bf16 (MEASURED_PEAKS.json)"))
    else:
        clk_mhz = (ch["clocks"] or {}).get("sm_max_mhz") or 2070.0
        pk = 152 * 128 * 2 * clk_mhz * 1e6 / 1e12
        line["roofline"] = dict(bound="fp32", achieved=achieved, peak=pk, unit="TFLOP/s",
                                frac=achieved / pk, traffic=None,
                                note="FP32 CUDA-core path; peak = 152 SMs x 128 FMA x 2 x max SM "
                                     "clock (nominal, no measured FP32 peak available)")
    line["plain"] = None
    if "fp32" in results and chosen != "fp32":
        pl = results["fp32"]
        line["plain"] = dict(value=inst_steps / pl["sec_per_step"], ms_per_step=pl["sec_per_step"] * 1e3,
                             speedup_chosen_over_plain=pl["sec_per_step"] / ch["sec_per_step"])
    for alt in results:
        if alt not in (chosen, "fp32"):
            a = results[alt]
            line.setdefault("alternatives", {})[alt] = dict(
                value=inst_steps / a["sec_per_step"], ms_per_step=a["sec_per_step"] * 1e3,
                speedup_over_plain=(results["fp32"]["sec_per_step"] / a["sec_per_step"]
                                    if "fp32" in results else None))
            if alt == "3xtf32" and tf32_peak:
                ach = wl["flops_per_step"] * nt / a["sec_per_step"] / 1e12
                line["alternatives"][alt].update(achieved_tflops=ach, tf32_peak_measured=tf32_peak,
                                                 frac=ach / tf32_peak)
    line["e2e"] = dict(value=inst_steps / e2e_t, unit=UNIT, ms_per_step=e2e_t * 1e3,
                       h2d_bytes_per_step=int(h2d), d2h_bytes_per_step=int(d2h),
                       api="pyqed_gb300.engine.Propagator.set_operators + propagate "
                           "(C ABI lgb_plan_set_operators/lgb_plan_propagate)")
    line["clocks"] = ch["clocks"]
    if not args.no_adjoint:
        line["adjoint"] = measure_adjoint(args, dev)
    if not args.no_large_n:
        line["large_n"] = measure_large_n(args, dev)
    if not args.no_redfield:
        line["redfield"] = measure_redfield(args, dev)
    if not args.no_heom:
        line["heom"] = measure_heom(args, dev, n_inst=args.heom_n_inst, nt=args.heom_nt)
    if not args.no_spectral:
        line["spectral"] = measure_spectral(args, dev)
    # CPU baseline (oracle port of the reference's dense algorithm) and accuracy
    if not args.no_cpu:
        line["cpu_baseline"], line["accuracy"] = cpu_baseline_and_accuracy(
            wl, results, args, chosen)
        if line["accuracy"] and chosen in line["accuracy"]:
            # the metric holds at |drho| <= 1e-5: say whether the chosen path met it
            line["accuracy_ok"] = line["accuracy"][chosen]["ok"]
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# adjoint cost: the metric's bwd/fwd on the driven workload
# ---------------------------------------------------------------------------
def measure_adjoint(args, dev):
    """256 driven instances, N=64, K=2, H(t) = H0 - E(t) mu, 2000 steps,
    loss sum_t |<O>(t) - target(t)|^2, gradients w.r.t. E(t) and gamma_k,
    checkpoints every 45 steps.  fwd = propagate with checkpoints,
    bwd = lgb_plan_adjoint (segment recompute + backward costate)."""
    import torch
    from pyqed_gb300 import workloads as W
    from pyqed_gb300.adjoint import DrivenBatch
    n_inst = args.adj_n_inst
    d = W.driven_batch(n_inst=n_inst, nt=args.adj_nt)
    nt = d["nt"]
    batch = DrivenBatch(d["H0"], [[m] for m in d["mu"]], d["L"], d["rho0"], [[o] for o in d["O"]],
                        d["dt"], nt, checkpoint_every=45, device=dev)
    # the loss target: the observables of the perturbed pulse E + dE
    target = batch.forward(d["E_target"][None, :], d["gamma"]).detach().clone()
    E = d["E"][None, :]
    stream = torch.cuda.current_stream(dev)

    def once():
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        obs = batch.forward(E, d["gamma"])
        e1.record(stream)
        g = 2.0 * (obs - target)
        batch.backward(g)
        e2.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), e1.elapsed_time(e2)
    for _ in range(max(1, min(args.warmup, 2))):
        once()
    fw, bw = [], []
    for _ in range(max(1, min(args.steps, 3))):
        a, b = once()
        fw.append(a)
        bw.append(b)
    f, b = float(np.mean(fw)), float(np.mean(bw))
    flops = 64 * 3 * 64 ** 3 * n_inst * nt
    return dict(workload="driven%d" % n_inst, n_inst=n_inst, N=64, K=2, nt=nt, checkpoint_every=45,
                fwd_ms=f, bwd_ms=b, bwd_over_fwd=b / f,
                fwd_instance_steps_per_s=n_inst * nt / (f / 1e3),
                fwd_tflops=flops / (f / 1e3) / 1e12,
                loss="sum_t |<O>(t) - target(t)|^2, target from the forward run of E + dE",
                note="fwd: the CTA kernel with checkpoints every 45 steps -- with dense collapse "
                     "operators at N <= 88 every precision request (fp32, 3xtf32, 3xbf16) runs this "
                     "FP32 kernel, so it is the chosen forward of this workload; bwd: segment "
                     "recompute + costate kernel (includes the gradient contractions)")


# ---------------------------------------------------------------------------
# single large instances (GEMM schedule): the split-precision tensor-core
# GEMMs against the plain FP32 GEMMs
# ---------------------------------------------------------------------------
def measure_large_n(args, dev):
    """GUE N=256 (K=4, dt=0.01, 10000 steps) and N=1024 (K=8, scale 0.02,
    rank-4 rho0, dt=0.005, 1000 steps): ms per RK4 step of each path over
    ``--large-nt`` steps, and each path's max-abs rho error after the
    workload's full length against the reference's own ``_fast_lindblad``
    result (tests/golden/gue256_long.npz: the whole final state;
    gue1024_long.npz: rows 0..15 and the diagonal), when the fixture is
    present and the seeded inputs match it."""
    import hashlib
    import torch
    from pyqed_gb300 import workloads as W
    from pyqed_gb300.engine import Propagator, pack
    out = {}
    gold = os.path.join(ROOT, "tests", "golden")

    def digest(*arrays):
        h = hashlib.sha256()
        for a in arrays:
            h.update(np.ascontiguousarray(a, dtype=np.complex128).tobytes())
        return h.hexdigest()
    cases = [("gue256", dict(N=256, K=4, seed=2, dt=0.01, nt=10000)),
             ("gue1024", dict(N=1024, K=8, scale=0.02, rank=4, seed=4, dt=0.005, nt=1000))]
    want = set(getattr(args, "large_cases", "gue256,gue1024").split(","))
    paths = [p for p in getattr(args, "large_paths", "3xtf32,3xbf16,fp32").split(",") if p]
    for name, kw in cases:
        if name not in want:
            continue
        w = W.gue_instance(**kw)
        N, K, dt, nt_full = kw["N"], kw["K"], kw["dt"], kw["nt"]
        H, C, R0 = pack([w["H"]]), pack(w["c_ops"]), pack([w["rho0"]])

        def run(prec, nt, timed):
            prop = Propagator([N], nt=nt, dt=dt, n_cops=K, cops_kind="dense", precision=prec,
                              schedule="gemm", device=dev)
            prop.set_operators(H, C)
            r0 = prop.to_device(R0)
            o = prop.alloc_outputs(want_obs=False, want_rho=True)
            ms = None
            if timed:
                prop.propagate_device(r0, None, o)  # warm-up (library heuristics, caches)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                prop.propagate_device(r0, None, o)
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / nt
            else:
                prop.propagate_device(r0, None, o)
                torch.cuda.synchronize()
            prop.check_errors()
            rho = prop.unpack_rho(o[1])[0]
            prop.close()
            return ms, rho
        ref = None
        fx = os.path.join(gold, name + "_long.npz")
        if os.path.exists(fx) and not getattr(args, "no_large_errors", False):
            g = np.load(fx)
            if name == "gue256" and digest(w["H"], *w["c_ops"], w["rho0"]) == str(g["digest"]):
                ref = lambda r, g=g: float(np.abs(r - g["rho"]).max())  # noqa: E731
            elif name == "gue1024" and digest(w["H"], *w["c_ops"]) == str(g["digest_ops"]):
                ref = lambda r, g=g: float(max(np.abs(r[:16, :] - g["rows"]).max(),  # noqa: E731
                                               np.abs(np.diag(r) - g["diag"]).max()))
        flops = 64 * (1 + K) * N ** 3
        res = {}
        for prec in paths:
            ms, _ = run(prec, args.large_nt, True)
            res[prec] = dict(ms_per_step=ms, tflops_algorithmic=flops / (ms / 1e3) / 1e12)
            if ref is not None:
                _, rfull = run(prec, nt_full, False)
                res[prec]["max_abs_err_rho_full_length"] = ref(rfull)
        for prec in ("3xtf32", "3xbf16"):
            if prec in res and "fp32" in res:
                res[prec]["speedup_over_fp32"] = res["fp32"]["ms_per_step"] / res[prec]["ms_per_step"]
        out[name] = dict(N=N, K=K, dt=dt, steps_timed=args.large_nt, steps_full=nt_full, paths=res,
                         reference=("the reference's _fast_lindblad after %d steps (%s_long.npz)" % (nt_full, name)
                                    if ref is not None else "fixture absent: errors not measured"))
    out["note"] = ("split paths: hand-written TMA + tcgen05 complex GEMMs; N = 256: the persistent "
                   "kernel (lgb_gemm_persist.cu, one launch for all steps), N = 1024: the graph-replayed "
                   "kernels (lgb_gemm_tc.cu); fp32: cuBLAS CGEMM, pedantic math; algorithmic "
                   "64(1+K)N^3 flops per step")
    return out


# ---------------------------------------------------------------------------
# Redfield (pyqed/oqs.py:30-100, 364-459, 519-563): batched systems
# ---------------------------------------------------------------------------
def measure_redfield(args, dev, n_inst=2048, n=8, nt=1000, dt=0.1):
    """2048 disordered chains (N = 8, one Ohmic bath per site), 1000 RK4 steps
    of vec(rho) with the 64 x 64 generator: instance-steps/s per precision
    (CUDA events, generators resident), the generator build time, and the
    oracle's numpy rate for the same algorithm on a sample."""
    import torch
    from pyqed_gb300 import workloads as W
    from pyqed_gb300.redfield import _Plan, _eigen_parts, build_tensors
    chains = [W.redfield_chain(n=n, seed=100 + b) for b in range(n_inst)]
    parts = [_eigen_parts(c["H"], c["a_ops"], c["spectra"]) for c in chains]
    build_tensors(parts[:2], dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    R = build_tensors(parts, dev)
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    Ot = np.concatenate([np.concatenate([(p[1].conj().T @ e @ p[1]).T.flatten() for e in c["e_ops"]])
                         for c, p in zip(chains, parts)])
    r0 = np.concatenate([(p[1].conj().T @ c["rho0"] @ p[1]).flatten() for c, p in zip(chains, parts)])
    M = n * n
    flops = 32 * M * M  # 4 stages x complex GEMV (8 real flops per complex MAC)
    out = dict(workload="redfield_chain%d x %d" % (n, n_inst), N=n, n_inst=n_inst, nt=nt, dt=dt)
    for prec in ("fp32", "fp64"):
        plan = _Plan([n] * n_inst, nt, dt, 2, prec, 0, dev)
        plan.set(R, torch.from_numpy(Ot).to(dev))
        r0d = torch.from_numpy(r0).to(dev)
        plan.propagate(r0d)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        plan.propagate(r0d)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        plan.close()
        out[prec] = dict(seconds=t, instance_steps_per_s=n_inst * nt / t,
                         tflops=flops * n_inst * nt / t / 1e12)
    out["tensor_build_seconds"] = t_build
    if not args.no_cpu:
        from oracle import redfield_oracle as RO
        sample, steps = 16, 50
        # propagation only (the tensor builds are excluded above)
        cpu_t = 0.0
        for c in chains[:sample]:
            Rr, V = RO.redfield_tensor(c["H"], c["a_ops"], c["spectra"])
            y = (V.conj().T @ c["rho0"] @ V).flatten()
            t1 = time.perf_counter()
            for _ in range(steps):
                y = RO.rk4_vec(y, Rr, dt)
            cpu_t += time.perf_counter() - t1
        out["cpu_baseline"] = dict(instance_steps_per_s=sample * steps / cpu_t, kind="port",
                                   sample="%d chains x %d RK4 steps, numpy complex128" % (sample, steps))
    out["note"] = ("one CTA per system; FP32 (N^2 <= 64): the 64 x 64 generator in registers, four "
                   "threads per row; FP64: the generator (64 KB) in shared memory, warp-per-row GEMV "
                   "per stage; flops = 32 N^4 per instance-step")
    return out


def measure_size_class(args, dev, N=65, n_inst=152, nt=400, dt=0.05):
    """One size class of the exciton family alone: n_inst instances of
    dimension N (exciton_instance(N - 1, i, seed=5), dephasing on every site,
    the transition dipole as the observable), 3xTF32, nt RK4 steps.  Reports
    the per-instance-step time and the cycles per RK4 stage at 2.07 GHz; with
    n_inst = 152 every SM holds one instance, so this is the per-stage cost
    of that size's tensor-core kernel (N = 65 runs the border kernel)."""
    import torch
    from pyqed_gb300 import workloads as W
    from pyqed_gb300.batch import prepare_batch
    from pyqed_gb300.engine import Propagator
    insts = [W.exciton_instance(N - 1, index=i, seed=5) for i in range(n_inst)]
    bi = prepare_batch([x["H"] for x in insts], [[np.diag(c) for c in x["c_diag"]] for x in insts],
                       [x["rho_g"] for x in insts], [[x["mu"]] for x in insts])
    prop = Propagator(bi.dims, nt=nt, dt=dt, n_cops=bi.n_cops, cops_kind=bi.cops_kind, n_eops=1,
                      precision=args.precision)
    prop.set_operators(bi.H, bi.cops, bi.eops, bi.dops)
    r0 = prop.to_device(bi.rho0)
    o = prop.alloc_outputs(want_obs=True, want_rho=False)
    prop.propagate_device(r0, None, o)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    prop.propagate_device(r0, None, o)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    prop.close()
    return dict(workload="exciton N=%d x %d" % (N, n_inst), N=N, n_inst=n_inst, nt=nt, precision=args.precision,
                ms=ms, us_per_step=ms * 1e3 / nt, cycles_per_stage_at_2070mhz=ms * 1e-3 / nt / 4 * 2.07e9)


def heom_flops(N, nado, diag_sz=False):
    """Algorithmic flops of one sweep (one instance-step): level 0 and level
    nado-2 take two commutators (4 complex N^3 products), the levels between
    three brackets whose [sz, X_{n-1}] and {sz, X_{n-1}} share sz X and X sz
    (6 products); 8 real flops per complex multiply-add.  With a diagonal sz
    only the two [H, X_n] products per level are N^3."""
    L = nado
    if diag_sz:
        return (L - 1) * 2 * 8 * N ** 3
    prods = 4 if L == 2 else 8 + 6 * max(0, L - 3)
    return prods * 8 * N ** 3


def measure_heom(args, dev, n_inst=4096, n=8, nado=8, nt=1000, dt=0.01):
    """4096 disordered 8-site chains, each with its own Drude bath (one
    exponential mode), an 8-level hierarchy, 1000 Euler sweeps: instance-steps/s
    per precision (CUDA events, operators resident), and the oracle's numpy
    rate for the reference's sweep on a sample."""
    import torch
    from pyqed_gb300 import workloads as W
    from pyqed_gb300 import _capi as C
    from pyqed_gb300.heom import _Plan, _pack, bath_run
    e = W.heom_ensemble(n_inst, n, seed=13)
    bath = [bath_run(e["temperature"][b], e["cutoff"][b], e["reorganization"][b]) for b in range(n_inst)]
    coef = np.array([[g, d.real, d.imag] for g, d in bath]).ravel()
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    Hd, Sd, Cd = t(_pack(e["H"])), t(_pack(e["sz"])), t(coef)
    Od = t(_pack([o.T for es in e["e_ops"] for o in es]))
    r0 = t(_pack(e["rho0"]))
    flops, flops_diag = heom_flops(n, nado), heom_flops(n, nado, diag_sz=True)
    out = dict(workload="heom_chain%d x %d, %d levels" % (n, n_inst, nado), N=n, n_inst=n_inst, nado=nado,
               nt=nt, dt=dt)
    # the chains' sz is diagonal: the O(N^2) sz path; "fp32_dense_sz" times the
    # general (dense sz) kernel on the same systems
    for key, prec, flags in (("fp32", "fp32", C.HEOM_DIAG_SZ), ("fp64", "fp64", C.HEOM_DIAG_SZ),
                             ("fp32_dense_sz", "fp32", 0)):
        plan = _Plan([n] * n_inst, nt, dt, nado, 2, prec, flags, dev)
        plan.set(Hd, Sd, Cd, Od)
        res = plan.propagate(r0)
        torch.cuda.synchronize()
        best = None
        for _ in range(2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            plan.propagate(r0, out=res)
            e1.record()
            torch.cuda.synchronize()
            sec = e0.elapsed_time(e1) / 1e3
            best = sec if best is None else min(best, sec)
        plan.check_errors()
        fl = flops_diag if flags else flops
        out[key] = dict(seconds=best, instance_steps_per_s=n_inst * nt / best,
                        tflops=fl * n_inst * nt / best / 1e12, layout=plan.layout())
        plan.close()
    # the reference's spin-boson setting as a parameter sweep: 65536 two-level
    # systems (16 per warp), 10 levels, FP32, diagonal sz
    nsb, sb_levels = 65536, 10
    sb = W.heom_spin_boson()
    rng = np.random.default_rng(17)
    sbath = [bath_run(T, cu, lam) for T, cu, lam in zip(rng.uniform(0.5, 2.0, nsb), rng.uniform(0.2, 1.0, nsb),
                                                        rng.uniform(0.01, 0.2, nsb))]
    plan = _Plan([2] * nsb, nt, dt, sb_levels, 1, "fp32", C.HEOM_DIAG_SZ, dev)
    plan.set(t(np.tile(sb["H"].ravel(), nsb)), t(np.tile(sb["sz"].ravel(), nsb)),
             t(np.array([[g, d.real, d.imag] for g, d in sbath]).ravel()), t(np.tile(sb["sz"].T.ravel(), nsb)))
    r0s = t(np.tile(sb["rho0"].ravel(), nsb))
    res = plan.propagate(r0s)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    plan.propagate(r0s, out=res)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    plan.check_errors()
    out["spinboson"] = dict(n_inst=nsb, N=2, nado=sb_levels, nt=nt, seconds=sec,
                            instance_steps_per_s=nsb * nt / sec, layout=plan.layout())
    plan.close()
    if not args.no_cpu:
        from oracle import heom_oracle as HO
        sample, steps = 16, 100
        cpu_t = 0.0
        for b in range(sample):
            ado = np.zeros((nado, n, n), complex)
            ado[0] = e["rho0"][b]
            t1 = time.perf_counter()
            for _ in range(steps):
                HO.sweep(ado, e["H"][b], e["sz"][b], bath[b][0], bath[b][1], dt)
                [np.trace(o @ ado[0]) for o in e["e_ops"][b]]
            cpu_t += time.perf_counter() - t1
        out["cpu_baseline"] = dict(instance_steps_per_s=sample * steps / cpu_t, kind="port",
                                   sample="%d chains x %d sweeps, numpy complex128" % (sample, steps))
        ado = np.zeros((sb_levels, 2, 2), complex)
        ado[0] = sb["rho0"]
        t1 = time.perf_counter()
        for _ in range(200):
            HO.sweep(ado, sb["H"], sb["sz"], sbath[0][0], sbath[0][1], dt)
            np.trace(sb["sz"] @ ado[0])
        out["spinboson"]["cpu_baseline"] = dict(instance_steps_per_s=200 / (time.perf_counter() - t1), kind="port",
                                                sample="1 system x 200 sweeps, numpy complex128")
    out["note"] = ("one thread group per system (a warp: one thread per column and row pair), -iH, sz and "
                   "the %d levels in shared memory, one group barrier per level; flops per instance-step = "
                   "%d with the diagonal sz, %d with a dense sz (commutator products, 8 flops per complex "
                   "MAC)" % (nado, flops_diag, flops))
    return out


def measure_spectral(args, dev, nfock=8, n_t=100000, n_tau=512):
    """Eigen-decomposition solver on the Jaynes-Cummings system with 8 Fock
    states (N = 16, 256 modes): correlation_2op_1t at 1e5 time points and the
    two-time correlation_3op_2t on a 512 x 512 grid (GPU, CUDA events), the
    host eigendecomposition, and numpy on the same mode sums."""
    import torch
    from pyqed_gb300 import workloads as W
    from pyqed_gb300.spectral import Lindblad_solver
    jc = W.jaynes_cummings(nfock=nfock)
    H, c_ops, rho0 = jc["H"], jc["c_ops"], jc["rho0"]
    a, b = jc["e_ops"][0], jc["e_ops"][1]
    sol = Lindblad_solver(H, c_ops, device=dev)
    t0 = time.perf_counter()
    sol.eigenstates(complex_norm=True)
    t_eig = time.perf_counter() - t0
    tl = np.linspace(0.0, 200.0, n_t)
    tau = np.linspace(0.0, 50.0, n_tau)
    sol.correlation_2op_1t(rho0, [a, b], tl[:1000])
    sol.correlation_3op_2t(rho0, [a, b, a], tau[:8], tau[:8])
    out = dict(workload="jc%d spectral" % (2 * nfock), modes=int(sol.dim), n_t=n_t, n_tau=n_tau,
               eig_seconds_host=t_eig)
    for key, fn in (("corr_1t", lambda: sol.correlation_2op_1t(rho0, [a, b], tl)),
                    ("corr_3op_2t", lambda: sol.correlation_3op_2t(rho0, [a, b, a], tau, tau))):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        out[key + "_seconds"] = time.perf_counter() - t1
    if not args.no_cpu:
        lam = sol.eigvals
        co = sol._coeff_2op(rho0, a, b).cpu().numpy()
        t1 = time.perf_counter()
        _ = np.exp(np.outer(tl[:10000], lam)) @ co
        out["corr_1t_numpy_seconds_10k_points"] = time.perf_counter() - t1
    out["note"] = ("wall time per call incl. host mode weights and copies; the mode sums run in "
                   "lgb_spectral_sum (FP64), the 2t grid as two ZGEMMs (lgb_spectral_2t)")
    return out


# ---------------------------------------------------------------------------
# CPU baseline / reference arm (the oracle port; the only oracle use here)
# ---------------------------------------------------------------------------
def _sample_indices(dims, count):
    order = np.argsort(dims, kind="stable")
    q = ((np.arange(count) + 0.5) / count * len(dims)).astype(int)
    return sorted(int(order[i]) for i in q)


def cpu_port_rate(wl, n_sample, steps, csr=False):
    """Reference algorithm (the RHS of pyqed/oqs.py:697-715 + the RK4 of
    pyqed/phys.py:1051-1064), restated by the oracle, on a stratified sample
    of instances: dense numpy complex128 as ``_fast_lindblad``
    (pyqed/oqs.py:1492-1594) computes it, or with ``csr`` on scipy.sparse
    CSR operators and state as the reference's public ``run`` (``_lindblad``,
    pyqed/oqs.py:1596-1696) does."""
    from oracle import lindblad_oracle as O
    bi = wl["bi"]
    dims = bi.dims
    idx = _sample_indices(dims, min(n_sample, len(dims)))
    off = np.concatenate([[0], np.cumsum(dims.astype(np.int64) ** 2)])
    doff = np.concatenate([[0], np.cumsum(dims.astype(np.int64))])
    K = bi.n_cops
    tot = 0.0
    for b in idx:
        N = int(dims[b])
        H = bi.H[off[b]:off[b + 1]].reshape(N, N)
        if bi.cops_kind == "diag":
            cd = bi.cops[K * doff[b]: K * doff[b + 1]].reshape(K, N)
            cops = [np.diag(c) for c in cd]
        elif bi.cops_kind == "dense":
            cops = list(bi.cops[K * off[b]: K * off[b + 1]].reshape(K, N, N))
        else:
            cops = []
        rho = bi.rho0[off[b]:off[b + 1]].reshape(N, N).copy()
        if csr:
            from scipy.sparse import csr_matrix
            H, rho = csr_matrix(H), csr_matrix(rho)
            cops = [csr_matrix(c) for c in cops]
        t0 = time.perf_counter()
        for _ in range(steps):
            rho = O.rk4_step(rho, wl["dt"], H, cops)
        tot += time.perf_counter() - t0
    # mean time per instance-step over a sample stratified by N = the
    # workload's mean; rate over the whole batch follows
    mean_t = tot / (len(idx) * steps)
    return 1.0 / mean_t, idx


def cpu_baseline_and_accuracy(wl, results, args, chosen):
    import multiprocessing
    cores = os.cpu_count() or 1
    rate, idx = cpu_port_rate(wl, args.cpu_sample, args.cpu_steps)
    rate_csr, _ = cpu_port_rate(wl, args.cpu_sample, max(1, args.cpu_steps // 2), csr=True)
    cb = dict(value=rate, unit=UNIT, cores=cores, kind="port",
              sample="%d instances stratified by N x %d RK4 steps, dense numpy complex128 "
                     "(oracle restatement of the reference's RHS + rk4 as _fast_lindblad computes "
                     "it, BLAS threads = host)" % (len(idx), args.cpu_steps),
              csr_value=rate_csr,
              csr_sample="the same instances x %d steps with scipy.sparse CSR operators and state, "
                         "as the reference's public run (single-threaded scipy)"
                         % max(1, args.cpu_steps // 2))
    acc = None
    if wl.get("ex") is not None and args.workload == "exciton4096":
        from oracle import lindblad_oracle as O
        ex = wl["ex"]
        dims = wl["bi"].dims
        pick = _sample_indices(dims, args.acc_sample)
        # at least one instance of every padding class of the tensor-core
        # kernel (NP = 16, 32, 48, 64) and the largest (N = 65: the border)
        for lo, hi in ((1, 16), (17, 32), (33, 48), (49, 64), (65, 65)):
            cls = np.nonzero((dims >= lo) & (dims <= hi))[0]
            if cls.size and not any(lo <= dims[b] <= hi for b in pick):
                pick.append(int(cls[-1]))
        big = int(np.argmax(dims))
        if big not in pick:
            pick.append(big)
        pick = sorted(pick)
        acc = {}
        refs = {b: O.propagate_diag_correlation(ex["H"][b], ex["mu"][b], ex["rho_g"][b],
                                                ex["c_diag"][b], ex["dt"], wl["nt"],
                                                return_rho=True) for b in pick}
        for prec, r in results.items():
            errs = [np.abs(r["obs"][b, :, 0] - refs[b][0]).max() / np.abs(refs[b][0]).max()
                    for b in pick]
            rerr = []
            for b in pick:
                N = int(wl["bi"].dims[b])
                got = r["rho"][r["off"][b]:r["off"][b + 1]].reshape(N, N)
                rerr.append(np.abs(got - refs[b][1]).max())
            acc[prec] = dict(max_rel_err_C=float(max(errs)), max_abs_err_rho_final=float(max(rerr)),
                             ok=bool(max(errs) <= 1e-5 and max(rerr) <= 1e-5),
                             instances=pick, nt=wl["nt"],
                             reference="complex128 oracle (pyqed/oqs.py:717-791 recurrence)")
    del multiprocessing
    return cb, acc


def run_reference(args):
    """--impl reference: the reference's CPU algorithm (oracle port) on the
    host cores; one step = a bounded stratified sample of the workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    wl = make_workload(args.workload, args.n_inst, args.nt)
    for _ in range(args.warmup):
        cpu_port_rate(wl, max(2, args.cpu_sample // 4), 1)
    rates = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r, idx = cpu_port_rate(wl, args.cpu_sample, args.cpu_steps)
        rates.append(r)
    wall = time.perf_counter() - t0
    v = float(np.mean(rates))
    cores = os.cpu_count() or 1
    sample = ("%d instances stratified by N x %d RK4 steps per bench step, dense numpy complex128 "
              "restatement of the reference's RHS + rk4" % (len(idx), args.cpu_steps))
    line = dict(metric=METRIC, value=v, unit=UNIT, n_gpus=args.gpus, steps=args.steps,
                warmup=args.warmup, ms_per_step=wall / max(1, args.steps) * 1e3,
                higher_is_better=True, scaling="weak", vs_baseline=None, dtype="c128 (fp64)",
                data="synthetic (seeded generators, pyqed_gb300/workloads.py)",
                config=dict(make_workload_desc(wl), path="reference CPU (oracle port)"),
                impl="reference",
                cpu_baseline=dict(value=v, unit=UNIT, cores=cores, kind="port", sample=sample),
                e2e=dict(value=v, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0),
                gpu_launches=0)
    print(json.dumps(line))


def make_workload_desc(wl):
    return dict(wl["desc"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="exciton4096")
    ap.add_argument("--precision", default=os.environ.get("LGB_BENCH_PRECISION", "3xbf16"))
    ap.add_argument("--n-inst", type=int, default=None)
    ap.add_argument("--nt", type=int, default=None)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=32)
    ap.add_argument("--cpu-steps", type=int, default=4)
    ap.add_argument("--acc-sample", type=int, default=4)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--only-adjoint", action="store_true",
                    help="time only the adjoint (fwd + bwd) on the driven workload")
    ap.add_argument("--adj-n-inst", type=int, default=256)
    ap.add_argument("--adj-nt", type=int, default=2000)
    ap.add_argument("--no-redfield", action="store_true",
                    help="skip the batched Redfield section")
    ap.add_argument("--no-heom", action="store_true",
                    help="skip the batched HEOM section")
    ap.add_argument("--no-spectral", action="store_true",
                    help="skip the eigen-decomposition (spectral) section")
    ap.add_argument("--no-large-n", action="store_true",
                    help="skip the single large-instance (GEMM schedule) section")
    ap.add_argument("--large-nt", type=int, default=100)
    ap.add_argument("--large-cases", default="gue256,gue1024",
                    help="large-N section: comma-separated cases (gue256, gue1024)")
    ap.add_argument("--large-paths", default="3xtf32,3xbf16,fp32",
                    help="large-N section: comma-separated precisions")
    ap.add_argument("--no-large-errors", action="store_true",
                    help="large-N section: skip the full-length error runs")
    ap.add_argument("--only-large-n", action="store_true",
                    help="run only the single large-instance (GEMM schedule) section")
    ap.add_argument("--only-heom", action="store_true", help="run only the batched HEOM section")
    ap.add_argument("--heom-n-inst", type=int, default=4096)
    ap.add_argument("--heom-nt", type=int, default=1000)
    ap.add_argument("--only-redfield", action="store_true", help="run only the batched Redfield section")
    ap.add_argument("--rf-n-inst", type=int, default=2048)
    ap.add_argument("--rf-nt", type=int, default=1000)
    ap.add_argument("--only-size-class", type=int, default=None, metavar="N",
                    help="time one size class of the exciton family alone (N = 65: the border kernel)")
    ap.add_argument("--class-n-inst", type=int, default=152)
    ap.add_argument("--class-nt", type=int, default=400)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.only_large_n:
        import torch
        from pyqed_gb300.build import build
        build()
        print(json.dumps(dict(large_n=measure_large_n(args, torch.device("cuda", 0)))))
        return
    if args.only_heom:
        import torch
        from pyqed_gb300.build import build
        build()
        print(json.dumps(dict(heom=measure_heom(args, torch.device("cuda", 0), n_inst=args.heom_n_inst,
                                                nt=args.heom_nt))))
        return
    if args.only_redfield:
        import torch
        from pyqed_gb300.build import build
        build()
        print(json.dumps(dict(redfield=measure_redfield(args, torch.device("cuda", 0), n_inst=args.rf_n_inst,
                                                        nt=args.rf_nt))))
        return
    if args.only_size_class is not None:
        import torch
        from pyqed_gb300.build import build
        build()
        print(json.dumps(dict(size_class=measure_size_class(args, torch.device("cuda", 0), N=args.only_size_class,
                                                            n_inst=args.class_n_inst, nt=args.class_nt))))
        return
    if args.only_adjoint:
        import torch
        from pyqed_gb300.build import build
        build()
        print(json.dumps(dict(adjoint=measure_adjoint(args, torch.device("cuda", 0)))))
        return
    ctx = dist_context()
    if ctx is not None:
        # one rank per GPU, each propagating its share of the instances; the
        # extra sections (adjoint, large N, Redfield, HEOM, spectral, CPU
        # baseline) are single-GPU measurements
        args.no_adjoint = args.no_large_n = args.no_redfield = args.no_heom = True
        args.no_spectral = args.no_cpu = True
    try:
        run_gpu(args, ctx)
    finally:
        if ctx is not None:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
