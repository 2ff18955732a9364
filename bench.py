"""Benchmark: differentiated render + advect steps per second at 128^3 x 5 views.

One step = MacCormack advection of the density by the MAC velocity, render of
5 views (256x256 pixels, 128 depth samples, Beer-Lambert, BORDER), L2 loss to
target images, and the backward to density and velocity -- the per-iteration
work of the density / velocity reconstruction (configuration "differentiated
single step").  Inputs are seeded synthetic plumes.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--dtype f32|bf16] [--impl ngt|reference]

Prints one JSON line (rank 0).  ``--impl reference`` times the CPU
implementation of the same step (the NumPy restatement of the reference's
operators; the reference itself has no CPU path and its CUDA build needs
TensorFlow 1.12) on the host cores.
"""
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

METRIC = "fwd+bwd render+advect steps/s at 128^3 x 5 views"
WORKLOAD = "MacCormack advect (MC_SMOOTH, CLAMP, dt=1) + 5-view Beer-Lambert raymarch 256x256x128 (BORDER) + L2 + backward to density and MAC velocity, 128^3 grid"


# Arm CPU parts by MIDR part number (implementer 0x41), for the host description
_ARM_PARTS = {"0xd40": "Neoverse-V1", "0xd49": "Neoverse-N2", "0xd4f": "Neoverse-V2", "0xd84": "Neoverse-V3",
              "0xd8e": "Neoverse-N3"}


def host_cpu(cpuinfo="/proc/cpuinfo"):
    """The host the CPU baselines run on: architecture, logical CPUs and the CPU
    model (``model name`` on x86, the implementer / part words on Arm)."""
    import platform
    import re
    info = {"arch": platform.machine(), "logical_cpus": os.cpu_count()}
    try:
        with open(cpuinfo) as f:
            text = f.read()
    except OSError:
        return info
    m = re.search(r"^model name\s*:\s*(.+)$", text, re.M)
    if m:
        info["model"] = m.group(1).strip()
        return info
    parts = sorted(set(re.findall(r"^CPU part\s*:\s*(\S+)$", text, re.M)))
    impl = sorted(set(re.findall(r"^CPU implementer\s*:\s*(\S+)$", text, re.M)))
    if parts:
        names = [_ARM_PARTS.get(p, "part " + p) if impl == ["0x41"] else "part " + p for p in parts]
        info["model"] = ", ".join(names) + (" (implementer %s)" % "/".join(impl) if impl else "")
    return info


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--dtype", default="f32", choices=["f32", "bf16", "f16"])
    ap.add_argument("--impl", default="ngt", choices=["ngt", "reference"])
    ap.add_argument("--grad-mode", default="exact", choices=["exact", "reference"])
    ap.add_argument("--no-graph", action="store_true")
    # "full": also the same step in one process (about a minute of host time), beside the split over every core
    ap.add_argument("--cpu-baseline", default="on", choices=["on", "off", "full"])
    ap.add_argument("--kernel-stats", default="on", choices=["on", "off"])
    ap.add_argument("--workload", default="step", choices=["step", "chain", "large", "batch", "velocity"],
                    help="step: the headline differentiated step; chain: the checkpointed 120-frame plume "
                         "chain; large: 256x448x256 grid, 8 views at 512x512x256, 16-bit storage errors; "
                         "batch: 32 uneven scenes in one batched step; velocity: MAC velocity "
                         "self-advection at 128^3")
    ap.add_argument("--checkpoint-every", type=int, default=10)
    return ap.parse_args()


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ngt" else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value, device):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        t0 = time.time()
        while not self.lines and time.time() - t0 < 10 and self.proc.poll() is None:
            time.sleep(0.01)  # the first sample arrives before the timed region starts
        self.skip = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for ln in self.lines[getattr(self, "skip", 0):] or self.lines[-1:]:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# DRAM bytes (read + write) per call of the step's dominant library call in f32,
# summed over the call's kernels, each kernel captured alone by ncu (one launch,
# cold cache) on this workload.  They come from a profile, not from the run that
# prints them; the capture and its date go with the number.
NCU_TRAFFIC_F32 = {
    "raymarch_fwd_l2_bwd": {"bytes": 104.53e6 + 34.16e6 + 34.10e6,
                            "kernels": {"k_raymarch_fwd_bwd": 138.69e6, "k_quad_fold": 34.10e6},
                            "kind": "profile", "captured": "2026-12-04",
                            "profile": "profiles/render_fused_f32_128cube_5views.md"},
}
# The resources that bound that call's main kernel (k_raymarch_fwd_bwd), from the same
# capture: L1-to-L2 requests (quad gathers and float4 quad-gradient atomics).
NCU_LIMITER_F32 = {"raymarch_fwd_l2_bwd": {"resource": "L1-to-L2 requests (quad gathers + float4 atomics)",
                                           "l1tex2xbar_req_pct": 58.2, "lsu_wavefronts_pct": 48.6,
                                           "l2_atomic_input_pct": 32.6, "l1tex_pct": 65.3,
                                           "captured": "2026-12-04",
                                           "profile": "profiles/render_fused_f32_128cube_5views.md"}}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ------------------------------------------------------------------- CPU legs
# The CPU implementation of the step is the oracle, the NumPy restatement of the
# reference's operators (the reference itself has no CPU path: REGISTER__CPU is
# empty, resample_grid.cc:1179-1181, and its CUDA build needs TensorFlow 1.12).
# Every CPU step below is one FULL step of the headline workload -- 128^3
# MacCormack warp, 5 views of 256 x 256 x 128, image L2, backward to density and
# velocity -- split over spawned host processes by oracle.parallel (warp as
# z-slabs with halos, render as bands of image rows): nothing is sampled or
# scaled.
CPU_SAMPLE = ("one full step (128^3 MacCormack warp + 5-view 256x256x128 render + L2 + backward) of the oracle, "
              "the NumPy restatement of the reference operators (the reference has no CPU path), split over %d "
              "spawned host processes: warp and its adjoint as z-slabs with halos, render as 8-row image bands")


def cpu_inputs():
    """The headline workload's inputs and its targets (rendered by the oracle)."""
    import __graft_entry__
    __graft_entry__.load_package()
    from ngt_gb300 import workloads
    return workloads.config2()


def cpu_step(pool, nproc, w, targets):
    """Seconds of one full differentiated step of the oracle on the host."""
    from oracle import parallel
    t0 = time.perf_counter()
    parallel.render_advect_step(pool, nproc, w.rho, w.ux, w.uy, w.uz, w.M, w.V, w.P, w.F, targets, w.image_dhw,
                                w.depth_step)
    return time.perf_counter() - t0


# Wall-clock budget of the reference arm's timed steps (seconds): a run asking for
# more steps than fit stops there and reports ``steps_timed``.
REFERENCE_BUDGET_S = 240.0


def reference_setup():
    """(pool, processes, workload, targets) of the reference arm: a pool of spawned
    workers over every host CPU and the targets rendered by the oracle (untimed)."""
    from oracle import parallel
    w = cpu_inputs()
    pool, nproc = parallel.make_pool()
    try:
        tgt, _, _ = parallel.render_l2(pool, nproc, w.rho_target, w.depth_step, w.M, w.V, w.P, w.F, w.image_dhw)
    except BaseException:
        pool.close()
        raise
    return pool, nproc, w, np.ascontiguousarray(tgt[..., :1])


def reference_arm(args, world, rank):
    if rank != 0:
        return
    pool, nproc, w, tgt = reference_setup()
    times = []
    try:
        for _ in range(args.warmup):
            cpu_step(pool, nproc, w, tgt)
        t_begin = time.perf_counter()
        for _ in range(args.steps):
            times.append(cpu_step(pool, nproc, w, tgt))
            if time.perf_counter() - t_begin > REFERENCE_BUDGET_S:
                break
    finally:
        pool.close()
        pool.join()
    value = 1.0 / float(np.mean(times))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "steps_timed": len(times), "warmup": args.warmup, "ms_per_step": 1e3 / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": [128, 128, 128], "views": 5, "image": [256, 256],
                       "depth_samples": 128},
            "timed_s": float(np.sum(times)),
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": nproc, "kind": "port",
                             "sample": CPU_SAMPLE % nproc, "host": host_cpu()},
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------- GPU arm
def gpu_arm(args, world, rank, local):
    import torch
    import __graft_entry__
    __graft_entry__.load_package()
    from ngt_gb300 import _build, workloads
    from ngt_gb300.step import RenderAdvectStep
    _build.build_library()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = workloads.config2()
    st = {"f32": torch.float32, "bf16": torch.bfloat16, "f16": torch.float16}[args.dtype]

    def dt(a):
        return torch.as_tensor(a, device=dev).to(st).contiguous()

    rho, ux, uy, uz = dt(w.rho), dt(w.ux), dt(w.uy), dt(w.uz)
    # targets: render of the perturbed density (no advection)
    from ngt_gb300 import ops
    with torch.no_grad():
        tgt = ops.raymarch_grid_transform(torch.as_tensor(w.rho_target, device=dev)[None], w.M, w.V, w.P, w.F,
                                          w.image_dhw, emission_scale=(w.depth_step, w.depth_step))[..., :1]
    step = RenderAdvectStep(rho, ux, uy, uz, w.M, w.V, w.P, w.F, tgt, w.image_dhw, grad_mode=args.grad_mode)
    if not args.no_graph:
        step.capture()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        step.step()
    torch.cuda.synchronize()
    # timed region: per-step device time between events; L2 flushed between steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    t_wall0 = time.perf_counter()
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record(stream)
        step.step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    barrier(world)
    clk = clocks.stop()
    step_ms = float(np.sum([a.elapsed_time(b) for a, b in ev]))
    step_ms = max_over_ranks(world, step_ms, dev)
    ms_per_step = step_ms / args.steps
    value = world * 1e3 / ms_per_step  # whole job: every rank runs its own step (replicas)
    loss_val = float(step.loss.item())

    # per-call device times (no graph) for the roofline of the dominant kernel
    kernel = None
    if args.kernel_stats == "on":
        kernel = kernel_stats(step, torch, dev, w, st, max(10, args.steps // 2), flush)

    e2e = e2e_measure(torch, dev, w, st, tgt, args, flush)
    e2e_ops = e2e_measure(torch, dev, w, st, tgt, args, flush, fused=False)
    e2e_step = e2e_step_measure(torch, step, w, st, args, flush) if not args.no_graph else None
    samples = 2 * 2 * 128 ** 3 + 2 * 5 * 256 * 256 * 128
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.dtype,
            "data": "synthetic (seeded Gaussian-blob density, curl-noise MAC velocity, 5 orbit cameras)",
            "config": {"workload": WORKLOAD, "grid": [128, 128, 128], "views": 5, "image": [256, 256],
                       "depth_samples": 128, "grad_mode": args.grad_mode, "cuda_graph": not args.no_graph,
                       "l2": "flushed between timed steps (256 MiB write, outside the step events)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "voxel_samples_per_s": samples * value, "loss": loss_val,
            "gpu_launches": RenderAdvectStep.KERNELS_PER_STEP * args.steps,
            "wall_s_timed_region": t_wall,
            "algorithmic_bytes_per_step": workloads.algorithmic_bytes((128, 128, 128), 5, (256, 256),
                                                                      elem=torch.tensor([], dtype=st).element_size())}
    peak, peak_kind = measured_peak_hbm()
    line["hbm_frac_of_step"] = line["algorithmic_bytes_per_step"] / (ms_per_step * 1e-3) / (peak * 1e9)
    if kernel:
        name, avg_ms, nbytes, calls = kernel
        line["call_ms"] = calls  # every library call of the step, CUDA events, L2 flushed before each step
        achieved = nbytes / (avg_ms * 1e-3) / 1e9
        line["roofline"] = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "peak_kind": peak_kind,
                            "traffic": NCU_TRAFFIC_F32[name]["bytes"] if args.dtype == "f32" and name in NCU_TRAFFIC_F32
                            else None,
                            "algorithmic_bytes_per_launch": nbytes, "avg_ms": avg_ms}
        if args.dtype == "f32" and name in NCU_TRAFFIC_F32:
            t = NCU_TRAFFIC_F32[name]
            line["roofline"]["traffic_source"] = {k: t[k] for k in ("kind", "captured", "profile", "kernels")}
        if args.dtype == "f32" and name in NCU_LIMITER_F32:
            line["roofline"]["measured_limiter"] = NCU_LIMITER_F32[name]
    if clk:
        line["clocks"] = clk
    line["e2e"] = e2e
    line["e2e_ops"] = e2e_ops
    if e2e_step:
        line["e2e_step"] = e2e_step
    if rank == 0 and world == 1 and args.cpu_baseline in ("on", "full"):
        from oracle import parallel
        targets = np.ascontiguousarray(tgt.cpu().numpy())
        pool, nproc = parallel.make_pool()  # spawned workers: no CUDA in them
        try:
            t = cpu_step(pool, nproc, w, targets)
        finally:
            pool.close()
            pool.join()
        line["cpu_baseline"] = {"value": 1.0 / t, "unit": "steps/s", "cores": nproc, "kind": "port",
                                "sample": CPU_SAMPLE % nproc + "; the same inputs and targets as the GPU step",
                                "host": host_cpu()}
        if args.cpu_baseline == "full":
            pool1, _ = parallel.make_pool(1)
            try:
                t1 = cpu_step(pool1, 1, w, targets)
            finally:
                pool1.close()
                pool1.join()
            line["cpu_baseline"]["single_process"] = {"value": 1.0 / t1, "unit": "steps/s", "seconds": t1,
                                                      "sample": "the same full step in one process"}
    if rank == 0:
        print(json.dumps(line), flush=True)


def kernel_stats(step, torch, dev, w, st, iters, flush):
    """Average device time of each C-ABI call of the step (events around each
    call, L2 flushed before each step) and the algorithmic bytes it moves."""
    import ctypes
    from ngt_gb300.ops import _ptr
    es = torch.tensor([], dtype=st).element_size()
    n_rho = 128 ** 3
    n_u = 3 * 129 * 128 * 128
    px = 5 * 256 * 256
    nbytes = {
        "advect_fwd": es * (2 * n_rho + n_u),                 # rho, u read; rho' written
        "raymarch_quad": es * n_rho,                          # rho' read (its gather layout is scratch)
        # rho' read; image and image gradient written, target read; d rho' written
        "raymarch_fwd_l2_bwd": es * n_rho + 4 * (2 * px + px + 2 * px) + 4 * n_rho,
        "advect_bwd": es * (n_rho + n_u) + 4 * (n_rho + n_rho) + 4 * (n_rho + n_u),  # rho,u,fwd,grad in; grads out
    }
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # the step's library calls, in its order
    calls = [("advect_fwd", lambda: step._call("ngt_advect_maccormack_fwd", ctypes.byref(step.adv), s)),
             ("raymarch_quad", lambda: step._call("ngt_raymarch_quad", ctypes.byref(step.ray), _ptr(step.ray_quad), s)),
             ("raymarch_fwd_l2_bwd", lambda: step._call("ngt_raymarch_fwd_l2_bwd", ctypes.byref(step.ray_g), None,
                                                        _ptr(step.targets), 1, _ptr(step.loss), s)),
             ("advect_bwd", lambda: step._call("ngt_advect_maccormack_bwd", ctypes.byref(step.adv_g), s))]
    tot = {n: 0.0 for n, _ in calls}
    for it in range(iters + 2):
        flush.zero_()
        evs = []
        for n, fn in calls:
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            evs.append((n, a, b))
        torch.cuda.synchronize()
        if it >= 2:
            for n, a, b in evs:
                tot[n] += a.elapsed_time(b)
    name = max(tot, key=tot.get)
    return name, tot[name] / iters, nbytes[name], {n: tot[n] / iters for n in tot}


def e2e_measure(torch, dev, w, st, tgt, args, flush, fused=True):
    """Same step through the public autograd API, with the density and velocity
    copied from pinned host memory every step and the loss read back.  fused:
    the one differentiable call ``step.render_advect_loss``; else the three
    operators ``advect.warp`` -> ``ops.raymarch_grid_transform`` ->
    ``ops.image_l2_loss`` with autograd between them."""
    from ngt_gb300 import advect, ops
    from ngt_gb300.step import render_advect_loss
    host = [torch.as_tensor(a).to(st).pin_memory() for a in (w.rho, w.ux, w.uy, w.uz)]
    h2d = sum(t.numel() * t.element_size() for t in host)
    scale = (w.depth_step, w.depth_step)
    # the optimisation's density and velocity: device tensors that require grad,
    # as an optimiser keeps them; every step copies its inputs into them from
    # pinned host memory and clears their gradients
    ts = [torch.empty(t.shape, dtype=t.dtype, device=dev).requires_grad_() for t in host]

    def one():
        with torch.no_grad():
            for d, h in zip(ts, host):
                d.copy_(h, non_blocking=True)
        for d in ts:
            d.grad = None
        if fused:
            loss = render_advect_loss(ts[0], ts[1], ts[2], ts[3], w.M, w.V, w.P, w.F, tgt, w.image_dhw)
        else:
            r2 = advect.warp(ts[0], ts[1], ts[2], ts[3], dt=1.0, order=2, clamp="MC_SMOOTH", boundary="CLAMP")
            img = ops.raymarch_grid_transform(r2[None], w.M, w.V, w.P, w.F, w.image_dhw, emission_scale=scale)
            loss = ops.image_l2_loss(img, tgt)
        loss.backward()
        return float(loss.item())

    for _ in range(max(2, args.warmup)):
        one()
    torch.cuda.synchronize()
    n = max(5, args.steps // 2)
    tot = 0.0
    for _ in range(n):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        one()
        tot += time.perf_counter() - t0
    path = ("ngt_gb300.step.render_advect_loss (one autograd node), loss.backward()" if fused else
            "ngt_gb300.advect.warp + ngt_gb300.ops.raymarch_grid_transform + ops.image_l2_loss, loss.backward()")
    path += "; inputs copied into the optimisation's device tensors every step"
    return {"value": n / tot, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 4, "path": path}


def e2e_step_measure(torch, step, w, st, args, flush):
    """The fused step's public call (``RenderAdvectStep.step``, one CUDA graph)
    end to end: density and velocity copied from pinned host memory into the
    step's inputs every step, the loss read back."""
    host = [torch.as_tensor(a).to(st).pin_memory() for a in (w.rho, w.ux, w.uy, w.uz)]
    dst = [step.rho, step.ux, step.uy, step.uz]
    h2d = sum(t.numel() * t.element_size() for t in host)

    def one():
        for d, h in zip(dst, host):
            d.copy_(h, non_blocking=True)
        return float(step.step().item())

    for _ in range(max(2, args.warmup)):
        one()
    torch.cuda.synchronize()
    n = max(5, args.steps // 2)
    tot = 0.0
    for _ in range(n):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        one()
        tot += time.perf_counter() - t0
    return {"value": n / tot, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 4,
            "path": "ngt_gb300.step.RenderAdvectStep.step (one CUDA graph)"}


# ------------------------------------------------------------ other workloads
def _timed(torch, fn, steps, warmup, flush):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    stream = torch.cuda.current_stream()
    for i in range(steps):
        flush.zero_()
        ev[i][0].record(stream)
        fn()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    return float(np.mean([a.elapsed_time(b) for a, b in ev]))


def chain_arm(args, local):
    """The checkpointed multi-frame chain (96x176x96 plume, 120 frames, one
    192x192x96 camera): forward with checkpoints every K frames, backward with
    per-segment recompute, as one CUDA graph."""
    import torch
    import __graft_entry__
    __graft_entry__.load_package()
    from ngt_gb300 import _build, workloads
    from ngt_gb300.chain import AdvectRenderChain, chain_targets
    _build.build_library()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = workloads.config3()
    st = {"f32": torch.float32, "bf16": torch.bfloat16, "f16": torch.float16}[args.dtype]
    T = lambda a: torch.as_tensor(a, device=dev).to(st).contiguous()
    u = [T(w.ux), T(w.uy), T(w.uz)]
    tg = chain_targets(T(w.rho0_target), *u, T(w.source), w.M, w.V, w.P, w.F, w.image_dhw, w.frames)
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    ch = AdvectRenderChain(T(w.rho0), *u, T(w.source), w.M, w.V, w.P, w.F, tg, w.image_dhw, w.frames,
                           checkpoint_every=args.checkpoint_every)
    ch.capture()
    chain_bytes = torch.cuda.max_memory_allocated() - base
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    ms = _timed(torch, ch.run, args.steps, max(args.warmup, 3), flush)
    D, H, W = w.grid
    line = {"metric": "checkpointed plume chain fwd+bwd frames/s", "value": w.frames * 1e3 / ms,
            "unit": "frames/s", "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_chain": ms, "higher_is_better": True, "dtype": args.dtype, "data": "synthetic plume",
            "config": {"workload": "MacCormack + 1-view render per frame, %d frames, checkpoint every %d" %
                                   (w.frames, args.checkpoint_every),
                       "grid": [D, H, W], "image": list(w.image_dhw[1:]), "depth_samples": w.image_dhw[0],
                       "l2": "flushed between timed chains", "cuda_graph": True},
            "loss": float(ch.loss.item()), "chain_device_bytes": int(chain_bytes),
            "stored_densities": ch.nseg + ch.K + 3, "densities_without_checkpoints": 2 * w.frames}
    print(json.dumps(line), flush=True)


def large_arm(args, local):
    """The reduced-precision configuration: 256x448x256 density and MAC velocity,
    8 views at 512x512 with 256 depth samples; the step in FP32 and in 16-bit
    storage, and the errors of every image and gradient against the FP64 path."""
    import torch
    import __graft_entry__
    __graft_entry__.load_package()
    from ngt_gb300 import _build, ops, workloads
    from ngt_gb300.step import RenderAdvectStep
    _build.build_library()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = workloads.render_step(grid=(256, 448, 256), views=8, image=(512, 512), depth=256, max_u=2.0)
    with torch.no_grad():
        tgt = ops.raymarch_grid_transform(torch.as_tensor(w.rho_target, device=dev, dtype=torch.float64)[None],
                                          w.M, w.V, w.P, w.F, w.image_dhw,
                                          emission_scale=(w.depth_step, w.depth_step))[..., :1]
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def make(dt, vt=None):
        """The step with the density stored as dt and the faces as vt (default dt)."""
        vt = vt or dt
        t = [torch.as_tensor(w.rho, device=dev).to(dt).contiguous()] + \
            [torch.as_tensor(x, device=dev).to(vt).contiguous() for x in (w.ux, w.uy, w.uz)]
        return RenderAdvectStep(*t, w.M, w.V, w.P, w.F, tgt, w.image_dhw)

    results = {}
    ref = make(torch.float64)
    ref.step()
    torch.cuda.synchronize()
    ref_out = [ref.image.clone()] + [g.clone() for g in ref.gradients()]
    del ref
    names = ["image", "d_rho", "d_ux", "d_uy", "d_uz"]
    f32_out = None
    for name, dt, vt in (("f32", torch.float32, None), ("bf16", torch.bfloat16, None), ("f16", torch.float16, None),
                         ("bf16+f16", torch.bfloat16, torch.float16)):
        s = make(dt, vt)
        s.capture()
        ms = _timed(torch, s.step, args.steps, max(args.warmup, 3), flush)
        out = [s.image.clone()] + [g.clone() for g in s.gradients()]
        errs = {}
        for n, a, b in zip(names, out, ref_out):
            a, b = a.double(), b.double()
            errs[n] = {"rel_l2_vs_fp64": float((a - b).norm() / b.norm()),
                       "max_abs_vs_fp64": float((a - b).abs().max())}
            if f32_out is not None:
                c = f32_out[names.index(n)].double()
                errs[n]["rel_l2_vs_fp32"] = float((a - c).norm() / c.norm())
        if name == "f32":
            f32_out = out
        results[name] = {"ms_per_step": ms, "errors": errs}
        del s
        torch.cuda.empty_cache()
    line = {"metric": "fwd+bwd render+advect steps/s at 256x448x256 x 8 views (16-bit storage)",
            "value": 1e3 / results["bf16"]["ms_per_step"], "unit": "steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(args.warmup, 3), "higher_is_better": True, "dtype": "bf16 storage, f32 arithmetic",
            "data": "synthetic (seeded Gaussian blobs, curl-noise MAC velocity)",
            "config": {"workload": "MacCormack + 8-view Beer-Lambert raymarch 512x512x256 + L2 + backward",
                       "grid": [256, 448, 256], "views": 8, "image": [512, 512], "depth_samples": 256,
                       "l2": "flushed between timed steps"},
            "bf16_speedup_vs_f32": results["f32"]["ms_per_step"] / results["bf16"]["ms_per_step"],
            "f16_speedup_vs_f32": results["f32"]["ms_per_step"] / results["f16"]["ms_per_step"],
            "bf16_density_f16_velocity_speedup_vs_f32": results["f32"]["ms_per_step"] / results["bf16+f16"]["ms_per_step"],
            "runs": results}
    print(json.dumps(line), flush=True)


def batch_arm(args, local):
    """32 scenes of uneven size (axes 48-160, 1-8 cameras, images 64-256, depth
    32-128): the batched step (batched advection, the render's forward, loss and
    backward of every scene in one persistent launch with an autotuned grid) as one
    CUDA graph, against one library call per scene and operator captured in a CUDA
    graph as well."""
    import torch
    import __graft_entry__
    __graft_entry__.load_package()
    from ngt_gb300 import _build, ops, workloads
    from ngt_gb300.batch import BatchedScenes, Scene
    _build.build_library()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    st = {"f32": torch.float32, "bf16": torch.bfloat16, "f16": torch.float16}[args.dtype]
    ws = workloads.config4()
    sc = []
    for w in ws:
        with torch.no_grad():
            tgt = ops.raymarch_grid_transform(torch.as_tensor(w.rho_target, device=dev)[None], w.M, w.V, w.P, w.F,
                                              w.image_dhw, emission_scale=(w.depth_step, w.depth_step))[..., :1]
        T = lambda a: torch.as_tensor(a, device=dev).to(st).contiguous()
        sc.append(Scene(T(w.rho), T(w.ux), T(w.uy), T(w.uz), w.M, w.V, w.P, w.F, w.image_dhw, tgt))
    b = BatchedScenes(sc)
    tuned = b.autotune()
    b.capture()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    ms = _timed(torch, b.step, args.steps, max(args.warmup, 3), flush)
    loss = float(b.loss.item())
    # the same step as one call per scene and operator, also in a CUDA graph
    b.per_scene()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(side):
        b.per_scene()
    torch.cuda.synchronize()
    with torch.cuda.graph(g):
        b.per_scene_launch()
    ms_ps = _timed(torch, g.replay, args.steps, max(args.warmup, 3), flush)
    samples = sum(w.views * w.image_dhw[0] * w.image_dhw[1] * w.image_dhw[2] for w in ws) * 2 + \
        sum(2 * w.grid[0] * w.grid[1] * w.grid[2] for w in ws)
    line = {"metric": "batched uneven scenes fwd+bwd steps/s (32 scenes)", "value": 1e3 / ms, "unit": "steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
            "higher_is_better": True, "dtype": args.dtype, "data": "synthetic (seeded blobs, curl-noise velocity)",
            "config": {"workload": "32 scenes, axes 48-160, 1-8 cameras, images 64-256, depth 32-128; SL advect + "
                                   "render + L2 + backward", "cuda_graph": True, "l2": "flushed between timed steps",
                       "scenes": [[list(w.grid), w.views, list(w.image_dhw)] for w in ws]},
            "voxel_samples_per_s": samples * 1e3 / ms, "loss": loss,
            "per_scene_calls_ms_per_step": ms_ps, "speedup_vs_per_scene_calls": ms_ps / ms,
            "autotuned_blocks_per_sm": {"render_fwd_l2_bwd": tuned[0][0]},
            "autotune_ms": {"render_fwd_l2_bwd": tuned[0][1]}}
    print(json.dumps(line), flush=True)


def velocity_arm(args, local):
    """MAC velocity self-advection (``VelocityGrid.warped``: every face component
    MacCormack-advected on its own lattice by the velocity resampled there) at
    128^3, forward and backward through the C ABI as one CUDA graph, against the
    oracle's NumPy restatement on one host core (a 32^3 sample scaled by cells)."""
    import ctypes
    import torch
    import __graft_entry__
    __graft_entry__.load_package()
    from ngt_gb300 import _build, _lib as L, synthetic
    from ngt_gb300.ops import _ptr
    from oracle import advect as oadvect
    _build.build_library()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    st = {"f32": torch.float32, "bf16": torch.bfloat16, "f16": torch.float16}[args.dtype]
    n = 128
    u = [torch.as_tensor(a, device=dev).to(st).contiguous()
         for a in synthetic.curl_noise_mac((n, n, n), max_u=2.0, seed=1)]
    outs = [torch.empty_like(t) for t in u]
    fwds = [torch.empty(t.shape, dtype=torch.float32, device=dev) for t in u]
    rng = np.random.default_rng(5)
    gout = [torch.as_tensor(rng.standard_normal(tuple(t.shape)).astype(np.float32), device=dev) for t in u]
    gin = [torch.empty(t.shape, dtype=torch.float32, device=dev) for t in u]
    a = L.AdvectVelocityArgs()
    a.dtype = {torch.float32: L.F32, torch.bfloat16: L.BF16, torch.float16: L.F16}[st]
    a.grid_dhw = L.I64x3(n, n, n)
    a.vel_x, a.vel_y, a.vel_z = (_ptr(t) for t in u)
    a.dt, a.order, a.clamp, a.boundary = 1.0, 2, L.CLAMP["MC_SMOOTH"], L.BOUNDARY["CLAMP"]
    a.out_x, a.out_y, a.out_z = (_ptr(t) for t in outs)
    a.fwd_x, a.fwd_y, a.fwd_z = (_ptr(t) for t in fwds)
    # per component: the stored lookup, the MC_SMOOTH revert mask, the corner extrema
    scratch = [(torch.empty(tuple(t.shape) + (3,), device=dev), torch.empty(t.shape, dtype=torch.uint8, device=dev),
                torch.empty(tuple(t.shape) + (2,), device=dev)) for t in u]
    for c, (lut, mask, ext) in enumerate(scratch):
        a.lookup[c], a.mask[c], a.extrema[c] = _ptr(lut), _ptr(mask), _ptr(ext)
    g = L.AdvectVelocityGradArgs()
    g.fwd = a
    g.grad_x, g.grad_y, g.grad_z = (_ptr(t) for t in gout)
    g.vel_x_grad, g.vel_y_grad, g.vel_z_grad = (_ptr(t) for t in gin)
    g.grad_mode = L.GRAD["exact"]
    lib = L.load()
    ws = torch.empty(int(lib.ngt_advect_velocity_bwd_workspace_bytes(ctypes.byref(g))), dtype=torch.uint8,
                     device=dev)
    g.workspace, g.workspace_bytes = _ptr(ws), ws.numel()

    def launch():
        s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        L.call("ngt_advect_velocity_fwd", ctypes.byref(a), s)
        L.call("ngt_advect_velocity_bwd", ctypes.byref(g), s)

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        launch()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        launch()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    ms = _timed(torch, graph.replay, args.steps, max(args.warmup, 3), flush)
    # the oracle on one core, a 32^3 sample scaled by the cell count
    m = 32
    uc = synthetic.curl_noise_mac((m, m, m), max_u=2.0, seed=1)
    t0 = time.perf_counter()
    outs_o = oadvect.velocity_maccormack(*uc)
    oadvect.velocity_maccormack_grad(*uc, outs_o)
    t_cpu = (time.perf_counter() - t0) * (n / m) ** 3
    line = {"metric": "MAC velocity self-advection fwd+bwd steps/s at 128^3", "value": 1e3 / ms, "unit": "steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
            "higher_is_better": True, "dtype": args.dtype, "data": "synthetic (seeded curl-noise MAC velocity)",
            "config": {"workload": "MacCormack (MC_SMOOTH, CLAMP, dt=1) of the three face grids of a 128^3 MAC "
                                   "velocity on their own lattices, forward + backward", "cuda_graph": True,
                       "l2": "flushed between timed steps"},
            "cpu_baseline": {"value": 1.0 / t_cpu, "unit": "steps/s", "cores": 1, "kind": "port",
                             "sample": "oracle (NumPy fp32, one process): 32^3 grid, scaled x%d" % (n // m) ** 3,
                             "host": host_cpu()}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_init(args)
    if args.impl == "reference":
        reference_arm(args, world, rank)
    elif args.workload == "chain":
        chain_arm(args, local)
    elif args.workload == "large":
        large_arm(args, local)
    elif args.workload == "batch":
        batch_arm(args, local)
    elif args.workload == "velocity":
        velocity_arm(args, local)
    else:
        gpu_arm(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
