#!/usr/bin/env python
"""Swarm log-likelihood evaluations/s on the glycine-like workload
(N=4000 training points, d=24 features, rbf ARD over 17 dims + periodic over
7 dihedrals, concentrated likelihood, swarm of 40 particles) -- one "step" is
one PSO iteration's swarm evaluated in one graph-captured batched pass.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl fgpu|reference]

* value       : swarm evaluations/s with theta already resident in HBM
                (device-pointer entry point), max time over ranks.
* e2e         : the same metric through the public batched C-ABI call with
                host buffers (theta H2D and ll/info D2H inside the timed region).
* plain       : evaluations/s of the one-particle-per-call drop-in
                (fgpu_loglik), over 40 particles.
* roofline    : the dominant kernel, the tensor-core trailing update
                (k_ozaki_update): the fp16 tensor flops it issues (7 digit
                planes, 28 digit pairs per 128 x 64 x 128 tile) over its
                CUDA-event time inside the timed region, against the measured
                sustained bf16 peak (MEASURED_PEAKS.json); its FP64-equivalent
                rate is set beside the FP64 DGEMM peak measured live.
                `traffic` is scaled from the committed ncu capture
                (profiles/traffic.json: DRAM bytes per 128 x 64 tile) to the
                tiles of one launch.
* build       : the kernel-matrix build's algorithmic HBM bytes
                (8 N(N+1)/2 written + 8 N d + 8 N read per evaluation) over the
                build stage's time, against the measured HBM bandwidth.
* cpu_baseline: the C restatement of the reference's OpenMP CPU path on a
                bounded sample of particles, all host cores.
Inputs are larger than L2: each step writes 40 K matrices (5.3 GB).
``--impl reference`` times only the CPU restatement (the reference itself is
Fortran and cannot be built on these machines), on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "ferebus-v7_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "swarm logL evals/s (N=4000,d=24) batched vs plain on 1 GB300; FP64/HBM roofline %"
UNIT = "evals/s"
WORKLOAD = "glycine-like swarm: N=4000, d=24 (rbf 17 dims + periodic 7 dihedrals), concentrated, S=40"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def update_flops(N, nrhs, tb=64):
    """Algorithmic flops of all trailing updates of one factorisation:
    step s updates the lower triangle (incl. diagonal) of the remaining
    t = N - tb (s+1) columns plus the nrhs right-hand-side rows, rank tb."""
    tot = 0.0
    s = 0
    while True:
        t = N - tb * (s + 1)
        if t <= 0:
            break
        tot += 2.0 * tb * (t * (t + 1) / 2.0 + nrhs * t)
        s += 1
    return tot


def tensor_update_flops(N, nslice=7, nb=128, tn=64):
    """fp16 tensor-core flops the split-integer trailing update issues for one
    factorisation: per step s, m(m+1) output tiles of nb x tn (m trailing
    128-row tiles), each nb*tn*nb multiply-adds per digit pair, and
    nslice(nslice+1)/2 digit pairs."""
    nt = -(-N // nb)
    pairs = nslice * (nslice + 1) // 2
    tiles = sum((nt - s - 1) * (nt - s) for s in range(nt))
    return 2.0 * nb * tn * nb * pairs * tiles


def fp64_peak_tflops(torch):
    """Live FP64 peak: cuBLAS DGEMM 8192^3, best of 3."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def cpu_baseline(problem, mu, sample, threads):
    """Time the C restatement of the reference's CPU path on ``sample`` particles."""
    from oracle.build_ref import RefCPU
    ref = RefCPU(problem.X, problem.y, mu, problem.kspec, problem.likelihood, problem.noise,
                 problem.optimise_noise)
    th = problem.thetas(sample, seed=7)
    t0 = time.perf_counter()
    ll, info = ref.loglik_batch(th, threads)
    dt = time.perf_counter() - t0
    ref.close()
    return sample / dt, dt, ll, info


def host_info():
    try:
        model = subprocess.run("lscpu | grep 'Model name' | head -1", shell=True, capture_output=True,
                               text=True).stdout.split(":")[-1].strip()
    except Exception:
        model = "unknown"
    return os.cpu_count(), model


def workload_config(p, S, ws):
    """The `config` object of both arms' JSON lines."""
    return {"workload": WORKLOAD, "N": p.N, "d": p.d, "swarm": S, "likelihood": "concentrated",
            "kernel": "rbf(17) + periodic(7)",
            "l2": "inputs larger than L2: 40 K matrices = 5.3 GB written per step",
            "parallelism": f"replicas x{ws} (independent swarms per GPU)"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        if rank != 0:
            dist.barrier()
            dist.destroy_process_group()
            return
    from fgpu import synth
    from fgpu.gpr import mean_vector
    p = synth.config3()
    mu = mean_vector(p.mean, p.X, p.y)
    cores, model = host_info()
    sample = args.ref_sample or cores
    from oracle.build_ref import RefCPU
    ref = RefCPU(p.X, p.y, mu, p.kspec, p.likelihood, p.noise, p.optimise_noise)
    th = p.thetas(sample * (args.warmup + args.steps), seed=11)
    for w in range(args.warmup):
        ref.loglik_batch(th[w * sample:(w + 1) * sample], cores)
    t0 = time.perf_counter()
    for k in range(args.steps):
        o = (args.warmup + k) * sample
        ref.loglik_batch(th[o:o + sample], cores)
    dt = (time.perf_counter() - t0) / args.steps
    ref.close()
    v = sample / dt
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, shapes of the glycine-like config)",
            "config": workload_config(p, args.swarm, ws),
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{sample} of the swarm's particles per step ({model}); C restatement of "
                                       "the reference's OpenMP path (distance tensors + dgemv + dpotrf/dpotrs)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


def host_mem_available():
    try:
        for ln in open("/proc/meminfo"):
            if ln.startswith("MemAvailable:"):
                return int(ln.split()[1]) * 1024
    except OSError:
        pass
    return 0


def shape_problems(key):
    """(problems, swarm size, description) of one benchmark shape."""
    from fgpu import synth
    if key == "water_like_500":
        return [synth.config1()], 20, "water-like: N=500, d=3, rbf(1,2)+periodic(3), constant mean, marginal, S=20"
    if key == "methanol_like_2000":
        return [synth.config2()], 50, "methanol-like: N=2000, d=12, rbf(1-9)+periodic(10-12), marginal, S=50"
    if key == "atoms_33_ragged":
        return synth.config4(), 30, ("33 atoms, N ~ U{500..6000}, d=93, rbf+periodic(30 dihedrals), linear mean, "
                                     "marginal, 30 particles each: 990 problems per step")
    if key == "large_n_10000":
        return [synth.config5()], 16, ("large-N: N=10000, d=30, rbf+periodic, quadratic mean, optimised noise "
                                       "in [1e-12, 1e-6], S=16")
    raise KeyError(key)


def tune_shape(probs, mus, S):
    """The autotuner's configuration for this batch (fgpu.autotune: each
    candidate timed on a sample of the batch's largest problems)."""
    from fgpu import autotune
    wl = [autotune.Workload(q.X, q.y, mu, q.kspec, q.likelihood, q.noise, q.optimise_noise, S)
          for q, mu in zip(probs, mus)]
    dev, sms = autotune.device_identity()
    cfg, ms, hit = autotune.tune(wl, device=dev, sms=sms)
    return cfg, {"choice": cfg.name, "candidates_ms_per_sample_replay": ms, "from_cache": hit,
                 "sample": "the batch's largest problems, 8 evaluations"}


def measure_shape(key, torch, stream, steps, warmup, tpeak, cores, cpu_model, no_cpu):
    """Throughput, end-to-end rate, update roofline and a bounded CPU sample
    of one benchmark shape: every particle of every problem in one batch plan,
    in the configuration the autotuner picks for the shape."""
    from fgpu import Engine, Plan, autotune
    from fgpu.gpr import mean_vector
    probs, S, desc = shape_problems(key)
    mus = [mean_vector(q.mean, q.X, q.y) for q in probs]
    cfg, tuned = tune_shape(probs, mus, S)
    with autotune.use(cfg):
        engines = [Engine(q.X, q.y, mu, q.kspec, q.likelihood, q.noise, q.optimise_noise)
                   for q, mu in zip(probs, mus)]
    flat = [e for e in engines for _ in range(S)]
    nth = max(e.ntheta for e in engines)
    plan = Plan(flat, ldtheta=nth)
    nwaves, arena = plan.waves()
    total = warmup + steps
    th = np.zeros((total, len(flat), nth))
    for a, q in enumerate(probs):
        t = q.thetas(S * total, seed=40 + a).reshape(total, S, q.ntheta)
        th[:, a * S:(a + 1) * S, :q.ntheta] = t
    th_dev = torch.tensor(th, dtype=torch.float64, device="cuda")
    ll_dev = torch.empty((total, len(flat)), dtype=torch.float64, device="cuda")
    info_dev = torch.empty((total, len(flat)), dtype=torch.int32, device="cuda")
    plan.set_profiling("update")

    def step(k):
        plan.run_device(th_dev[k].data_ptr(), ll_dev[k].data_ptr(), info_dev[k].data_ptr(), stream.cuda_stream)

    for w in range(warmup):
        step(w)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(steps):
        step(warmup + k)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    upd_ms, upd_n = plan.stage_times()["update"]
    launches = plan.launches()
    fail = float(np.mean(info_dev[warmup:].cpu().numpy() != 0))
    plan.set_profiling(False)
    t0 = time.perf_counter()
    for k in range(steps):
        plan.run(th[warmup + k])
    e2e_s = (time.perf_counter() - t0) / steps
    tflops = sum(tensor_update_flops(q.N) * S for q in probs)
    achieved = tflops / (upd_ms * 1e-3) / 1e12 if upd_ms > 0 and cfg.trailing == "tcgen05" else None
    out = {"workload": desc, "problems_per_step": len(flat), "value": len(flat) / (ms * 1e-3), "unit": UNIT,
           "ms_per_step": ms, "tuned": tuned, "waves": nwaves, "workspace_arena_gb": arena / 1e9,
           "e2e": {"value": len(flat) / e2e_s, "unit": UNIT, "h2d_bytes_per_step": len(flat) * nth * 8,
                   "d2h_bytes_per_step": len(flat) * 12},
           "roofline": {"bound": "tensor", "kernel": "k_ozaki_update" if cfg.trailing == "tcgen05" else
                        "k_update (FP64; no tensor-core roofline)", "achieved": achieved, "peak": tpeak,
                        "unit": "TFLOP/s", "frac": achieved / tpeak if achieved else None,
                        "update_ms_per_step": upd_ms, "update_launches": upd_n},
           "gpu_launches": launches * steps, "cholesky_failure_rate": fail}
    del plan, th_dev, ll_dev, info_dev
    for e in engines:
        e.close()
    if no_cpu:
        return out
    # bounded CPU sample: one particle per core of up to three problems (for
    # the ragged batch the atoms at the 10th, 50th and 90th size percentile,
    # skipping any whose d x N x N distance tensors would not fit in host memory)
    from oracle.build_ref import RefCPU
    order = sorted(range(len(probs)), key=lambda a: probs[a].N)
    pick = sorted({order[int(f * (len(order) - 1))] for f in (0.1, 0.5, 0.9)}) if len(probs) > 1 else [0]
    done, secs, names, used = 0, 0.0, [], 0
    for a in pick:
        q = probs[a]
        threads, why = ref_cpu_threads(q, cores)
        if threads < 1:
            names.append(f"N={q.N} skipped ({why})")
            continue
        ref = RefCPU(q.X, q.y, mus[a], q.kspec, q.likelihood, q.noise, q.optimise_noise)
        t = q.thetas(threads, seed=77)
        t0 = time.perf_counter()
        ref.loglik_batch(t, threads)
        secs += time.perf_counter() - t0
        ref.close()
        done += threads
        used = max(used, threads)
        names.append(f"N={q.N}: {threads} in parallel" + (f" ({why})" if why else ""))
    if done:
        out["cpu_baseline"] = {"value": done / secs, "unit": UNIT, "cores": used, "kind": "port",
                               "sample": f"{done} particles ({'; '.join(names)}), in {secs:.1f} s "
                                         f"({cpu_model}); C restatement of the reference's OpenMP CPU path"}
    return out


def ref_cpu_threads(q, cores):
    """Particles the C restatement can evaluate in parallel in host memory:
    it holds two d x N x N tensors, and every particle thread its own copy of
    a leaf's active-dimension slice (n x N x N, as the reference copies it)
    and a few N x N matrices.  Returns (threads, reason when fewer than cores)."""
    from fgpu.kernel_spec import parse_kspec
    avail = host_mem_available() or 64e9
    nn = 8.0 * q.N * q.N
    tensors = 2 * q.d * nn
    slices = [len(nd[2]) for nd in parse_kspec(q.kspec) if nd[0] == "leaf" and nd[1] in (1, 2)]
    per_thread = (max(slices) if slices and max(slices) < q.d else 0) * nn + 5 * nn
    room = 0.5 * avail - tensors
    threads = int(min(cores, room // per_thread)) if room > 0 else 0
    if threads >= cores:
        return cores, ""
    return threads, (f"{tensors / 1e9:.0f} GB of tensors + {per_thread / 1e9:.1f} GB per particle "
                     f"against {avail / 1e9:.0f} GB of host memory")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fgpu", choices=("fgpu", "reference"))
    ap.add_argument("--swarm", type=int, default=40)
    ap.add_argument("--plain", type=int, default=40, help="particles timed on the plain path")
    ap.add_argument("--cpu-sample", type=int, default=0, help="particles in the CPU baseline sample")
    ap.add_argument("--ref-sample", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--trailing", default="auto", choices=("auto", "tcgen05", "fp64"),
                    help="trailing-update arithmetic of the Cholesky (auto: the autotuner's choice)")
    ap.add_argument("--shapes", default="water_like_500,methanol_like_2000,atoms_33_ragged,large_n_10000",
                    help="other benchmark shapes measured after the headline ('none' to skip)")
    ap.add_argument("--shape-steps", type=int, default=3)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from fgpu import Engine, Plan, autotune, synth
    from fgpu.build import build_library
    from fgpu.gpr import mean_vector
    build_library()
    p = synth.config3()
    mu = mean_vector(p.mean, p.X, p.y)
    S = args.swarm
    tuned = None
    if args.trailing == "auto":
        cfg, tuned = tune_shape([p], [mu], S)
    else:
        cfg = autotune.Config(args.trailing, "tc" if args.trailing == "tcgen05" else "fp64")
    mode = cfg.trailing
    with autotune.use(cfg):
        eng = Engine(p.X, p.y, mu, p.kspec, p.likelihood, p.noise, p.optimise_noise)
    plan = Plan([eng] * S)
    nth = eng.ntheta
    total = args.warmup + args.steps
    th_host = p.thetas(S * total, seed=1 + rank).reshape(total, S, nth)
    th_dev = torch.tensor(th_host, dtype=torch.float64, device="cuda")
    ll_dev = torch.empty((total, S), dtype=torch.float64, device="cuda")
    info_dev = torch.empty((total, S), dtype=torch.int32, device="cuda")
    # a dedicated stream: the plan's graph, the timing events and the
    # synchronisation below all live on it (torch's default stream has handle 0,
    # which the C-ABI would read as "use the plan's own stream")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    # CUDA-event nodes around the trailing-update launches only: the kernel
    # the roofline is quoted on is timed live inside the timed region, and
    # the rest of the graph runs as it does unprofiled
    plan.set_profiling("update")

    def step(k):
        plan.run_device(th_dev[k].data_ptr(), ll_dev[k].data_ptr(), info_dev[k].data_ptr(), stream.cuda_stream)

    for w in range(args.warmup):
        step(w)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for k in range(args.steps):
            step(args.warmup + k)
        e1.record(stream)
        torch.cuda.synchronize()
    launches_per_step = plan.launches()
    ms = e0.elapsed_time(e1) / args.steps
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t)
    value = S * ws / (ms * 1e-3)
    stages = plan.stage_times()
    info_all = info_dev[args.warmup:].cpu().numpy()
    fail_rate = float(np.mean(info_all != 0))

    # e2e: the public batched call with host buffers (theta H2D, ll/info D2H)
    from fgpu import loglik_batch
    eng_list = [eng] * S
    loglik_batch(eng_list, list(th_host[0]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        loglik_batch(eng_list, list(th_host[args.warmup + k]))
    e2e_s = (time.perf_counter() - t0) / args.steps
    if ws > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t)
    e2e = {"value": S * ws / e2e_s, "unit": UNIT, "h2d_bytes_per_step": S * nth * 8,
           "d2h_bytes_per_step": S * (8 + 4)}

    # plain one-particle-per-call drop-in
    eng.loglik(th_host[0][0])
    t0 = time.perf_counter()
    for k in range(args.plain):
        eng.loglik(th_host[args.warmup][k % S])
    plain_v = args.plain / (time.perf_counter() - t0)

    # the adjoint (gradient polish) at the same shape, one particle: the
    # factor, likelihood and alpha from the tensor-core evaluation (the plain
    # path's graph), then FP64 work 2 N^3 / 3 (triangular inverse N^3/3,
    # K^-1 = L^-T L^-1 N^3/3) + the fused dK pass (~10 flops per entry and dim)
    eng.grad(th_host[0][0])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(2):
        eng.grad(th_host[args.warmup][k])
    grad_s = (time.perf_counter() - t0) / 2
    grad_flops = 2.0 * float(p.N) ** 3 / 3.0 + 10.0 * p.N * (p.N + 1) / 2 * p.d

    # per-stage breakdown (diagnostic): one more, untimed replay with event
    # nodes around every launch
    plan.set_profiling(True)
    step(args.warmup)
    torch.cuda.synchronize()
    breakdown = plan.stage_times()
    plan.set_profiling(False)
    del plan
    torch.cuda.empty_cache()
    fp64_peak = fp64_peak_tflops(torch)
    upd_ms, upd_n = stages["update"]
    fp64_flops = update_flops(p.N, 0 if mode == "tcgen05" else 2, tb=128 if mode == "tcgen05" else 64) * S
    fp64_equiv = fp64_flops / (upd_ms * 1e-3) / 1e12 if upd_ms > 0 else None
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic.json")
    if mode == "tcgen05" and os.path.exists(tf) and upd_n:
        # bytes per 128 x 64 tile from one ncu capture, scaled to this run's
        # tiles per launch (traffic grows with the tiles processed)
        try:
            per_tile = json.load(open(tf))["k_ozaki_update_bytes_per_tile"]
            nt = -(-p.N // 128)
            tiles = sum((nt - s - 1) * (nt - s) for s in range(nt)) * S
            traffic = per_tile * tiles / upd_n
        except Exception:
            traffic = None
    stage_ms = {k: v[0] for k, v in breakdown.items() if v[1]}
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peaks = json.load(open(peaks_path)) if os.path.exists(peaks_path) else {}
    # the kernel-matrix build against HBM: algorithmic bytes per evaluation
    # (lower triangle of K written, X and y / mu read) over the build stage
    build_bytes = S * (8.0 * p.N * (p.N + 1) / 2 + 8.0 * p.N * p.d + 8.0 * p.N)
    hbm = peaks.get("hbm_gbs") or 6800.0
    build_ms = stage_ms.get("build")
    build = {"bytes_per_step": build_bytes, "ms_per_step": build_ms,
             "achieved_gbs": build_bytes / (build_ms * 1e-3) / 1e9 if build_ms else None,
             "peak_gbs": hbm, "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks.get("hbm_gbs")
             else "fallback 6.8 TB/s (profiling recipe)"}
    build["hbm_frac"] = build["achieved_gbs"] / hbm if build["achieved_gbs"] else None
    tpeak = peaks.get("bf16_tflops_sustained")
    src = "MEASURED_PEAKS.json bf16_tflops_sustained (dense fp16/bf16 tensor, kernel timed inside a long step)"
    if not tpeak:
        tpeak, src = 1700.0, "fallback: 1.7 PFLOP/s sustained bf16 (profiling recipe)"
    if mode == "tcgen05":
        tflops = tensor_update_flops(p.N) * S
        achieved = tflops / (upd_ms * 1e-3) / 1e12 if upd_ms > 0 else None
        roof = {"bound": "tensor", "achieved": achieved, "peak": tpeak, "unit": "TFLOP/s",
                "frac": (achieved / tpeak) if achieved else None, "traffic": traffic,
                "traffic_source": "DRAM bytes per 128 x 64 tile from the committed ncu capture "
                                  "(profiles/traffic.json) x tiles per launch; not measured in this run",
                "kernel": "k_ozaki_update (tcgen05.mma kind::f16, 7 fp16 digit planes, exact int64 accumulation)",
                "peak_source": src, "tensor_flops_per_step": tflops, "launches_per_step": upd_n,
                "fp64_equivalent": {"achieved": fp64_equiv, "fp64_peak": fp64_peak, "unit": "TFLOP/s",
                                    "ratio": (fp64_equiv / fp64_peak) if fp64_equiv else None,
                                    "fp64_peak_source": "measured live: cuBLAS DGEMM 8192^3"},
                "stage_ms_last_step": stage_ms}
    else:
        roof = {"bound": "tensor", "achieved": fp64_equiv, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": (fp64_equiv / fp64_peak) if fp64_equiv else None, "traffic": traffic,
                "kernel": "k_update (FP64 mma.sync m8n8k4 trailing update)",
                "peak_source": "measured live in this run: cuBLAS DGEMM 8192^3 FP64 (not in MEASURED_PEAKS.json)",
                "algorithmic_flops_per_step": fp64_flops, "launches_per_step": upd_n,
                "stage_ms_last_step": stage_ms}
    cpu = None
    if rank == 0 and not args.no_cpu:
        cores, model = host_info()
        sample = args.cpu_sample or 5 * cores  # ~10 s of CPU work on the 16-core host
        try:
            v, dt, _, _ = cpu_baseline(p, mu, sample, cores)
            cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": f"{sample} particles of the same workload in {dt:.1f} s on {cores} threads ({model}); "
                             "C restatement of the reference's OpenMP CPU path"}
        except Exception as exc:  # report, never fall back
            cpu = {"value": None, "unit": UNIT, "cores": cores, "kind": "port", "sample": f"failed: {exc}"}
    clocks = clk.summary()
    shapes = {}
    if rank == 0 and args.shapes != "none":
        cores, cpu_model = host_info()
        for key in args.shapes.split(","):
            try:
                shapes[key] = measure_shape(key, torch, stream, args.shape_steps, 3, tpeak, cores, cpu_model,
                                            args.no_cpu)
            except Exception as exc:  # report, never fall back
                shapes[key] = {"error": f"{type(exc).__name__}: {exc}"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, shapes of the glycine-like config)",
            "config": workload_config(p, S, ws),
            "trailing_update": mode, "engine_config": cfg.name, "tuned": tuned,
            "roofline": roof, "build": build, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": launches_per_step * args.steps,
            "plain": {"value": plain_v, "unit": UNIT, "particles": args.plain,
                      "calls": "fgpu_loglik from one host thread, one call after the other"},
            "grad": {"ms": grad_s * 1e3, "fp64_flops": grad_flops,
                     "fp64_tflops": grad_flops / grad_s / 1e12, "fp64_peak_tflops": fp64_peak,
                     "frac": grad_flops / grad_s / 1e12 / fp64_peak,
                     "what": "fgpu_grad (d logL / d theta), one particle, host wall clock: the tensor-core "
                             "evaluation's factor, then K^-1 and the dK pass in FP64 (fp64_flops: that FP64 part)"},
            "batched_over_plain": value / ws / plain_v if plain_v else None,
            "shapes": shapes,
            "cholesky_failure_rate": fail_rate}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
