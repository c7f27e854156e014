#!/usr/bin/env python
"""Momentum-loop integration benchmark on GB300.

Workload (default): C2, the finite-T 3+1D loop -- 384 integrals (T in {0.05, 0.2, 1.0} x 128
external momenta), each 129 Matsubara modes x 64 q x 32 cos = 264192 integrand points, one
seeded 64x128 FP32 dressing table Z(mode, |q|).

Arms:
  ours (default)      one step = one batched, fused FP32-compensated evaluation of the whole
                      workload (libgbint, inputs resident in HBM) -> `value` (integrals/s);
                      `e2e` = the same through the public API with the dressing table uploaded
                      from pinned host memory and the results read back every step.  Beside it:
                      the plain per-integral FP64 GPU path (the reference's execution pattern,
                      the 20x denominator), the fused FP64 path, p50/p99 latencies, the roofline
                      against this GPU's measured FP32/MUFU peaks and the CPU baseline (the FP64
                      oracle on all host cores).
  --impl reference    the reference's CPU integrator restated (the FP64 oracle port; DiFfRG's
                      own build needs deal.II/TBB/GSL/RMM, absent here) on all host cores.

Multi-GPU: replicas (integrals are independent; no data-path collective) -- every rank runs the
full workload on its GPU, time = max over ranks, value = all ranks' integrals / time.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "integrals/s and p99 request latency, batched FP32-comp vs plain FP64, 1 GPU"
UNIT = "integrals/s"
# algorithmic work per integrand point after hoisting the per-row invariants: F basic FP32 flops
# (FMA = 2, add/mul = 1), S special functions (log, exp/expm1, div, rcp, sqrt); C2 counts each
# sign of the Matsubara frequency as a point, as the reference does.
#   C1 PROP1: x2 (2), log index (2), fraction (1), lerp (3), Z x2 + R (2), weights (2); log, expm1, div, rcp
#   C2 FTLOOP: C1's terms + bilinear (6 instead of 3) + w^2 + x2 (1) + mode fraction hoisted; 4 specials
#   C3 PROP3: r2, t2, s (6), three log-axis lookups (3 x 6), Z r2 + R (2), products + sum (4);
#             3 logs + expm1, div, rcp
#   C5 VERT4: r2 (2), one log index shared by both tables (3), two bilinears (2 x 7), Z r2 + R (2),
#             products + sum (4); log, expm1, div, rcp
PER_POINT = {"C1": (12, 4), "C2": (18, 4), "C3": (30, 6), "C5": (25, 4)}
# dram__bytes_read.sum + dram__bytes_write.sum of one launch of the dominant kernel, from one ncu
# capture of that kernel (summaries under profiles/, named for kernel and workload); a changed
# kernel needs a new capture -- the JSON line carries these as "traffic" with their source
TRAFFIC_BYTES_PER_LAUNCH = {"C2": 1497600, "C3": 6239488, "C5": 819456}
# thread instructions executed per integrand point by the dominant kernel (smsp__inst_executed.sum
# x 32 / points, same captures): with the measured step time they give the issue rate, the
# bound this double-float code actually meets (one warp instruction per SM sub-partition and cycle)
INSTR_PER_POINT = {"C2": 47, "C3": 150.5, "C5": 111}
CAPTURE_NOTE = ("ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,smsp__inst_executed.sum capture of the "
                "dominant kernel on this workload (profiles/)")


def evaluated_points(w):
    """Integrand points the kernel actually evaluates per launch (the quadrature counts both
    members of a folded phi pair and both signs of +-omega at W = 0; the kernels evaluate each
    once and double its weight)."""
    name = w["name"]
    if name == "C1":
        return len(w["p"]) * w["nq"] * w["nc"]
    if name == "C2":  # every integral has W = 0: modes n = 0..M evaluated once
        return len(w["p"]) * (w["M"] + 1) * w["nq"] * w["nc"]
    if name == "C3":
        o = w["orders"].astype(np.int64)
        return int((o[:, 0] * o[:, 1] * ((o[:, 2] + 1) // 2)).sum())
    if name == "C5":
        nq, n1, n2, n3 = w["n"]
        return len(w["P"]) * nq * n1 * n2 * ((n3 + 1) // 2)
    return None


def evaluated_block(w, points, frac32, fracxu):
    """The roofline fractions against the points the kernel evaluates (beside the quadrature's
    count, which the headline metric and the reference use)."""
    ev = evaluated_points(w)
    if not ev:
        return None
    r = ev / points
    return {"points_per_launch": ev, "of_quadrature_points": r, "fp32_frac": frac32 * r, "xu_frac": fracxu * r}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="C2", choices=["C1", "C2", "C3", "C5"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the C4 serving measurement")
    ap.add_argument("--no-legs", action="store_true", help="skip the C1/C3/C5 and C++ drop-in measurements")
    return ap.parse_args()


from diffrg_gb300.replicas import aggregate_rate, dist_env, max_over_ranks  # noqa: E402


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=2)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(w, W, reps=2):
    """The FP64 oracle (C++ restatement of the reference CPU integrators) on all host cores."""
    from oracle import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    W.oracle_values(w, O, threads=threads, subset=np.arange(4))  # warm caches
    n = len(w["p"]) if "p" in w else len(w["P"])
    t0 = time.perf_counter()
    for _ in range(reps):
        ref = W.oracle_values(w, O, threads=threads)
    dt = (time.perf_counter() - t0) / reps
    return ref, {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
                 "sample": "the whole %s workload (%d integrals), %d repetitions, FP64 OpenMP over integrals"
                           % (w["name"], n, reps)}


def workload_name(name):
    """The workload label both arms print in config.workload."""
    return {"C1": "C1 d=4 loop: 64 p x 64 q x 32 cos",
            "C2": "C2 finite-T 3+1D loop: 3 T x 128 p, n=-64..64 x 64 q x 32 cos",
            "C3": "C3 4096 uneven 3D loops, GL orders 16..256 per axis",
            "C5": "C5 4D vertex loop: 128 x (128 q x 64 cos1 x 32 cos2 x 16 phi)"}.get(name, name)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from diffrg_gb300 import workloads as W
    from oracle import oracle as O

    O.build()
    w = getattr(W, args.workload.lower())()
    threads = os.cpu_count() or 1
    n = len(w["p"]) if "p" in w else len(w["P"])
    # each step: the whole workload (all integrals), as the GPU arm's step
    sub = np.arange(n)
    for _ in range(max(1, args.warmup)):
        W.oracle_values(w, O, threads=threads, subset=sub[:8])
    t0 = time.perf_counter()
    for _ in range(args.steps):
        W.oracle_values(w, O, threads=threads, subset=sub)
    dt = time.perf_counter() - t0
    value = sub.size * args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": workload_name(args.workload), "integrals_per_step": int(sub.size),
                       "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "all %d %s integrals per step, FP64 restatement of the reference CPU "
                                       "integrators, OpenMP over integrals" % (n, args.workload)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def workload_leg(name, ctx, stream, flush, steps, warmup, oracle_threads):
    """One further workload (C1, C3, C5) measured the way the headline is: `value` = fused FP32C
    integrals/s with inputs resident in HBM (CUDA events, L2 flushed between steps), `e2e` = the
    same through the C ABI with the tables uploaded from pinned host memory and the results read
    back every step; the reference-pattern FP64 GPU path; max/median relative error of every
    integral of the workload against the FP64 oracle."""
    import ctypes as C

    import torch

    from diffrg_gb300 import capi
    from diffrg_gb300 import workloads as W

    L = capi.lib()
    sh = stream.cuda_stream
    w = getattr(W, name.lower())()
    items, tabs = W.engine_items(w)
    n_int = len(items)
    T = [ctx.table(sp, d) for sp, d in tabs]
    ctx.autotune(items, T, "fp32c")
    tune = ctx.tune_report()
    b32 = ctx.batch(items, T, "fp32c")
    points = b32.points
    for _ in range(warmup):
        b32.run(stream=sh)
    torch.cuda.synchronize()
    per = []
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b32.run(stream=sh)
        e1.record(stream)
        per.append((e0, e1))
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in per]
    res32 = b32.results(stream=sh)
    pinned = [torch.from_numpy(np.ascontiguousarray(d, dtype=np.float32)).pin_memory() for _, d in tabs]
    host_out = torch.zeros(n_int, dtype=torch.float64).pin_memory()

    def e2e_step():
        for t, pt in zip(T, pinned):
            ctx.check(L.gb_table_update(ctx.h, t.h, C.cast(pt.data_ptr(), C.POINTER(C.c_float)), C.c_void_p(sh)))
        ctx.check(L.gb_batch_run_graph(ctx.h, b32.h, C.c_void_p(sh)))
        ctx.check(L.gb_batch_results(ctx.h, b32.h, C.cast(host_out.data_ptr(), C.POINTER(C.c_double)), C.c_void_p(sh)))

    for _ in range(warmup):
        e2e_step()
    torch.cuda.synchronize()
    lat = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        e2e_step()
        lat.append(time.perf_counter() - s0)
    b64 = ctx.batch(items, T, "fp64")
    b64.run_plain(16)  # warm-up
    t0 = time.perf_counter()
    resp = b64.run_plain(16)
    plain_dt = time.perf_counter() - t0
    out = {"workload": workload_name(name), "integrals_per_step": n_int, "points_per_step": points,
           "value": n_int / (statistics.mean(ms) / 1e3), "unit": UNIT, "ms_per_step": statistics.mean(ms),
           "steps": steps, "e2e": {"value": n_int / statistics.mean(lat), "unit": UNIT,
                                   "h2d_bytes_per_step": sum(pt.numel() * 4 for pt in pinned),
                                   "d2h_bytes_per_step": n_int * 8},
           "plain_fp64_gpu": {"value": n_int / plain_dt, "unit": UNIT, "ms_per_step": plain_dt * 1e3}}
    out["fp32c_over_plain_fp64"] = out["value"] / out["plain_fp64_gpu"]["value"]
    out["autotune"] = tune
    if name in PER_POINT:
        F, S = PER_POINT[name]
        out["per_point"] = {"F": F, "S": S}
    if oracle_threads:
        from oracle import oracle as O

        O.build()
        t0 = time.perf_counter()
        ref = W.oracle_values(w, O, threads=oracle_threads)
        cpu_dt = time.perf_counter() - t0
        e = np.abs(res32 - ref) / np.abs(ref)
        ep = np.abs(resp - ref) / np.abs(ref)
        out["accuracy"] = {"fp32c_max_rel_err_vs_oracle": float(e.max()), "fp32c_median_rel_err": float(np.median(e)),
                           "plain_fp64_max_rel_err_vs_oracle": float(ep.max()), "integrals_checked": int(n_int)}
        out["cpu_oracle"] = {"value": n_int / cpu_dt, "unit": UNIT, "cores": oracle_threads, "kind": "port"}
    b32.close()
    b64.close()
    for t in T:
        t.close()
    return out


def cpp_dropin(steps):
    """The C++ drop-in path on a generator-layout flow (diffrg_gb300/bench/dropin_bench.cu): a
    seven-table vertex loop through IntegratorAngleGPU::request over 128 external momenta, batched
    (get_data: one persistent launch), one launch per request, and the reference's execution
    pattern (per-integral kernel, thrust::reduce when the future is read)."""
    from diffrg_gb300 import cppapi

    exe = cppapi.build_dropin_bench()
    r = subprocess.run([exe, str(max(3, steps)), "3"], capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        return {"error": (r.stdout + r.stderr)[-500:]}
    return json.loads(r.stdout.strip().splitlines()[-1])


def serving_c4(device):
    """C4: one Cash-Karp step (6 right-hand sides x 4096 integrals) of the served flow, with
    Poisson arrivals at 2000 integrals/s and saturated (each evaluation submitted at once);
    latency = submit -> result ready, from the library's request loop."""
    from diffrg_gb300 import serving as SV
    from diffrg_gb300.engine import Context

    w = SV.c4()
    ctx = Context(device)
    ctx.serve_start(8, 2048)
    f = SV.Flow(ctx, w, rate=None)
    f.integrals_at(0.0, w["y0"])  # warm-up: arenas, quadrature axes
    out = {"workload": "C4 served RK45 (Cash-Karp) flow: 32 dressing functions x 128 p, requests of 8-2048 "
                       "integrals (2D PROP1 / 3D PROP3, GL orders 32-128 per axis), tables updated every stage",
           "integrals_per_rhs": w["integrals_per_rhs"], "points_per_rhs": w["points_per_rhs"],
           "max_inflight_batches": 8, "max_batch_items": 2048}

    def one_step(rate):
        f.rate = rate
        ctx.reset_stats()
        r0, i0 = f.requests, f.integrals
        t0 = time.perf_counter()
        SV.cash_karp_step(f.rhs, 0.0, w["y0"].copy(), 0.2)
        wall = time.perf_counter() - t0
        st = ctx.stats()
        return {"requests": f.requests - r0, "integrals": f.integrals - i0, "wall_s": wall,
                "integrals_per_s": (f.integrals - i0) / wall, "p50_ms": st["p50_latency_s"] * 1e3,
                "p99_ms": st["p99_latency_s"] * 1e3, "max_ms": st["max_latency_s"] * 1e3,
                "batches": st["batches_launched"], "gpu_busy_frac": st["busy_seconds"] / wall,
                "rejected": st["rejected"]}

    out["saturated"] = one_step(None)
    out["poisson"] = one_step(w["rate"])
    out["poisson"]["offered_integrals_per_s"] = w["rate"]
    out["head_of_line"] = head_of_line(ctx, f.tlist, w, "fp32c")
    # the reference's pattern on the same integrals: one launch + CUB + sync per integral
    b = ctx.batch(SV.rhs_items(w, 1.0), f.tlist, "fp64")
    b.run_plain(16)
    t0 = time.perf_counter()
    b.run_plain(16)
    out["plain_fp64_integrals_per_s"] = b.n / (time.perf_counter() - t0)
    out["saturated_over_plain_fp64"] = out["saturated"]["integrals_per_s"] / out["plain_fp64_integrals_per_s"]
    b.close()
    f.close()
    ctx.close()
    out["fp64_loops"] = serving_loops(device)
    return out


def head_of_line(ctx, tlist, w, precision, reps=20):
    """Latency of a small request (8 2D integrals) submitted right behind a large one (2048 3D
    integrals, the largest request size of C4) against the same small request alone: what a
    small request pays for arriving while the GPU is full of another's work."""
    from diffrg_gb300 import serving as SV

    items = SV.rhs_items(w, 1.0)
    per = len(w["p"])
    big = [items[i * per + j] for i in range(1, SV.N_FUNC, 2) for j in range(per)][:2048]
    probe = items[:8]

    def lat(with_big):
        v = []
        for _ in range(reps):
            tb = ctx.submit(big, tlist, precision) if with_big else None
            t0 = time.perf_counter()
            ctx.submit(probe, tlist, precision).wait(timeout=300)
            v.append((time.perf_counter() - t0) * 1e3)
            if tb is not None:
                tb.wait(timeout=300)
        v.sort()
        return {"p50_ms": v[len(v) // 2], "max_ms": v[-1]}

    lat(False)  # warm: axes of both sizes
    lat(True)
    t0 = time.perf_counter()
    ctx.submit(big, tlist, precision).wait(timeout=300)
    return {"precision": precision, "probe_integrals": len(probe), "large_integrals": len(big), "reps": reps,
            "large_alone_ms": (time.perf_counter() - t0) * 1e3,
            "probe_alone": lat(False), "probe_behind_large": lat(True)}


def serving_loops(device):
    """One C4 right-hand side (4096 integrals, 1.12e9 points) in FP64 through the host dispatcher
    (gb_serve_start) and through the device-resident loop (gb_serve_start_device), saturated and
    with Poisson arrivals at 2000 integrals/s.  Both loops see the same request sizes and arrival
    times (same seed); latency = submit -> result in host memory."""
    from diffrg_gb300 import serving as SV
    from diffrg_gb300.engine import Context

    w = SV.c4()
    out = {"workload": "C4 right-hand side in FP64 (4096 integrals in requests of 8-2048), same sizes and "
                       "arrival times for both loops", "precision": "fp64"}
    vals = {}
    for name in ("host", "device"):
        ctx = Context(device)
        f = None
        try:
            if name == "host":
                ctx.serve_start(8, 2048)
            else:
                ctx.serve_start_device(ring_slots=16, max_items=2048, max_units=1 << 21, idle_seconds=0.05)
            f = SV.Flow(ctx, w, precision="fp64", rate=None)
            f.integrals_at(0.0, w["y0"])  # warm-up: arenas, quadrature axes, module load
            res = {}
            for mode, rate in (("saturated", None), ("poisson", w["rate"])):
                f.rate = rate
                f.rng = np.random.default_rng(SV.SEEDS["C4"] + 11)
                ctx.reset_stats()
                t0 = time.perf_counter()
                v = f.integrals_at(0.0, w["y0"])
                wall = time.perf_counter() - t0
                st = ctx.stats()
                res[mode] = {"requests": st["completed"], "wall_s": wall, "integrals_per_s": v.size / wall,
                             "p50_ms": st["p50_latency_s"] * 1e3, "p99_ms": st["p99_latency_s"] * 1e3,
                             "max_ms": st["max_latency_s"] * 1e3}
                vals[(name, mode)] = v.ravel()
            res["head_of_line"] = head_of_line(ctx, f.tlist, w, "fp64", reps=5)
            if name == "device":
                res["loop"] = ctx.device_loop_info()
            out[name] = res
        finally:
            if f is not None:
                f.close()
            ctx.close()
    a, b = vals[("host", "poisson")], vals[("device", "poisson")]
    out["device_vs_host_max_rel_diff"] = float(np.max(np.abs(a - b) / np.abs(a)))
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank, world, local = dist_env()
    import torch

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    from diffrg_gb300 import build as B
    from diffrg_gb300 import capi
    from diffrg_gb300 import workloads as W
    from diffrg_gb300.engine import Context

    B.build()
    import ctypes as C

    w = getattr(W, args.workload.lower())()
    items, tabs = W.engine_items(w)
    n_int = len(items)
    ctx = Context(local)
    L = capi.lib()
    T = [ctx.table(s, d) for s, d in tabs]
    # CTA widths of the FP32-compensated kernels for this GPU and workload (library autotuner)
    tuned = ctx.autotune(items, T, "fp32c")
    tune_report = ctx.tune_report()
    b32 = ctx.batch(items, T, "fp32c")
    b64 = ctx.batch(items, T, "fp64")
    points = b32.points
    # a dedicated (non-default) stream: the library launches on exactly this stream, so the CUDA
    # events recorded on it bracket the kernels (handle 0 would mean "the context's own stream")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    assert sh != 0
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2 (129 MB)
    # one step captured as a CUDA graph: its kernel nodes are the launches per step (the
    # hoisted-factor kernel + one fused persistent kernel per item kind)
    step_graph = ctx.capture(lambda: b32.run(stream=sh), stream=sh)
    launches_per_step = step_graph.kernel_launches

    def timed(batch, steps, warm, graph=None):
        run = (lambda: graph.replay(stream=sh)) if graph else (lambda: batch.run(stream=sh))
        for _ in range(warm):
            run()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for i in range(steps):
            flush.zero_()
            ev[i][0].record(stream)
            run()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        per = [a.elapsed_time(b) for a, b in ev]
        return per

    # ---------------------------------------------------------------- main (device-resident) timing
    sampler = ClockSampler(local)
    sampler.start()
    per32 = timed(b32, args.steps, args.warmup)
    clocks = sampler.stop()
    tot = max_over_ranks(sum(per32) / 1e3, device="cuda")
    value = aggregate_rate(n_int, args.steps, world, tot)
    res32 = b32.results(stream=sh)

    # ---------------------------------------------------------------- e2e through the public API
    # every step: dressing table H2D from pinned host memory (RG-step update), fused run, results D2H
    pinned = [torch.from_numpy(np.ascontiguousarray(d, dtype=np.float32)).pin_memory() for _, d in tabs]
    host_out = torch.zeros(n_int, dtype=torch.float64).pin_memory()
    h2d = sum(p.numel() * 4 for p in pinned)
    d2h = n_int * 8

    def e2e_step():
        for t, p in zip(T, pinned):
            ctx.check(L.gb_table_update(ctx.h, t.h, C.cast(p.data_ptr(), C.POINTER(C.c_float)), C.c_void_p(sh)))
        # the batch's fixed sweep replays as a CUDA graph (captured on first use); the tables it
        # reads were updated just before, as for every right-hand side of a time stepper
        ctx.check(L.gb_batch_run_graph(ctx.h, b32.h, C.c_void_p(sh)))
        ctx.check(L.gb_batch_results(ctx.h, b32.h, C.cast(host_out.data_ptr(), C.POINTER(C.c_double)), C.c_void_p(sh)))

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    lat = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        e2e_step()
        lat.append(time.perf_counter() - s0)
    e2e_total = sum(lat)
    e2e_value = aggregate_rate(n_int, args.steps, world, max_over_ranks(e2e_total, device="cuda"))

    # ---------------------------------------------------------------- the same step replayed as a graph
    per_graph = timed(b32, args.steps, args.warmup, graph=step_graph)
    graph_value = n_int / (statistics.mean(per_graph) / 1e3)
    step_graph.close()

    # ---------------------------------------------------------------- fused FP64 and plain FP64 paths
    per64 = timed(b64, max(3, args.steps // 4), 2)
    fused64 = n_int / (statistics.mean(per64) / 1e3)
    res64 = b64.results(stream=sh)
    plain = None
    if not args.no_plain:
        b64.run_plain(16)  # warm-up (allocations, CUB)
        reps = 2
        t0 = time.perf_counter()
        for _ in range(reps):
            resp = b64.run_plain(16)
        plain_dt = (time.perf_counter() - t0) / reps
        plain = {"value": n_int / plain_dt, "unit": UNIT, "ms_per_step": plain_dt * 1e3,
                 "pattern": "one launch per integral writing one FP64 value per point, CUB DeviceReduce, "
                            "D2H + stream sync per integral, 16 pooled streams"}

    # ---------------------------------------------------------------- single-integral request latency
    single = ctx.batch(items[:1], T, "fp32c")
    one = np.zeros(1)
    for _ in range(5):
        single.get()
    sl = []
    for _ in range(50):
        s0 = time.perf_counter()
        single.get()
        sl.append(time.perf_counter() - s0)
    single.close()

    # ---------------------------------------------------------------- roofline
    fp32_peak, mufu_peak, fp64_peak = ctx.measure_peaks()
    pts_per_s = points / (statistics.mean(per32) / 1e3)
    flops_pp, specials_pp = PER_POINT[args.workload]
    fp32_achieved = flops_pp * pts_per_s / 1e12
    xu_achieved = specials_pp * pts_per_s / 1e9
    frac32 = fp32_achieved / fp32_peak
    fracxu = xu_achieved / mufu_peak
    traffic = TRAFFIC_BYTES_PER_LAUNCH.get(args.workload)
    roof = {"bound": "xu" if fracxu >= frac32 else "fp32",
            "achieved": xu_achieved if fracxu >= frac32 else fp32_achieved,
            "peak": mufu_peak if fracxu >= frac32 else fp32_peak,
            "unit": "Gop/s" if fracxu >= frac32 else "TFLOP/s",
            "frac": max(frac32, fracxu), "traffic": traffic, "traffic_source": CAPTURE_NOTE,
            "fp32": {"achieved": fp32_achieved, "peak": fp32_peak, "unit": "TFLOP/s", "frac": frac32},
            "xu": {"achieved": xu_achieved, "peak": mufu_peak, "unit": "Gop/s", "frac": fracxu},
            "per_point": {"F": flops_pp, "S": specials_pp},
            "points_per_launch": points,
            "evaluated": evaluated_block(w, points, frac32, fracxu),
            "peak_source": "measured in this run by the library's FFMA/MUFU probes (gb_measure_peaks); "
                           "MEASURED_PEAKS.json lists only HBM and BF16",
            "fp64_peak_tflops": fp64_peak}
    ipp = INSTR_PER_POINT.get(args.workload)
    sm_mhz = clocks.get("sm_mhz") or 0
    if ipp and sm_mhz:
        import ctypes as _C

        dev, nsm = _C.c_int(), _C.c_int()
        L.gb_device_info(ctx.h, _C.byref(dev), _C.byref(nsm))
        issue_peak = nsm.value * 4 * sm_mhz * 1e6 / 1e9  # G warp instructions/s
        issue_achieved = ipp * pts_per_s / 32 / 1e9
        roof["issue"] = {"achieved": issue_achieved, "peak": issue_peak, "unit": "G warp-instr/s",
                         "frac": issue_achieved / issue_peak, "instr_per_point": ipp,
                         "note": "executed double-float instructions (ncu count per point) at the sampled SM clock"}

    # ---------------------------------------------------------------- accuracy + CPU baseline
    cpu = None
    err = None
    if rank == 0 and not args.no_cpu:
        ref, cpu = cpu_baseline(w, W)
        e = np.abs(res32 - ref) / np.abs(ref)
        e64 = np.abs(res64 - ref) / np.abs(ref)
        err = {"fp32c_max_rel_err_vs_oracle": float(e.max()), "fp32c_median_rel_err": float(np.median(e)),
               "fp64_fused_max_rel_err_vs_oracle": float(e64.max())}
        if plain is not None:
            err["plain_fp64_max_rel_err_vs_oracle"] = float((np.abs(resp - ref) / np.abs(ref)).max())

    serve = None if args.no_serve else serving_c4(local)

    # ---------------------------------------------------------------- the other workloads, C++ drop-in path
    legs = {}
    if not args.no_legs:
        for other in ("C1", "C3", "C5"):
            if other != args.workload:
                legs[other] = workload_leg(other, ctx, stream, flush, max(3, min(args.steps, 10)), 3,
                                           (os.cpu_count() or 1) if (rank == 0 and not args.no_cpu) else 0)
    dropin = None if args.no_legs else cpp_dropin(min(args.steps, 20))

    lat_ms = sorted(x * 1e3 for x in lat)
    sl_ms = sorted(x * 1e3 for x in sl)

    def pct(v, q):
        return v[min(len(v) - 1, int(round(q * (len(v) - 1))))]

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.mean(per32), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (compensated) + f64 reduction",
            "data": "synthetic (seeded tables and momenta, no dataset)",
            "config": {"workload": workload_name(args.workload),
                       "integrals_per_step": n_int, "points_per_step": points,
                       "l2": "flushed between steps (256 MiB write)", "parallelism": "replicas" if world > 1 else "1 GPU"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clocks,
            "roofline": roof,
            "plain_fp64_gpu": plain,
            "fp32c_over_plain_fp64": (value / world) / plain["value"] if plain else None,
            "fused_fp64_gpu": {"value": fused64, "unit": UNIT},
            "graph_replay": {"value": graph_value * world, "unit": UNIT, "ms_per_step": statistics.mean(per_graph),
                             "kernel_launches_per_step": launches_per_step},
            "latency_ms": {"batch_e2e_p50": pct(lat_ms, 0.5), "batch_e2e_p99": pct(lat_ms, 0.99),
                           "single_integral_get_p50": pct(sl_ms, 0.5), "single_integral_get_p99": pct(sl_ms, 0.99)},
            "accuracy": err,
            "autotune": {"cta_threads_by_kind_slot": tuned, "report": tune_report},
            "serving": serve,
            "workloads": legs,
            "cpp_dropin": dropin,
            "cpu_baseline": cpu}
    if serve:
        line["latency_ms"]["serving_c4_p50"] = serve["poisson"]["p50_ms"]
        line["latency_ms"]["serving_c4_p99"] = serve["poisson"]["p99_ms"]
    if rank == 0:
        print(json.dumps(line))
    b32.close()
    b64.close()
    for t in T:
        t.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
