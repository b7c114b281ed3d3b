"""Benchmark of the headline workload: LSD radix sort of 2^28 uint32 keys +
uint32 values (uniform 32-bit keys, values = index) on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

One step = one in-place radix sort of 2^28 key/value pairs through the C ABI
(mgpu_radix_sort).  Before each step a device copy restores an unsorted input
(outside the step's CUDA event pair); the input is 2 GiB (> L2), so no L2
flush is needed.  `value` is device throughput (Mkeys/s from the mean of the
per-step event times); `e2e` is the same metric through the C ABI with the
keys/values starting and ending in pinned host memory.
`roofline` covers the dominant kernel (onesweep_pass): 16 algorithmic bytes
per key per launch, divided by its mean event-timed duration.

--impl reference times the CPU implementation of the same sort (the host
oracle's parallel stable sort by radix bits over all host threads; the
reference itself is Circle/Vulkan shaders and cannot run on this machine) on a
bounded sample of the workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "mgpu-shaders_gb300"))
sys.path.insert(0, REPO)

N_KEYS = 1 << 28
SEED = 0x6D677075 + 2
METRIC = "Mkeys/s (2^28 u32 key + u32 value radix sort)"
ALG_BYTES_PER_KEY = 68          # 4 passes x (4+4 read + 4+4 write) + 4 histogram read
PASS_BYTES_PER_KEY = 16         # one onesweep_pass launch
CPU_SAMPLE = 1 << 24


def config(dist="uniform"):
    return {
        "workload": "radix_sort_kv u32 keys + u32 values, 2^28, %s 32-bit keys" % dist,
        "count": N_KEYS,
        "key_dtype": "u32",
        "val_dtype": "u32",
        "digit_bits": 8,
        "l2": "inputs larger than L2 (2 GiB unsorted input restored before each step, "
              "outside the step's events)",
        "seed": SEED,
    }


def make_input(n, dist="uniform", seed=SEED):
    rng = np.random.default_rng(seed)
    if dist == "uniform":
        k = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    elif dist == "and2":
        k = (rng.integers(0, 2 ** 32, n, dtype=np.uint64) &
             rng.integers(0, 2 ** 32, n, dtype=np.uint64)).astype(np.uint32)
    else:
        table = rng.integers(0, 2 ** 32, 256, dtype=np.uint64).astype(np.uint32)
        k = table[rng.integers(0, 256, n)]
    return k, np.arange(n, dtype=np.uint32)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join(REPO, "gpurun_out", "clocks_bench.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_baseline(threads, sample=CPU_SAMPLE, min_seconds=10.0, max_reps=8):
    """The host oracle's parallel stable radix-order sort on `sample` keys,
    repeated until about min_seconds of CPU work; Mkeys/s (median)."""
    from oracle import oracle
    k0, v0 = make_input(sample)
    rates = []
    t_total = 0.0
    while len(rates) < max_reps and (t_total < min_seconds or len(rates) < 3):
        k = k0.copy()
        v = v0.copy()
        t = time.perf_counter()
        oracle.sort_parallel_inplace(k, v, "radix", threads)
        dt = time.perf_counter() - t
        t_total += dt
        rates.append(sample / dt / 1e6)
    return statistics.median(rates), len(rates)


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    from oracle import oracle
    k0, v0 = make_input(CPU_SAMPLE)
    for _ in range(args.warmup):
        k, v = k0.copy(), v0.copy()
        oracle.sort_parallel_inplace(k, v, "radix", threads)
    times = []
    for _ in range(args.steps):
        k, v = k0.copy(), v0.copy()
        t = time.perf_counter()
        oracle.sort_parallel_inplace(k, v, "radix", threads)
        times.append(time.perf_counter() - t)
    value = CPU_SAMPLE * len(times) / sum(times) / 1e6
    sample = "%d-key sample of the workload per step (same generator and seed)" % CPU_SAMPLE
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mkeys/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": config(),
        "cpu_baseline": {"value": value, "unit": "Mkeys/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "Mkeys/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "reference shaders need Circle + Vulkan (unavailable on this box); timed: the "
                "host oracle's std::thread stable sort by radix bits",
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mgpu", choices=["mgpu", "reference"])
    ap.add_argument("--n", type=int, default=N_KEYS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import mgpu_gb300 as mg

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist

    n = args.n
    steps, warmup = args.steps, max(3, args.warmup)
    ctx = mg.Context(local)
    keys_h, vals_h = make_input(n, seed=SEED + rank)

    # Each step sorts an unsorted 2 GiB copy (> L2), restored from the pristine
    # input by a device copy that lies outside the step's event pair.
    pristine_k = mg.DeviceArray.from_numpy(keys_h)
    pristine_v = mg.DeviceArray.from_numpy(vals_h)
    copies = [(mg.DeviceArray(n, np.uint32), mg.DeviceArray(n, np.uint32)) for _ in range(2)]

    def restore(i):
        copies[i % 2][0].copy_from(pristine_k)
        copies[i % 2][1].copy_from(pristine_v)

    aux_bytes = ctx.radix_sort_aux_size(np.uint32, np.uint32, n)
    aux_t = torch.empty(aux_bytes, dtype=torch.uint8, device="cuda")
    aux = (aux_t.data_ptr(), aux_bytes)

    for w in range(warmup):
        restore(w)
        ctx.radix_sort(copies[w % 2][0], copies[w % 2][1], aux=aux)
    ctx.synchronize()
    torch.cuda.synchronize()

    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    launches = 0
    for i in range(steps):
        restore(i)
        ev[i][0].record(stream)
        l0 = ctx.launch_count
        ctx.radix_sort(copies[i % 2][0], copies[i % 2][1], aux=aux)
        launches += ctx.launch_count - l0
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    clk = clocks.stop()
    ctx.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = sum(step_ms) / steps
    if pg:
        t = torch.tensor([ms], device="cuda")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())

    # Correctness of the last timed output (cheap properties).
    gk = copies[(steps - 1) % 2][0].numpy()
    gv = copies[(steps - 1) % 2][1].numpy()
    ok_sorted = bool(np.all(gk[1:] >= gk[:-1])) and bool(np.array_equal(keys_h[gv], gk))

    # Per-kernel event timing for the roofline (same workload, fresh copies).
    prof_steps = min(steps, 4)
    ctx.synchronize()
    for i in range(prof_steps):
        restore(i)
        ctx.profile(True)
        ctx.radix_sort(copies[i % 2][0], copies[i % 2][1], aux=aux)
        ctx.profile(False)
    prof = ctx.profile_read()
    p_launches, p_ms = prof.get("onesweep_pass", (0, 0.0))
    pass_ms = p_ms / max(1, p_launches)
    achieved = PASS_BYTES_PER_KEY * n / (pass_ms * 1e-3) / 1e9 if pass_ms else None
    peaks_path = os.path.join(REPO, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        peak = json.load(open(peaks_path)).get("hbm_gbs", peak)
        peak_src = "measured"
    traffic = None
    tp = os.path.join(REPO, "profiles", "onesweep_pass_traffic.json")
    if os.path.exists(tp):
        t = json.load(open(tp))
        traffic = t.get("bytes_per_key", 0) * n or None

    # End to end through the C ABI: pinned host -> device, sort, device -> host.
    e2e_steps = min(steps, 3)
    hk = torch.from_numpy(keys_h).pin_memory()
    hv = torch.from_numpy(vals_h).pin_memory()
    ok_k = torch.empty_like(hk).pin_memory()
    ok_v = torch.empty_like(hv).pin_memory()
    dk, dv = copies[0]
    lib = mg.lib()
    nbytes = 4 * n
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        ctx._check(lib.mgpu_memcpy(ctx.handle, dk.ptr, hk.data_ptr(), nbytes))
        ctx._check(lib.mgpu_memcpy(ctx.handle, dv.ptr, hv.data_ptr(), nbytes))
        ctx.radix_sort(dk, dv, aux=aux)
        ctx._check(lib.mgpu_memcpy(ctx.handle, ok_k.data_ptr(), dk.ptr, nbytes))
        ctx._check(lib.mgpu_memcpy(ctx.handle, ok_v.data_ptr(), dv.ptr, nbytes))
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / e2e_steps
    e2e_ok = bool(np.array_equal(keys_h[ok_v.numpy()], ok_k.numpy()))

    value = n * world / (ms * 1e-3) / 1e6
    line = {
        "metric": METRIC, "value": value, "unit": "Mkeys/s", "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic", "config": config(),
        "gpu_launches": launches,
        "hbm_gbs_at_68B_per_key": ALG_BYTES_PER_KEY * n / (ms * 1e-3) / 1e9,
        "roofline": {"bound": "hbm", "kernel": "onesweep_pass", "achieved": achieved,
                     "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "peak_source": peak_src, "launch_ms": pass_ms,
                     "bytes_per_launch": PASS_BYTES_PER_KEY * n},
        "kernels_ms_per_step": {k: v[1] / prof_steps for k, v in prof.items()},
        "e2e": {"value": n * world / (e2e_ms * 1e-3) / 1e6, "unit": "Mkeys/s",
                "h2d_bytes_per_step": 2 * nbytes, "d2h_bytes_per_step": 2 * nbytes,
                "ms_per_step": e2e_ms},
        "clocks": clk,
        "checks": {"timed_output_sorted_stable": ok_sorted, "e2e_output": e2e_ok},
    }
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, reps = cpu_baseline(threads)
        line["cpu_baseline"] = {
            "value": v, "unit": "Mkeys/s", "cores": threads, "kind": "port",
            "sample": "%d-key sample of the same generator, %d runs (median), host oracle "
                      "std::thread stable sort by radix bits" % (CPU_SAMPLE, reps)}
    if rank == 0:
        print(json.dumps(line))
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
