"""Benchmark: batched stochastic KPM moments on one GB300 (and N replicas under torchrun).

Workload (default): 32 Anderson-disordered graphene flakes of uneven size
(sites drawn uniformly in [50k, 400k], onsite energies uniform in
[-0.5, 0.5] eV), 64 Rademacher starters per flake, 4096 moments (rounded to
4098 as the reference does), FP32 recursion vectors with FP64 moment sums,
spectral bounds by FP64 Lanczos. All flakes and vectors advance together:
every Chebyshev step is one kernel launch over the block-diagonal matrix.

A step = the full moment computation of the workload (init + 2048 recursion
launches + collection). Metric: Gnnz*vec/s = (M/2) * nnz * vectors / time,
the unit of the reference's Stats::eps (cppcore/src/kpm/Stats.cpp:49-51)
times the vector count. Inputs are larger than L2 (vector blocks ~1.8 GB), so
no explicit L2 flush is needed between steps.

`--impl reference` times the reference's CPU algorithm (the oracle's
multithreaded restatement of DefaultCompute: ELL, interleaved recursion,
8-vector batches, one thread per core) on a bounded sample of the same
workload, on rank 0.
"""
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

METRIC = "KPM Gnnz*vec/s (batched FP32 recursion, FP64 moment sums; moment err vs FP64 stated)"
UNIT = "Gnnz*vec/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--flakes", type=int, default=32)
    p.add_argument("--vectors", type=int, default=64)
    p.add_argument("--moments", type=int, default=4096)
    p.add_argument("--min-sites", type=int, default=50_000)
    p.add_argument("--max-sites", type=int, default=400_000)
    p.add_argument("--seed", type=int, default=1234)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-error", action="store_true", help="skip the FP64 moment-error check")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of one CPU sample")
    return p.parse_args()


def build_workload(args, rank):
    from pybinding_gb300 import lattice as L
    import scipy.sparse as sp
    rng = np.random.default_rng(args.seed + 1000 * rank)
    sizes = rng.integers(args.min_sites, args.max_sites + 1, size=args.flakes)
    hs = []
    for i, n in enumerate(sizes):
        m = L.graphene_flake(int(n), onsite_modifiers=[L.anderson_disorder(1.0, args.seed + 7919 * i + rank)])
        hs.append(m.hamiltonian)
    offsets = np.concatenate([[0], np.cumsum([h.shape[0] for h in hs])]).astype(np.int64)
    h = sp.block_diag(hs, format="csr").astype(np.float32)
    h.sort_indices()
    return hs, h, offsets


def rademacher(rng, n):
    return np.where(rng.integers(0, 2, size=n, dtype=np.int8) == 0, -1.0, 1.0).astype(np.float32)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

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
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def cpu_reference(hs, args, threads, target_seconds, seed):
    """Time the oracle's multithreaded DefaultCompute restatement on one flake of the workload."""
    from oracle import oracle as O
    # the flake closest to the mean size, its own Lanczos-free bounds (the bench's scale is per flake)
    sizes = np.array([h.shape[0] for h in hs])
    h = hs[int(np.argmin(np.abs(sizes - sizes.mean())))].astype(np.float32)
    a, b = O.scale(-9.0, 9.0)
    r = O.optimize(h, [0], [0], a, b)
    n = h.shape[0]
    k = 8
    R = k * threads
    rng = np.random.default_rng(seed)
    st = np.stack([rademacher(rng, n) for _ in range(R)])
    st = O.reorder_vector(st, r["reorder_map"])
    nnz = h.nnz
    # calibrate: a short run, then size M for about target_seconds
    M0 = 34
    _, sec0 = O.bench_diag(r["h2"], r["slices"], st, M0, k, threads)
    rate = (M0 / 2) * nnz * R / sec0
    steps = max(8, int(target_seconds * rate / (nnz * R)))
    M = O.round_num_moments(2 * steps)
    _, sec = O.bench_diag(r["h2"], r["slices"], st, M, k, threads)
    work = (M / 2) * nnz * R
    return dict(value=work / sec / 1e9, seconds=sec, M=M, R=R, n=n, nnz=nnz,
                sample="one %d-site flake of the workload (nnz %d), %d Rademacher vectors in %d-vector batches, "
                       "%d moments, ELL interleaved, %d threads" % (n, nnz, R, k, M, threads))


def run_reference(args, rank, world):
    if rank != 0:
        return
    hs, _, _ = build_workload(args, 0)
    threads = os.cpu_count() or 1
    vals = []
    last = None
    for i in range(args.warmup + args.steps):
        res = cpu_reference(hs, args, threads, args.cpu_seconds / 2, args.seed + i)
        if i >= args.warmup:
            vals.append(res["value"])
            last = res
    v = float(np.median(vals))
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": last["seconds"] * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
           "config": workload_config(args, hs),
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": last["sample"]},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def workload_config(args, hs):
    return {"workload": "batched stochastic DOS moments: %d disordered graphene flakes U[%d,%d] sites, "
                        "%d Rademacher vectors each, %d moments" % (args.flakes, args.min_sites, args.max_sites,
                                                                    args.vectors, args.moments),
            "flakes": args.flakes, "sites": int(sum(h.shape[0] for h in hs)),
            "nnz": int(sum(h.nnz for h in hs)), "vectors_per_flake": args.vectors,
            "moments": int(args.moments + ((4 - (args.moments - 2) % 4) % 4)),
            "recursion": "fp32 vectors, fp64 moment sums", "bounds": "fp64 Lanczos per flake",
            "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas" if args.gpus > 1 else "single"}


def run_gpu(args, rank, world, local_rank):
    import torch
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    from pybinding_gb300 import _native
    hs, h, offsets = build_workload(args, rank)
    nsys = len(hs)
    rows = h.shape[0]
    R = args.vectors
    rng = np.random.default_rng(args.seed + 17 + rank)
    starters = np.empty((R * rows,), np.float32)
    pos = 0
    for hh in hs:  # [system][vector][site]
        n = hh.shape[0]
        for _ in range(R):
            starters[pos:pos + n] = rademacher(rng, n)
            pos += n
    cfg = _native.make_config()  # Lanczos bounds, Jackson, auto precision (fp32 vectors for an f32 H)
    eng = _native.Engine(h, cfg, system_offsets=offsets)
    for s in range(nsys):
        eng.scaling_factors(s)
    stream = torch.cuda.ExternalStream(eng.stream())
    d_st = torch.from_numpy(starters).cuda()
    torch.cuda.synchronize()

    def step_device():
        return eng.moments_diag(args.moments, None, average=True, on_device_ptr=d_st.data_ptr(), num_vectors=R)

    for _ in range(args.warmup):
        step_device()
    M = eng.stats().num_moments
    nnz = int(h.nnz)
    work = (M / 2) * nnz * R  # nnz*vec per step
    clocks = ClockSampler(local_rank)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    rec_times = []
    for _ in range(args.steps):
        step_device()
        rec_times.append(eng.stats().moments_time)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    t = e0.elapsed_time(e1) * 1e-3
    if dist is not None:
        tt = torch.tensor([t], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    value = world * work * args.steps / t / 1e9

    # dominant kernel: the recursion step, timed by the engine's events on its own stream
    rec = float(np.median(rec_times))
    fuse = int(eng.stats().steps_per_launch)
    launches = 1 + (M // 2 - 1) // fuse  # init + recursion launches
    avg_launch = rec / launches
    nrows = rows
    # per launch: matrix once (FP32 hi/lo value pair + int32 column per non-zero, row extents);
    # one step reads x and y_old and writes y_new (3 vector passes), a fused two-step launch
    # reads P and Q and writes both (4 vector passes for 2 steps)
    vec_bytes = (3 if fuse == 1 else 4) * nrows * R * 4
    alg_bytes = nnz * (8 + 4) + 4 * (nrows + 1) + vec_bytes
    achieved = alg_bytes / avg_launch / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = None
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "diag_step_traffic.json")))
        if prof.get("steps_per_launch", 1) == fuse:
            traffic = prof.get("dram_bytes_per_launch_scaled_to_bench")
    except (OSError, ValueError):
        pass

    e2e = None
    if not args.no_e2e:
        import torch as _t
        pinned = _t.empty(starters.size, dtype=_t.float32, pin_memory=True)
        pinned.numpy()[:] = starters
        host = pinned.numpy()
        eng.moments_diag(args.moments, host, average=True)  # warm the staging buffers
        barrier()
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.steps):
            eng.moments_diag(args.moments, host, average=True)
        f1.record(stream)
        torch.cuda.synchronize()
        barrier()
        te = max(f0.elapsed_time(f1) * 1e-3, time.perf_counter() - w0)
        if dist is not None:
            tt = torch.tensor([te], device="cuda")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            te = float(tt.item())
        e2e = {"value": world * work * args.steps / te / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": int(starters.nbytes), "d2h_bytes_per_step": int(nsys * M * 16)}

    err = None
    if not args.no_error:
        m32 = eng.moments_diag(args.moments, None, average=False, on_device_ptr=d_st.data_ptr(), num_vectors=R)
        eng.close()
        cfg64 = _native.make_config(precision="fp64")
        e64 = _native.Engine(h, cfg64, system_offsets=offsets)
        m64 = e64.moments_diag(args.moments, None, average=False, on_device_ptr=d_st.data_ptr(), num_vectors=R)
        e64.close()
        # per-vector moments, and the stochastic-trace moments (average over the vectors of a
        # flake, as the reference's BatchAccumulator returns them), each relative to its max |mu|
        err = {"per_vector_max": float(np.max(np.abs(m32 - m64)) / np.max(np.abs(m64))),
               "vector_averaged_max": float(np.max(np.abs(m32.mean(1) - m64.mean(1))) / np.max(np.abs(m64.mean(1))))}
    else:
        eng.close()

    cpu = None
    if rank == 0:
        cpu = cpu_reference(hs, args, os.cpu_count() or 1, args.cpu_seconds, args.seed)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": workload_config(args, hs),
               "moment_error_vs_fp64": err,
               "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": traffic,
                            "kernel": "diag_step_kernel<float,4,16>" if fuse == 1 else "diag_pair_kernel<float,4,16>",
                            "steps_per_launch": fuse, "alg_bytes_per_launch": alg_bytes,
                            "avg_launch_ms": avg_launch * 1e3, "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
               "cpu_baseline": {"value": cpu["value"], "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                "sample": cpu["sample"]},
               "e2e": e2e,
               "clocks": clk,
               "gpu_launches": int(args.steps * (launches + 3))}
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
