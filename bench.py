"""Benchmark: batched stochastic KPM moments on one GB300 (and N replicas under torchrun).

Workload (default): 32 Anderson-disordered graphene flakes of uneven size
(sites drawn uniformly in [50k, 400k], onsite energies uniform in
[-0.5, 0.5] eV), 64 Rademacher starters per flake, 4096 moments (rounded to
4098 as the reference does), FP32 recursion vectors (row sums compensated by an
FMA per term) with FP64 moment sums,
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

`--workload` selects one of the other configurations instead (one JSON line
each, same keys; they are measurements of the other hot-path rows, not the
headline): `dos_c128_60k` (60k-site complex128 graphene DOS, 8 vectors, 2048
moments), `conductivity` (1M-site graphene at 20 T, complex128, 16 vectors,
512 x 512 moments matrix on the tensor cores), `adjoint` (256k-site strained
graphene, DOS misfit gradient, 32 vectors, 1024 moments, FP32) and
`anderson3d` (160^3 simple cubic, 256 vectors, 8192 moments, FP32, plus LDOS
at 4096 sites).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "KPM Gnnz\u00b7vec/s & HBM GB/s: batched FP32 vs plain FP64 at moment err \u22641e-6"
UNIT = "Gnnz*vec/s"


# dram__bytes_read.sum + dram__bytes_write.sum of one launch of the FP32 step with 64 vectors per
# row on the 4-flake case of the same workload: 1,070,628,096 bytes over 1,362,158 rows for
# diag_step_kernel<float,4,16> (chained FMAs); diag_step_cr_kernel<float,4,16> (compensated rows,
# the same loads and stores) measured 1,070,174,464 (ncu, one launch each)
DIAG_STEP_DRAM_BYTES_PER_ROW = 1070628096.0 / 1362158


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
    p.add_argument("--cond-sites", type=int, default=1_000_000, help="sites of the conductivity workload")
    p.add_argument("--cond-precision", default="auto", choices=["auto", "fp32"],
                   help="conductivity recursion: auto (complex128 for the complex128 H) or fp32 (complex64 "
                        "vectors; the line then also reports sigma's deviation from an FP64 run)")
    p.add_argument("--adj-sites", type=int, default=256_000, help="sites of the adjoint workload")
    p.add_argument("--cube", type=int, default=160, help="edge of the 3D Anderson cube")
    p.add_argument("--cube-vectors", type=int, default=256, help="vectors of the 3D Anderson workload")
    p.add_argument("--cube-moments", type=int, default=8192, help="moments of the 3D Anderson workload")
    p.add_argument("--ldos-sites", type=int, default=4096, help="LDOS sites of the 3D Anderson workload (0: none)")
    p.add_argument("--staging", default="auto", choices=["auto", "registers", "prefetch"],
                   help="diagonal step's matrix entries: per-row loads or staged a chunk ahead (auto = by timing)")
    p.add_argument("--precision", default="auto", choices=["auto", "fp32", "fp32p", "fp32x"],
                   help="FP32 recursion row sums: chained FMAs (fp32), compensated by an FMA per term "
                        "(fp32p = auto) or by TwoSum (fp32x)")
    p.add_argument("--fuse", type=int, default=0, choices=[0, 1, 2],
                   help="steps per launch (0 = chosen by timing)")
    p.add_argument("--adj-moments", type=int, default=1024, help="moments of the adjoint workload")
    p.add_argument("--workload", default="dos_batch",
                   choices=["dos_batch", "dos_c128_60k", "conductivity", "adjoint", "anderson3d", "lattice", "sweep"])
    p.add_argument("--sweep-models", type=int, default=32, help="models of the sweep workload")
    p.add_argument("--sweep-sites", type=int, default=100_000, help="sites per model of the sweep workload")
    p.add_argument("--lattice-sites", type=int, default=4_000_000, help="sites of the lattice-build workload")
    return p.parse_args()


def build_workload(args, rank):
    from pybinding_gb300 import lattice as L
    from pybinding_gb300.chebyshev import block_diagonal
    rng = np.random.default_rng(args.seed + 1000 * rank)
    sizes = rng.integers(args.min_sites, args.max_sites + 1, size=args.flakes)
    hs = []
    for i, n in enumerate(sizes):
        m = L.graphene_flake(int(n), onsite_modifiers=[L.anderson_disorder(1.0, args.seed + 7919 * i + rank)])
        hs.append(m.hamiltonian)
    offsets = np.concatenate([[0], np.cumsum([h.shape[0] for h in hs])]).astype(np.int64)
    h = block_diagonal([x.astype(np.float32) for x in hs])
    return hs, h, offsets


def job_rate(work, seconds, dist=None, device="cpu"):
    """Whole-job throughput of replicas: the units every rank processed over the slowest rank's
    time (ranks run different seeds, so their work differs). Returns (units/s, max seconds)."""
    if dist is None:
        return work / seconds, seconds
    import torch
    w = torch.tensor([float(work)], dtype=torch.float64, device=device)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(w.item()) / float(t.item()), float(t.item())


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


class CpuWorkload:
    """The timed CPU baseline over the whole batched workload: the oracle's restatement of the
    reference's DefaultCompute DOS path (ELL, interleaved recursion, 8-vector float batches --
    the reference's float SIMD batch on AVX, kpm/default/Compute.cpp:52-88 with
    support/simd.hpp:35-43), built -O3 with FMA contraction (and -mcpu=native on aarch64), every
    (flake, batch) pair on one pool of all host threads. Each sample runs every flake with all its
    vectors for a moment count sized to the time target: the metric is a rate, and the rate of a
    step does not depend on how many steps run."""

    K = 8

    def __init__(self, hs, vectors, seed, threads):
        from oracle import oracle as O
        self.O = O
        self.threads = threads
        self.vectors = vectors
        a, b = O.scale(-9.0, 9.0)  # timing only: one range for all flakes
        rng = np.random.default_rng(seed)
        self.systems = []
        self.nnz = 0
        for h in hs:
            r = O.optimize(h.astype(np.float32), [0], [0], a, b)
            st = np.stack([rademacher(rng, h.shape[0]) for _ in range(vectors)])
            self.systems.append((r["h2"], r["slices"], O.reorder_vector(st, r["reorder_map"])))
            self.nnz += int(h.nnz)
        self.rate = None

    def sample(self, target_seconds):
        """One timed sample of about target_seconds; returns (Gnnz*vec/s, seconds, M)."""
        O = self.O
        if self.rate is None:  # calibrate on 8 steps
            _, sec0 = O.bench_diag_multi(self.systems, 18, self.K, self.threads)
            self.rate = 9 * self.nnz * self.vectors / sec0
        steps = max(8, int(target_seconds * self.rate / (self.nnz * self.vectors)))
        M = O.round_num_moments(2 * steps)
        _, sec = O.bench_diag_multi(self.systems, M, self.K, self.threads)
        work = (M / 2) * self.nnz * self.vectors
        self.rate = work / sec
        return work / sec / 1e9, sec, M

    def describe(self, M):
        return ("all %d flakes of the workload (nnz %d), %d Rademacher vectors each in %d-vector float batches, "
                "%d moments per sample, ELL interleaved, %d threads, timed build -O3 %s" % (
                    len(self.systems), self.nnz, self.vectors, self.K, M, self.threads,
                    " ".join(self.O._fast_flags()[1:])))


def run_reference(args, rank, world):
    if rank != 0:
        return
    hs, _, _ = build_workload(args, 0)
    threads = os.cpu_count() or 1
    cpu = CpuWorkload(hs, args.vectors, args.seed, threads)
    vals = []
    last = None
    for i in range(args.warmup + args.steps):
        v, sec, M = cpu.sample(args.cpu_seconds / 2)
        if i >= args.warmup:
            vals.append(v)
            last = (sec, M)
    v = float(np.median(vals))
    cfg = workload_config(args, hs)
    cfg["sample_moments"] = int(last[1])
    cfg["recursion"] = ("the reference's CPU algorithm in its own arithmetic (the oracle's restatement of "
                        "kpm::DefaultCompute: float vectors and values, ELL, interleaved steps)")
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": last[0] * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
           "config": cfg,
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": cpu.describe(last[1])},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def oracle_check(h, a, b, starters, M, got64, got32):
    """The FP64 oracle's moments of two vectors of one flake (the CPU leg's checker): errors of
    the engine's FP64 and FP32 moments of those vectors, relative to max |mu|."""
    from oracle import oracle as O
    r = O.optimize(h.astype(np.float64), [0], [0], a, b)
    ref = O.moments_diag(r["h2"], O.reorder_vector(starters.astype(np.float64), r["reorder_map"]), M,
                         slices=r["slices"])
    scale = np.max(np.abs(ref))
    return {"fp64_vs_oracle": float(np.max(np.abs(got64 - ref)) / scale),
            "fp32_vs_oracle": float(np.max(np.abs(got32 - ref)) / scale)}


def step_kernel(stats, precision, elem="float"):
    """Name of the recursion kernel the engine ran last (its stats) for an FP32 precision mode."""
    comp = precision in ("auto", "fp32p", "fp32x") and elem == "float"
    if int(stats.steps_per_launch) == 2:
        name = "diag_pair_kernel"
    elif int(stats.prefetch):
        name = "diag_pf_kernel"
    else:
        name = "diag_step_cr_kernel" if comp else "diag_step_kernel"
    rows = {"fp32x": "TwoSum-compensated rows", "fp32": "chained-FMA rows"}.get(
        precision, "FMA-compensated rows") if elem == "float" else "FP64"
    return "%s<%s,%d,%d> (%s)" % (name, elem, int(stats.elems_per_lane), int(stats.lanes_per_row), rows)


def workload_config(args, hs):
    return {"workload": "batched stochastic DOS moments: %d disordered graphene flakes U[%d,%d] sites, "
                        "%d Rademacher vectors each, %d moments" % (args.flakes, args.min_sites, args.max_sites,
                                                                    args.vectors, args.moments),
            "flakes": args.flakes, "sites": int(sum(h.shape[0] for h in hs)),
            "nnz": int(sum(h.nnz for h in hs)), "vectors_per_flake": args.vectors,
            "moments": int(args.moments + ((4 - (args.moments - 2) % 4) % 4)),
            "recursion": "fp32 vectors, %s, fp64 moment sums" % (
                {"fp32x": "fp32 row sums compensated by TwoSum", "fp32": "fp32 row sums of chained FMAs"}.get(
                    getattr(args, "precision", "auto"), "fp32 row sums compensated by an FMA per term (auto)")),
            "bounds": "fp64 Lanczos per flake",
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
    # Lanczos bounds, Jackson, auto precision (fp32 vectors for an f32 H)
    cfg = _native.make_config(staging=args.staging, fuse_steps=args.fuse, precision=args.precision)
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
    rate, t = job_rate(work * args.steps, t, dist, "cuda")
    value = rate / 1e9

    # dominant kernel: the recursion step, timed by the engine's events on its own stream
    rec = float(np.median(rec_times))
    fuse = int(eng.stats().steps_per_launch)
    lane_map = (int(eng.stats().elems_per_lane), int(eng.stats().lanes_per_row))
    kernel_name = step_kernel(eng.stats(), args.precision)
    tiling = {"tile_rows": int(eng.stats().tile_rows), "unroll": int(eng.stats().unroll),
              "prefetch": int(eng.stats().prefetch)}
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
    # DRAM traffic per launch from an ncu capture of the same kernel and lane mapping, scaled
    # to this workload's rows (traffic grows with rows x vectors)
    traffic = DIAG_STEP_DRAM_BYTES_PER_ROW * nrows if (fuse == 1 and lane_map == (4, 16) and R == 64) else None

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
        rate_e, te = job_rate(work * args.steps, te, dist, "cuda")
        e2e = {"value": rate_e / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": int(starters.nbytes), "d2h_bytes_per_step": int(nsys * M * 16)}

    def variant(prec, elem_bytes):
        """The same workload in another recursion precision, timed on the device like `value`:
        its line entry, its per-vector moments and whether its Lanczos bounds are the same bits."""
        e = _native.Engine(h, _native.make_config(precision=prec), system_offsets=offsets)
        same = all(e.energy_bounds(s) == bounds32[s] for s in range(nsys))
        sv = torch.cuda.ExternalStream(e.stream())

        def run():
            return e.moments_diag(args.moments, None, average=False, on_device_ptr=d_st.data_ptr(), num_vectors=R)

        mu = run()  # warm (tuning) + the moments
        nv = max(1, min(args.steps, 3))
        torch.cuda.synchronize()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(sv)
        recs = []
        for _ in range(nv):
            run()
            recs.append(e.stats().moments_time)
        g1.record(sv)
        torch.cuda.synchronize()
        tv = g0.elapsed_time(g1) * 1e-3 / nv
        sv_st = e.stats()
        fz = int(sv_st.steps_per_launch)
        nl = 1 + (M // 2 - 1) // fz
        alg_v = nnz * (8 + 4) + 4 * (nrows + 1) + (3 if fz == 1 else 4) * nrows * R * elem_bytes
        avg_v = float(np.median(recs)) / nl
        out = {"value": work / tv / 1e9, "unit": UNIT, "ms_per_step": tv * 1e3, "timed_steps": nv,
               "kernel": step_kernel(sv_st, prec, "double" if elem_bytes == 8 else "float"),
               "roofline": {"bound": "hbm", "achieved": alg_v / avg_v / 1e9, "peak": peak, "unit": "GB/s",
                            "frac": alg_v / avg_v / 1e9 / peak, "alg_bytes_per_launch": alg_v,
                            "avg_launch_ms": avg_v * 1e3}}
        e.close()
        return out, mu, same

    def errors(m, ref):
        # per-vector moments, and the stochastic-trace moments (average over the vectors of a
        # flake, as the reference's BatchAccumulator returns them), each relative to its max |mu|
        return {"per_vector_max": float(np.max(np.abs(m - ref)) / np.max(np.abs(ref))),
                "vector_averaged_max": float(np.max(np.abs(m.mean(1) - ref.mean(1))) / np.max(np.abs(ref.mean(1))))}

    # the plain FP64 recursion of the same workload (the other half of the metric), whose moments
    # are the error reference of the FP32 ones (the engines' Lanczos bounds are the same bits:
    # their sums run in a fixed order), and the FP32 recursion with chained-FMA row sums
    err = None
    fp64 = None
    fp32_fma = None
    if not args.no_error:
        m32 = eng.moments_diag(args.moments, None, average=False, on_device_ptr=d_st.data_ptr(), num_vectors=R)
        bounds32 = [eng.energy_bounds(s) for s in range(nsys)]
        scales = [eng.scaling_factors(s) for s in range(nsys)]
        eng.close()
        fp64, m64, same_bounds = variant("fp64", 8)
        err = errors(m32, m64)
        err["reference"] = "FP64 recursion of the same workload (GPU), identical Lanczos bounds: %s" % same_bounds
        if args.precision != "fp32":
            fp32_fma, mf, _ = variant("fp32", 4)
            fp32_fma["moment_error_vs_fp64"] = errors(mf, m64)
    else:
        eng.close()

    cpu = None
    if rank == 0:
        # CPU leg: the timed CPU baseline on the whole workload, and the FP64 oracle as the checker of
        # the largest flake's first two vectors (the FP64 GPU run above is pinned to it there)
        cpu_run = CpuWorkload(hs, R, args.seed, os.cpu_count() or 1)
        v, sec, Ms = cpu_run.sample(args.cpu_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": cpu_run.describe(Ms)}
        del cpu_run
        if err is not None:
            big = int(np.argmax([x.shape[0] for x in hs]))
            a, b = scales[big]
            st_big = starters[R * int(offsets[big]):R * int(offsets[big + 1])].reshape(R, -1)[:2]
            chk = oracle_check(hs[big].astype(np.float32), a, b, st_big, M, m64[big, :2], m32[big, :2])
            err.update({"oracle_flake_sites": int(hs[big].shape[0]), "oracle_vectors": 2, **chk})

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": workload_config(args, hs),
               "moment_error_vs_fp64": err,
               "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": traffic,
                            "kernel": kernel_name,
                            "steps_per_launch": fuse, "tiling": tiling, "alg_bytes_per_launch": alg_bytes,
                            "avg_launch_ms": avg_launch * 1e3, "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
               "cpu_baseline": cpu,
               "fp64": fp64,
               "fp32_chained_fma": fp32_fma,
               "e2e": e2e,
               "clocks": clk,
               "gpu_launches": int(args.steps * (launches + 3))}
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ---------------------------------------------------------------- other configurations
def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def _timed(fn, steps, warmup, stream):
    """Run fn warmup + steps times; device time of the timed steps (CUDA events on `stream`),
    the wall time, and the clocks seen meanwhile."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    w0 = time.perf_counter()
    e0.record(stream)
    outs = [fn() for _ in range(steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    return e0.elapsed_time(e1) * 1e-3, wall, clocks.stop(), outs


def _jackson_broadening(num_moments, a):
    """Broadening for which calc_* takes exactly num_moments Jackson moments (Kernel.cpp:6-20)."""
    from pybinding_gb300 import _native
    lo, hi = 1e-6, 10.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if _native.required_num_moments("jackson", 4.0, mid / a) > num_moments:
            lo = mid
        else:
            hi = mid
    return hi


def _line(args, metric, value, unit, hib, t_step, config, dtype, **extra):
    out = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": hib, "scaling": "weak",
           "vs_baseline": None, "dtype": dtype, "data": "synthetic", "config": config}
    out.update(extra)
    print(json.dumps(out), flush=True)


def workload_dos_c128_60k(args, stream_of):
    """60,000-site complex128 graphene flake (t = -2.8 eV, onsite 0), 8 random-phase vectors,
    2048 moments (2050 after rounding), Jackson, Lanczos bounds, DOS at 1000 energies in [-9, 9]."""
    from pybinding_gb300 import _native, lattice as L
    m = L.graphene_flake(60000, is_complex=True, is_double=True)
    h = m.hamiltonian.astype(np.complex128)
    eng = _native.Engine(h, _native.make_config(fuse_steps=args.fuse, staging=args.staging))
    a, b = eng.scaling_factors()
    broadening = _jackson_broadening(2048, a)
    energy = np.linspace(-9, 9, 1000)
    stream = stream_of(eng)
    t, wall, clk, _ = _timed(lambda: eng.calc_dos(energy, broadening, 8), args.steps, args.warmup, stream)
    st = eng.stats()
    M = st.num_moments
    work = (M / 2) * h.nnz * 8
    rec = st.moments_time
    steps = M // 2
    spl = max(1, int(st.steps_per_launch))  # 1 or 2 steps per launch
    launches = 1 + -(-(steps - 1) // spl)
    alg = h.nnz * 20 + 4 * (h.shape[0] + 1) + 3 * h.shape[0] * 8 * 16  # per step
    achieved = alg / (rec / steps) / 1e9
    err = None
    if not args.no_error:  # the reference's 8 random-phase starters: engine moments against the FP64 oracle
        from oracle import oracle as O
        st_ref = O.random_starters(h.shape[0], 8, np.complex128)
        mu = eng.moments_diag(2048, st_ref[None])[0]
        r = O.optimize(h, [0], [0], a, b)
        ref = O.moments_diag(r["h2"], O.reorder_vector(st_ref, r["reorder_map"]), mu.shape[1], slices=r["slices"])
        err = {"per_vector_max_vs_oracle": float(np.max(np.abs(mu - ref)) / np.max(np.abs(ref))),
               "vectors": 8, "moments": int(mu.shape[1]),
               "starters": "the reference's random-phase starters (std::mt19937 default seed)"}
    cpu = None
    if args.cpu_seconds > 0:
        from oracle import oracle as O
        r = O.optimize(h, [0], [0], a, b)
        rng = np.random.default_rng(1)
        st0 = np.exp(2j * np.pi * rng.random((8, h.shape[0])))
        st0 = O.reorder_vector(st0, r["reorder_map"])
        Ms = 514
        threads = os.cpu_count() or 1
        _, sec = O.bench_diag(r["h2"], r["slices"], st0, Ms, 2, threads)
        cpu = {"value": (Ms / 2) * h.nnz * 8 / sec / 1e9, "unit": "Gnnz*vec/s", "cores": min(threads, 4),
               "kind": "port",
               "sample": "the same flake and 8 complex128 vectors in 2-vector batches (the reference's complex128 "
                         "SIMD batch, support/simd.hpp:35-43), %d moments, a pool of %d threads of which the 4 "
                         "batches keep 4 busy (kpm/default/Compute.cpp:52-88), timed build -O3 %s" % (
                             Ms, threads, " ".join(O._fast_flags()[1:]))}
    _line(args, "KPM DOS (complex128) Gnnz*vec/s", work / (t / args.steps) / 1e9, "Gnnz*vec/s", True,
          t / args.steps,
          {"workload": "graphene DOS: 60k sites complex128, 8 random-phase vectors, 2048 moments, 1000 energies",
           "sites": int(h.shape[0]), "nnz": int(h.nnz), "moments": int(M), "broadening_eV": broadening,
           "l2": "L2-resident working set (matrix ~4 MB, vectors 8 x 1 MB): latency-bound, no flush"},
          "c128",
          roofline={"bound": "l2 (latency)", "achieved": achieved, "unit": "GB/s",
                    "note": "working set fits in L2; HBM fraction not meaningful",
                    "avg_step_us": rec / steps * 1e6, "alg_bytes_per_step": alg, "steps_per_launch": spl,
                    "kernel": "diag_step_kernel" if spl == 1 else "diag_pair_kernel"},
          e2e={"value": work / (wall / args.steps) / 1e9, "unit": "Gnnz*vec/s", "h2d_bytes_per_step": 8000,
               "d2h_bytes_per_step": 8000},
          moment_error_vs_fp64=err, cpu_baseline=cpu, clocks=clk, time_per_dos_ms=t / args.steps * 1e3,
          gpu_launches=int(args.steps * (launches + 4)))


def workload_conductivity(args, stream_of):
    """Kubo-Bastin sigma_xx: 1M-site graphene under 20 T (Peierls phases, complex128), velocity
    from bond x-displacements, 16 random-phase vectors, 512 moments, Jackson; mu_mn on the tensor
    cores (tcgen05 TF32 three-product split of FP32 planes)."""
    from pybinding_gb300 import _native, lattice as L
    m = L.graphene_flake(args.cond_sites, hopping_modifiers=[L.constant_magnetic_field(20.0)], is_complex=True,
                         is_double=True)
    h = m.hamiltonian.astype(np.complex128)
    x = m.system.x
    eng = _native.Engine(h, _native.make_config(energy_range=(-9.0, 9.0), precision=args.cond_precision))
    a, b = eng.scaling_factors()
    broadening = _jackson_broadening(512, a)
    chem = np.linspace(-1.5, 1.5, 31)
    stream = stream_of(eng)
    t, wall, clk, outs = _timed(lambda: eng.calc_conductivity(x, x, chem, broadening, 0.0, 16, 1000, gemm_mode=1),
                                args.steps, args.warmup, stream)
    deviation = None
    if args.cond_precision == "fp32":  # sigma against the complex128 recursion (same tensor-core GEMM)
        e64 = _native.Engine(h, _native.make_config(energy_range=(-9.0, 9.0), precision="fp64"))
        s64 = e64.calc_conductivity(x, x, chem, broadening, 0.0, 16, 1000, gemm_mode=1).real
        e64.close()
        deviation = float(np.max(np.abs(outs[-1].real - s64)) / np.max(np.abs(s64)))
        eng.calc_conductivity(x, x, chem, broadening, 0.0, 16, 1000, gemm_mode=1)  # stats of this engine again
    st = eng.stats()
    gemm_dev = None
    if not args.no_error:  # one random vector: tcgen05 split-TF32 mu_mn against the FP64 CUDA-core GEMM
        s_tc = eng.calc_conductivity(x, x, chem, broadening, 0.0, 1, 1000, gemm_mode=1).real
        s_64 = eng.calc_conductivity(x, x, chem, broadening, 0.0, 1, 1000, gemm_mode=0).real
        gemm_dev = {"sigma_rel_deviation_tc_vs_fp64_gemm": float(np.max(np.abs(s_tc - s_64)) / np.max(np.abs(s_64))),
                    "vectors": 1,
                    "note": "the recursion is FP64 (complex128) in both; its moments equal the FP64 oracle to "
                            "<1e-13 on the configuration's graphene flakes (tests)"}
        eng.calc_conductivity(x, x, chem, broadening, 0.0, 16, 1000, gemm_mode=1)
        st = eng.stats()
    M = st.num_moments
    n = h.shape[0]
    I = n * 16
    useful = 8.0 * M * M * I
    tensor = 3 * useful  # hi*hi + hi*lo + lo*hi
    peaks = _peaks()
    peak_tf32 = float(peaks.get("bf16_tflops", 1900.0)) / 2
    gemm = st.gemm_time
    rec = st.moments_time - gemm
    rec_work = 2 * M * h.nnz * 16
    _line(args, "Kubo-Bastin sigma_xx time per call (%d sites, 16 vectors, 512 moments)" % n, t / args.steps, "s",
          False, t / args.steps,
          {"workload": "conductivity: %d-site graphene, 20 T, complex128, 16 vectors, 512 moments, tensor-core mu_mn"
                       % n,
           "sites": int(n), "nnz": int(h.nnz), "moments": int(M), "vectors": 16, "broadening_eV": broadening,
           "gemm": "tcgen05 kind::tf32, hi/lo split (3 products), FP32 planes, FP64 slice sums"},
          ("c64" if args.cond_precision == "fp32" else "c128") + " recursion, tf32x3 GEMM",
          roofline={"bound": "tensor", "achieved": tensor / gemm / 1e12, "peak": peak_tf32, "unit": "TFLOP/s",
                    "frac": tensor / gemm / 1e12 / peak_tf32, "traffic": None,
                    "kernel": "mu_gemm_tc_kernel<true>",
                    "peak_source": "MEASURED_PEAKS.json bf16_tflops / 2 (dense TF32 runs at half the BF16 rate)",
                    "useful_tflops": useful / gemm / 1e12},
          breakdown={"recursion_s": rec, "recursion_gnnz_vec_per_s": rec_work / rec / 1e9, "gemm_s": gemm,
                     "reconstruction_and_host_s": t / args.steps - st.moments_time},
          e2e={"value": wall / args.steps, "unit": "s", "h2d_bytes_per_step": int(8 * n + 8 * 31),
               "d2h_bytes_per_step": int(16 * 31)},
          sigma_sample=[float(v.real) for v in outs[-1][:5]], sigma_rel_deviation_vs_fp64=deviation,
          moment_error_vs_fp64=gemm_dev, clocks=clk,
          gpu_launches=int(args.steps * (2 * (M + 2) + 6)))


def workload_adjoint(args, stream_of):
    """DOS-misfit gradient on 256k-site strained graphene (t_ij = -2.8 exp(-3.37 (d/a_cc - 1)),
    sinusoidal strain 5 %, period 20 nm), 32 Rademacher vectors, 1024 moments, FP32 recursion;
    target DOS from a 3 % strain. One step = forward moments + adjoint gradient (onsite + bonds)."""
    from pybinding_gb300 import _native, jackson_kernel, lattice as L
    from pybinding_gb300.adjoint import DiagonalMoments, moments_weights

    def flake(amp):
        return L.graphene_flake(args.adj_sites, hopping_modifiers=[L.strained_hopping(L.sinusoidal_strain(amp, 20.0))],
                                is_double=True)
    m = flake(0.05)
    h = m.hamiltonian.tocsr()
    h.sort_indices()
    n = h.shape[0]
    rng = np.random.default_rng(3)
    r0 = np.where(rng.integers(0, 2, (32, n)) == 0, -1.0, 1.0)
    rng_e = (-9.5, 9.5)
    op = DiagonalMoments(h, args.adj_moments, r0, rng_e, precision="fp32")
    ht = flake(0.03).hamiltonian.tocsr()
    ht.sort_indices()
    tgt = DiagonalMoments(ht, args.adj_moments, r0, rng_e, precision="fp32")
    energy = np.linspace(-8, 8, 400)
    W = moments_weights(energy, op.scaling, jackson_kernel(), op.num_moments)
    target = W @ tgt.moments(ht.data)
    eng_stream = stream_of(op._engine)
    times = {}

    def step():
        mu = op.moments(h.data)
        times["fwd"] = op._engine.stats().moments_time
        rho = W @ mu
        dl_dmu = W.T @ (2 * (rho - target))
        gv, go = op.gradient(h.data, dl_dmu)
        times["bwd"] = op._engine.stats().moments_time
        return float(np.sum((rho - target) ** 2)), gv, go

    t, wall, clk, outs = _timed(step, args.steps, args.warmup, eng_stream)
    M = op.num_moments
    nnz = h.nnz
    fwd_work = (M / 2) * nnz * 32
    # backward (all vectors kept, the automatic choice here): recomputation + adjoint recursion
    bwd_work = 2 * (M / 2) * nnz * 32
    # the same with sqrt(M/2) checkpoints: one more forward pass, ~3 sqrt(M/2) vectors of memory
    op.checkpoint = int(np.ceil(np.sqrt(M // 2)))
    op.gradient(h.data, np.ones(M))
    t_sqrt = op._engine.stats().moments_time
    op.checkpoint = 0
    _line(args, "adjoint DOS-misfit gradient time per forward+backward (%d sites, 32 vectors, %d moments)" % (n, M),
          t / args.steps, "s", False, t / args.steps,
          {"workload": "adjoint gradients: %d-site strained graphene, 32 vectors, %d moments, fp32" % (n, M),
           "sites": int(n), "nnz": int(nnz), "moments": int(M),
           "checkpoint": "automatic (all vectors: they fit in HBM)"},
          "f32 recursion and gradient sums",
          breakdown={"forward_s": times["fwd"], "forward_gnnz_vec_per_s": fwd_work / times["fwd"] / 1e9,
                     "backward_s": times["bwd"], "backward_gnnz_vec_per_s": bwd_work / times["bwd"] / 1e9,
                     "backward_over_forward": times["bwd"] / times["fwd"],
                     "backward_sqrt_checkpoints_s": t_sqrt},
          loss=outs[-1][0], grad_norm=float(np.linalg.norm(outs[-1][1])),
          e2e={"value": wall / args.steps, "unit": "s", "h2d_bytes_per_step": int(2 * (8 * nnz + 4 * 32 * n)),
               "d2h_bytes_per_step": int(8 * (nnz + n) + 8 * M)},
          clocks=clk)


def workload_anderson3d(args, stream_of):
    """3D Anderson model: simple cubic 160^3 periodic, t = -1, onsite U[-8.25, 8.25], 256 Rademacher
    vectors, 8192 moments (8194), FP32 vectors / FP64 sums; then LDOS at 4096 sites (1024 moments)."""
    from pybinding_gb300 import _native, lattice as L
    Lc = args.cube
    rng = np.random.default_rng(5)
    h = L.simple_cubic_periodic(Lc, onsite=rng.uniform(-8.25, 8.25, Lc ** 3).astype(np.float32)).hamiltonian
    n = h.shape[0]
    R = args.cube_vectors
    eng = _native.Engine(h, _native.make_config(staging=args.staging, fuse_steps=args.fuse, precision=args.precision))
    eng.scaling_factors()
    st = (rng.integers(0, 2, (R, n), dtype=np.int8) * 2 - 1).astype(np.float32)
    import torch
    d_st = torch.from_numpy(st.reshape(-1)).cuda()
    stream = stream_of(eng)
    t, wall, clk, _ = _timed(lambda: eng.moments_diag(args.cube_moments, None, average=True, on_device_ptr=d_st.data_ptr(),
                                                      num_vectors=R), args.steps, args.warmup, stream)
    s = eng.stats()
    M = s.num_moments
    work = (M / 2) * h.nnz * R
    fuse = int(s.steps_per_launch)
    launches = 1 + (M // 2 - 1) // fuse
    vec_bytes = (3 if fuse == 1 else 4) * n * R * 4
    alg = h.nnz * 12 + 4 * (n + 1) + vec_bytes
    avg = s.moments_time / launches
    peak = float(_peaks().get("hbm_gbs", 6800.0))
    err = None
    if not args.no_error:
        R8 = min(8, R)
        st8 = st[:R8]
        m32 = eng.moments_diag(args.cube_moments, st8[None])[0]
        e64 = _native.Engine(h, _native.make_config(precision="fp64"))
        assert e64.energy_bounds() == eng.energy_bounds()
        m64 = e64.moments_diag(args.cube_moments, st8[None])[0]
        from oracle import oracle as O
        a, b = eng.scaling_factors()
        Mo = 130
        r = O.optimize(h.astype(np.float64), [0], [0], a, b)
        ref = O.moments_diag(r["h2"], O.reorder_vector(st8[:1].astype(np.float64), r["reorder_map"]), Mo,
                             slices=r["slices"])
        m64o = e64.moments_diag(Mo, st8[None, :1])[0]
        e64.close()
        err = {"per_vector_max": float(np.max(np.abs(m32 - m64)) / np.max(np.abs(m64))), "vectors": R8,
               "moments": int(m32.shape[1]),
               "vector_averaged": float(np.max(np.abs(m32.mean(0) - m64.mean(0))) / np.max(np.abs(m64.mean(0)))),
               "fp64_vs_oracle": float(np.max(np.abs(m64o - ref)) / np.max(np.abs(ref))),
               "fp64_vs_oracle_moments": Mo,
               "reference": "the engine's FP64 recursion on the same vectors and bounds; that recursion against "
                            "the FP64 oracle on one vector"}
        eng.moments_diag(args.cube_moments, None, average=True, on_device_ptr=d_st.data_ptr(), num_vectors=R)
        s = eng.stats()
    t_ldos = None
    if args.ldos_sites > 0:
        sites = rng.choice(n, args.ldos_sites, replace=False)
        a, b = eng.scaling_factors()
        t0 = time.perf_counter()
        eng.calc_ldos(sites, np.linspace(-10, 10, 200), _jackson_broadening(1024, a))
        t_ldos = time.perf_counter() - t0
    _line(args, "KPM Gnnz*vec/s (3D Anderson, %d vectors, %d moments, FP32)" % (R, M), work / (t / args.steps) / 1e9,
          "Gnnz*vec/s", True, t / args.steps,
          {"workload": "3D Anderson: simple cubic %d^3 periodic, W = 16.5, %d vectors, %d moments" % (Lc, R, M),
           "sites": int(n), "nnz": int(h.nnz), "moments": int(M), "vectors": R,
           "recursion": {"fp32x": "fp32 row sums compensated by TwoSum", "fp32": "fp32 row sums of chained FMAs"}.get(
               args.precision, "fp32 row sums compensated by an FMA per term (auto)"),
           "l2": "inputs larger than L2 (no flush)"},
          "f32",
          roofline={"bound": "hbm", "achieved": alg / avg / 1e9, "peak": peak, "unit": "GB/s",
                    "frac": alg / avg / 1e9 / peak, "traffic": None, "steps_per_launch": fuse,
                    "kernel": step_kernel(s, args.precision),
                    "lane_map": [int(s.elems_per_lane), int(s.lanes_per_row)], "tile_rows": int(s.tile_rows),
                    "unroll": int(s.unroll),
                    "alg_bytes_per_launch": alg, "avg_launch_ms": avg * 1e3,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
          moment_error_vs_fp64=err, ldos_sites=args.ldos_sites, ldos_1024_moments_s=t_ldos, clocks=clk,
          gpu_launches=int(args.steps * (launches + 3)))


def workload_lattice(args, stream_of):
    """Input build: a disordered graphene flake of --lattice-sites sites (onsite U[-0.5, 0.5] eV,
    float32) built by the GPU builder, end to end through ``build_honeycomb(device="gpu")``
    (device kernels, the onsite modifier on the host, copies both ways, the SciPy matrix);
    the host (numpy) build of the same flake is the CPU baseline."""
    from pybinding_gb300 import _native, lattice as L
    import scipy.sparse  # noqa: F401  (imported before the timed region)
    n_req = args.lattice_sites
    mods = [L.anderson_disorder(1.0, args.seed)]
    last = {}

    def step():
        m = L.graphene_flake(n_req, onsite_modifiers=mods, device="gpu")
        last["m"] = m
        return m
    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    wall = (time.perf_counter() - w0) / args.steps
    clk = clocks.stop()
    m = last["m"]
    n, nnz = m.hamiltonian.shape[0], m.hamiltonian.nnz
    # device-only time of one build: the same calls through the C ABI, modifier values precomputed
    v = L.rectangle(*_flake_dims(n_req))
    v0, v1, sub_pos, origin, s0, s1 = L._honeycomb_frame(v, L.GRAPHENE_A, L.GRAPHENE_A_CC, False)
    onsite = m.hamiltonian.diagonal().astype(np.float32)
    dev = []
    for _ in range(max(1, args.steps)):
        b = _native.LatticeBuild.honeycomb(s0, s1, origin, v0, v1, sub_pos, L._HONEYCOMB_HOPS, v, 2)
        b.csr(np.float32, hopping=L.GRAPHENE_T, onsite=onsite)
        t_build, t_csr, launches = b.times()
        dev.append(t_build + t_csr)
        b.close()
    t_dev = min(dev)
    foundation = 2 * s0 * s1
    # algorithmic bytes: foundation positions + flags written and read back, site positions,
    # onsite values in, CSR out
    alg = foundation * (12 + 4) * 2 + n * 12 + n * 4 + 4 * (n + 1) + nnz * 8
    peak = float(_peaks().get("hbm_gbs", 6800.0))
    t0 = time.perf_counter()
    ref = L.graphene_flake(n_req, onsite_modifiers=mods)
    t_cpu = time.perf_counter() - t0
    same = (ref.hamiltonian.indices.tobytes() == m.hamiltonian.indices.tobytes()
            and ref.hamiltonian.data.tobytes() == m.hamiltonian.data.tobytes())
    _line(args, "Msites/s (GPU build of a graphene flake Hamiltonian, end to end)", n / wall / 1e6, "Msites/s", True,
          wall, {"workload": "graphene flake build: %d sites, Anderson onsite U[-0.5, 0.5], float32 CSR" % n,
                 "sites": int(n), "nnz": int(nnz), "foundation_sites": int(foundation)},
          "f32",
          device_s=t_dev,
          roofline={"bound": "hbm", "achieved": alg / t_dev / 1e9, "peak": peak, "unit": "GB/s",
                    "frac": alg / t_dev / 1e9 / peak, "traffic": None, "kernel": "all builder kernels (one build)",
                    "alg_bytes_per_launch": alg, "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
          cpu_baseline={"value": n / t_cpu / 1e6, "unit": "Msites/s", "cores": 1, "kind": "port",
                        "sample": "the same flake built by the numpy host build (%.2f s), identical CSR: %s"
                                  % (t_cpu, same)},
          e2e={"value": n / wall / 1e6, "unit": "Msites/s", "h2d_bytes_per_step": int(n * 4),
               "d2h_bytes_per_step": int(n * 12 + 4 * (n + 1) + nnz * 8)},
          clocks=clk, gpu_launches=int(launches * args.steps))


def workload_sweep(args, stream_of):
    """Disorder sweep (``parallel_for`` over deferred LDOS): --sweep-models graphene flakes of
    --sweep-sites sites, onsite disorder of width 0..3 eV (float32 H), LDOS at the site nearest
    the centre on 200 energies in [-8, 8] eV, broadening 0.05 eV (Jackson). End to end per
    sweep: engines, reorder, Lanczos bounds, one batched recursion, reconstruction."""
    import pybinding_gb300 as pbg
    from pybinding_gb300 import lattice as L, parallel
    from oracle import oracle as O
    widths = np.linspace(0.0, 3.0, args.sweep_models)
    models = [L.graphene_flake(args.sweep_sites, onsite_modifiers=[L.anderson_disorder(w, 100 + i)], device="gpu")
              for i, w in enumerate(widths)]
    energy = np.linspace(-8, 8, 200)
    broadening = 0.05

    def jobs():
        return [pbg.kpm(m).deferred_ldos(energy, broadening, [0, 0]) for m in models]

    def step():
        js = jobs()
        parallel.compute_all(js)
        return js
    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        batched = step()
    wall = (time.perf_counter() - w0) / args.steps
    clk = clocks.stop()
    st = parallel.last_batch_stats
    t0 = time.perf_counter()
    jobs()
    t_jobs = time.perf_counter() - t0
    # the same jobs one by one (each its own engine and recursion), for the batching gain
    t0 = time.perf_counter()
    single = jobs()
    for j in single:
        j.compute()
    t_single = time.perf_counter() - t0
    diff = max(float(np.max(np.abs(b.result[:, 0] - np.squeeze(s.result))) / np.max(np.abs(s.result)))
               for b, s in zip(batched, single))
    n = sum(m.hamiltonian.shape[0] for m in models)
    nnz = sum(m.hamiltonian.nnz for m in models)
    M = int(st.num_moments)
    launches = M // 2
    avg = st.moments_time / launches
    # one vector (K = 1, FP32): matrix (hi/lo values + index) once, x, y_old, y_new
    alg = nnz * 12 + 4 * (n + 1) + 3 * n * 4
    peak = float(_peaks().get("hbm_gbs", 6800.0))
    # CPU: the oracle's LDOS (one thread) on one model of the sweep
    h0 = models[-1].hamiltonian
    idx0 = int(models[-1].system.find_nearest([0, 0]))
    t0 = time.perf_counter()
    O.core_ldos(h0, [idx0], energy, broadening)
    t_cpu = time.perf_counter() - t0
    _line(args, "LDOS sweep points/s (deferred LDOS of %d models, batched)" % len(models), len(models) / wall,
          "points/s", True, wall,
          {"workload": "disorder sweep: %d graphene flakes of %d sites, W = 0..3 eV, LDOS at the centre, "
                       "200 energies, broadening 0.05 eV" % (len(models), args.sweep_sites),
           "sites": int(n), "nnz": int(nnz), "moments": M},
          "f32",
          sequential_s=t_single, batched_s=wall, batched_vs_sequential_max_rel_diff=diff,
          recursion_s=st.moments_time, bounds_s=st.bounds_time, jobs_s=t_jobs,
          batch_assemble_s=parallel.last_batch_times.get("assemble_s"),
          engine_call_s=parallel.last_batch_times.get("call_s"), reorder_s=st.hamiltonian_time,
          roofline={"bound": "hbm", "achieved": alg / avg / 1e9, "peak": peak, "unit": "GB/s",
                    "frac": alg / avg / 1e9 / peak, "traffic": None, "kernel": "diag_step_kernel (K = 1)",
                    "alg_bytes_per_launch": alg, "avg_launch_ms": avg * 1e3,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
          cpu_baseline={"value": 1.0 / t_cpu, "unit": "points/s", "cores": 1, "kind": "port",
                        "sample": "one model of the sweep (%d sites), the oracle's Core::ldos: %.2f s"
                                  % (h0.shape[0], t_cpu)},
          e2e={"value": len(models) / wall, "unit": "points/s", "h2d_bytes_per_step": int(nnz * 12 + 4 * n),
               "d2h_bytes_per_step": int(len(models) * energy.size * 8)},
          clocks=clk, gpu_launches=int(args.steps * (launches + 2 * len(models) + 3)))


def _flake_dims(num_sites, aspect=1.0):
    from pybinding_gb300 import lattice as L
    area = num_sites / L.GRAPHENE_SITE_DENSITY
    w = math.sqrt(area * aspect)
    return w, area / w


def run_workload(args, rank, world, local_rank):
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "workload": args.workload,
                          "unavailable": "the reference arm is defined for the default workload; the CPU "
                                         "baseline of this one is in its own line"}), flush=True)
        return
    if rank != 0:
        return
    import torch
    torch.cuda.set_device(local_rank)

    def stream_of(eng):
        return torch.cuda.ExternalStream(eng.stream())
    {"dos_c128_60k": workload_dos_c128_60k, "conductivity": workload_conductivity, "adjoint": workload_adjoint,
     "anderson3d": workload_anderson3d, "lattice": workload_lattice,
     "sweep": workload_sweep}[args.workload](args, stream_of)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload != "dos_batch":
        run_workload(args, rank, world, local_rank)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
