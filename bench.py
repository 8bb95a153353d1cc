"""Benchmark of the GB300 SpGEMM engine (one JSON line on stdout).

Default workload: the skewed square product C = A x A, A 1,048,576^2 CSR with
lognormal row lengths (arithmetic mean 24, sigma 1.2, capped at 20,000), 70% of
the columns within +-2,048 of the diagonal and 30% uniform, FP64 U[-1, 1),
seeded synthetic data.  Metric: GFLOP/s = 2 x scalar products / time (the
reference's definition, two_sided_spgemm.cpp:188-192).

* value: device-resident operands, result left on the device; every timed step
  between its own CUDA events on the engine's stream; workloads whose inputs
  fit in L2 get an L2 flush between steps, outside the events.
* e2e: the same product through the C ABI with host (pinned) buffers
  (spg_multiply_to_host): the host->device copy of A and the device->host copy
  of C inside every step, the copy of C overlapping the computation.
* roofline: the numeric phase (K4, all bins), its algorithmic bytes over its
  CUDA-event time measured in every timed step.
* cpu_baseline: the reference's OpenMP row loop (the oracle port of
  spgemm_exchange.cpp:258-325, or the reference's own build where it loads) on
  a bounded slice of A's rows, timed on this host's cores.

--impl reference runs only the CPU reference on the same workload and prints
its own line.  With torchrun (N > 1) the rows of every product are sharded:
each rank multiplies the block of A's rows holding about P / N scalar products
against all of B on its own GPU (no collective inside the timed region), and
value sums the ranks' products over the slowest rank's time (strong scaling).
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "spgemm-hpc-thesis_gb300"))

L2_BYTES = 129 << 20

WORKLOADS = {
    "powerlaw": "skewed C=A*A, A 1048576^2 lognormal rows (mean 24, sigma 1.2, cap 20000), "
                "70% within +-2048 band, FP64 U[-1,1)",
    "uniform": "C=A*B, A and B 65536^2, 16 distinct uniform columns per row, FP64 U[-1,1)",
    "galerkin": "R*A then (R*A)*R^T, A 7-point Laplacian on 128^3, R 2x2x2 aggregation (262144 x 2097152)",
    "batched": "512 independent square C_i = A_i*B_i, rows log-uniform in [1000, 200000], 4-64 distinct uniform "
               "columns per row, FP64 U[-1,1); admitted in waves under a 150 GB budget",
    "served": "Poisson arrivals (50-2000 req/s) of products drawn from the uniform, power-law, Galerkin and "
              "batched size distributions (<= 2M rows), device-resident operands, 150 GB admission budget",
}
BATCH_PRODUCTS = 512
BATCH_MAX_PRODUCTS = 1 << 28  # scalar products per batch: ~8 ms of kernels, so the two lanes alternate
BATCH_SUBSET = 64  # products of the batched workload measured beside the headline line
SERVE_RATES = (50, 100, 200, 500, 1000, 2000)


def make_workload(name: str, rows: int = 0, count: int = 0):
    """[(A, B)] host operands of the workload's products (chained products are
    materialised once on the host).  rows != 0 shrinks the power-law matrix
    (profiling cases only)."""
    import spgemm_gb300 as sg
    if name == "powerlaw":
        a = sg.synth_powerlaw(rows or (1 << 20), 24.0, 1.2, 20000, 2048, 0.7, seed=1)
        return [(a, a)]
    if name == "uniform":
        return [(sg.synth_uniform(65536, 65536, 16, seed=1), sg.synth_uniform(65536, 65536, 16, seed=2))]
    if name == "galerkin":
        lap = sg.synth_laplacian3d(128)
        r = sg.synth_restriction(128)
        rt = sg.synth_restriction(128, transpose=True)
        with sg.Engine(int(os.environ.get("LOCAL_RANK", "0"))) as eng:
            ra = eng.multiply(r, lap)
        return [(r, lap), (ra, rt)]
    if name == "batched":
        rng = np.random.default_rng(4)
        sizes = np.exp(rng.uniform(np.log(1000), np.log(200000), size=BATCH_PRODUCTS)).astype(np.int64)
        if count:
            sizes = sizes[:count]
        return [(sg.synth_uniform(int(n), int(n), 4, 64, seed=2 * i + 1),
                 sg.synth_uniform(int(n), int(n), 4, 64, seed=2 * i + 2)) for i, n in enumerate(sizes)]
    if name == "served":
        return serve_pool()
    raise SystemExit(f"unknown workload {name}")


def serve_pool():
    """The request pool of the served stream: 6 products from each size
    distribution (uniform 65536^2 x 16; power-law with 2^12-2^18 rows; Galerkin
    R*A on 16^3-128^3 grids, 128^3 = 2,097,152 fine rows; the batched
    distribution's 1000-200000 rows x 4-64)."""
    import spgemm_gb300 as sg
    rng = np.random.default_rng(5)
    pool = []
    for i in range(6):
        pool.append((sg.synth_uniform(65536, 65536, 16, seed=100 + 2 * i),
                     sg.synth_uniform(65536, 65536, 16, seed=101 + 2 * i)))
    for i in range(6):
        n = int(np.exp(rng.uniform(np.log(4096), np.log(262144))))
        a = sg.synth_powerlaw(n, 24.0, 1.2, 20000, 2048, 0.7, seed=200 + i)
        pool.append((a, a))
    for g in (16, 32, 48, 64, 96, 128):
        pool.append((sg.synth_restriction(g), sg.synth_laplacian3d(g)))
    for i in range(6):
        n = int(np.exp(rng.uniform(np.log(1000), np.log(200000))))
        pool.append((sg.synth_uniform(n, n, 4, 64, seed=300 + 2 * i), sg.synth_uniform(n, n, 4, 64, seed=301 + 2 * i)))
    return pool


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def all_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def all_sum(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------------------
# CPU reference (the oracle port, or the reference's own build where it loads)
def cpu_reference():
    from oracle import build as obuild
    from oracle.oracle import Port, Reference
    obuild.build_oracle()
    if Reference.available():
        try:
            return Reference(), "reference"
        except OSError:
            pass
    return Port(), "port"


def row_slice(a, first: int, count: int):
    import spgemm_gb300 as sg
    rp = a.row_ptr[first:first + count + 1]
    lo, hi = int(rp[0]), int(rp[-1])
    return sg.Csr(count, a.cols, rp - lo, a.col[lo:hi], a.val[lo:hi])


def time_cpu_slice(impl, kind: str, a, b, first: int, count: int, threads: int) -> tuple[float, int]:
    """Seconds of one reference row-loop call on A[first:first+count] x B and its products."""
    import spgemm_gb300 as sg
    s = row_slice(a, first, count)
    products = sg.scalar_products_host(s, b)
    if kind == "reference":
        secs, _ = impl.spgemm_timed(s, b, threads=threads, chunk=64, repeats=1)
        return float(secs[0]), products
    t0 = time.perf_counter()
    impl.spgemm_omp_rows(s, b, 0, count, threads=threads, chunk=64)
    return time.perf_counter() - t0, products


CPU_SAMPLE_SECONDS = 8.0   # CPU work per timed reference step (and of the cpu_baseline sample)
CPU_SAMPLE_QUANTUM = 1 << 17  # sample sizes are whole multiples of this many rows (or all rows)


def cpu_sample_rows(impl, kind, a, b, threads: int, target_s: float = CPU_SAMPLE_SECONDS) -> tuple[int, int]:
    """A centred row slice sized to take about target_s seconds, rounded up to a
    multiple of CPU_SAMPLE_QUANTUM rows (all rows when that covers A), so that
    the reference arm and the GPU arm's cpu_baseline time the same rows."""
    m = a.rows
    n = min(m, 2048)
    first = max(0, m // 2 - n // 2)
    t, _ = time_cpu_slice(impl, kind, a, b, first, n, threads)
    want = n * target_s / max(t, 1e-6)
    n = int(min(m, -(-max(want, 1) // CPU_SAMPLE_QUANTUM) * CPU_SAMPLE_QUANTUM))
    first = max(0, m // 2 - n // 2)
    return first, n


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    pairs = make_workload(args.workload, args.rows)
    impl, kind = cpu_reference()
    threads = os.cpu_count() or 1
    a, b = pairs[0]
    first, n = cpu_sample_rows(impl, kind, a, b, threads)
    for _ in range(args.warmup):
        time_cpu_slice(impl, kind, a, b, first, n, threads)
    tot_t, tot_p = 0.0, 0
    for _ in range(args.steps):
        t, p = time_cpu_slice(impl, kind, a, b, first, n, threads)
        tot_t += t
        tot_p += p
    value = 2.0 * tot_p / tot_t / 1e9
    sample = f"rows [{first}, {first + n}) of A ({n} of {a.rows} rows) x B, first product of the workload"
    line = {
        "impl": "reference", "metric": "GFLOP/s", "value": value, "unit": "GFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "name": args.workload},
        "cpu_baseline": {"value": value, "unit": "GFLOP/s", "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
def device_measure(eng, pairs, dev_pairs, steps: int, warmup: int, local: int, world: int = 1):
    """Device-timed steps of one workload: every step multiplies all of its
    products with device-resident operands (results left on the device and
    freed), between CUDA events on the engine's stream; inputs smaller than L2
    get a 512 MiB write between steps, outside the events.  Returns the
    measurement, the roofline of the numeric phase and the bookkeeping."""
    import torch
    import spgemm_gb300 as sg
    products = sum(sg.scalar_products_host(a, b) for a, b in pairs)
    c_nnz = []
    for da, db in dev_pairs:  # one untimed product per pair: nnz(C) for the byte count
        r = eng.multiply(da, db, out="device")
        c_nnz.append(r.nnz)
        r.free()
    bytes_alg = sum(sg.algorithmic_bytes(a, b, sg.scalar_products_host(a, b), n)
                    for (a, b), n in zip(pairs, c_nnz))
    stream = torch.cuda.ExternalStream(eng.stream, device=torch.device("cuda", local))
    last_phases: dict = {}

    def step():
        launches = 0
        numeric_ms = 0.0
        for da, db in dev_pairs:
            r = eng.multiply(da, db, out="device")
            t = eng.last_timings()
            launches += t["launches"]
            numeric_ms += t["ms_numeric"]
            r.free()
        last_phases.clear()
        last_phases.update({k: v for k, v in t.items() if k.startswith("ms_")})
        return launches, numeric_ms

    in_bytes = sum(_csr_bytes(a) + (0 if b is a else _csr_bytes(b)) for a, b in pairs)
    flush = in_bytes < L2_BYTES
    flush_buf = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}") if flush else None
    for _ in range(warmup):
        step()
    barrier(world)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    launches = 0
    numeric_ms = 0.0
    with ClockSampler(local) as clocks:
        for e0, e1 in evs:
            if flush:
                with torch.cuda.stream(stream):
                    flush_buf.fill_(1)
            e0.record(stream)
            l, nm = step()
            e1.record(stream)
            launches += l
            numeric_ms += nm
        evs[-1][1].synchronize()
    torch.cuda.synchronize()
    barrier(world)
    t_ms = sum(e0.elapsed_time(e1) for e0, e1 in evs)
    pk = peaks()
    numeric_avg_s = numeric_ms / steps / 1e3
    achieved = bytes_alg / numeric_avg_s / 1e9 if numeric_avg_s > 0 else None
    roofline = {"bound": "hbm", "kernel": "K4 numeric phase (all bins, one step)", "achieved": achieved,
                "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": (achieved / pk["hbm_gbs"]) if achieved else None,
                "peak_source": pk["source"], "bytes_alg": int(bytes_alg),
                "pipeline_frac": bytes_alg / (t_ms / steps / 1e3) / 1e9 / pk["hbm_gbs"]}
    return {"t_ms": t_ms, "products": products, "c_nnz": c_nnz, "launches": launches, "roofline": roofline,
            "phases": dict(last_phases), "clocks": clocks.summary(), "flush": flush, "in_bytes": in_bytes}


def sub_record(name: str, steps: int, warmup: int, local: int) -> dict:
    """A secondary workload measured in the same run as the headline one."""
    import spgemm_gb300 as sg
    pairs = make_workload(name)
    with sg.Engine(local) as eng:
        dev_pairs = []
        for a, b in pairs:
            da = a.to_device(local)
            dev_pairs.append((da, da if b is a else b.to_device(local)))
        m = device_measure(eng, pairs, dev_pairs, steps, warmup, local)
    return {"workload": WORKLOADS[name], "value": 2.0 * m["products"] * steps / (m["t_ms"] / 1e3) / 1e9,
            "unit": "GFLOP/s", "steps": steps, "warmup": warmup, "ms_per_step": m["t_ms"] / steps,
            "products_per_step": int(m["products"]), "c_nnz": int(sum(m["c_nnz"])),
            "l2": "L2 flushed between timed steps (512 MiB write outside the events)" if m["flush"]
                  else "inputs larger than L2", "roofline": m["roofline"],
            "phases_ms_last_step": {k: v for k, v in m["phases"].items() if k != "ms_numeric_bin"},
            "gpu_launches": int(m["launches"])}


def batched_subset_record(local: int, count: int = BATCH_SUBSET) -> dict:
    """A seeded subset of the batched workload's products (the first `count` of
    its 512, same size distribution) through one spg_multiply_batch call per
    step, against the same products one spg_multiply call each."""
    import spgemm_gb300 as sg
    pairs = make_workload("batched", count=count)
    products = sum(sg.scalar_products_host(a, b) for a, b in pairs)
    with sg.Engine(local) as eng:
        dev = [(a.to_device(local), b.to_device(local)) for a, b in pairs]

        def batched():
            for r in eng.multiply_batch(dev, out="device"):
                r.free()
            return eng.last_timings()["launches"]

        device_ms = []

        def one_by_one():
            launches = 0
            device_ms.clear()
            for a, b in dev:
                eng.multiply(a, b, out="device").free()
                t = eng.last_timings()
                launches += t["launches"]
                device_ms.append(t["ms_total"])
            return launches

        for _ in range(2):
            batched()
            one_by_one()
        reps = 3
        tb = sum(_wall(batched)[0] for _ in range(reps)) / reps
        ts = sum(_wall(one_by_one)[0] for _ in range(reps)) / reps
        lb, ls = batched(), one_by_one()
        kernels_ms = sum(device_ms)  # first to last event of each call, summed
    return {"workload": WORKLOADS["batched"] + f" [first {count} of {BATCH_PRODUCTS} products]",
            "products": count, "rows_total": int(sum(a.rows for a, _ in pairs)),
            "scalar_products_per_step": int(products), "steps": reps,
            "timing": "host wall clock between device synchronisations",
            "batched": {"value": 2.0 * products / tb / 1e9, "unit": "GFLOP/s", "ms_per_step": 1e3 * tb,
                        "gpu_launches_per_step": int(lb), "what": "one spg_multiply_batch call"},
            "per_product": {"value": 2.0 * products / ts / 1e9, "unit": "GFLOP/s", "ms_per_step": 1e3 * ts,
                            "gpu_launches_per_step": int(ls), "what": "one spg_multiply call per product",
                            "device_ms_per_step": kernels_ms,
                            "host_overhead_ms_per_step": 1e3 * ts - kernels_ms,
                            "ceiling_over_per_product": 1e3 * ts / kernels_ms if kernels_ms > 0 else None},
            "batched_over_per_product": ts / tb}


def served_subset_record(local: int, requests: int = 200, rate: float = 1000.0) -> dict:
    """The served stream, bounded: the full request pool, every request queued at
    once (saturation) and a Poisson trace at one rate, through continuous
    batching (3 lanes, batches of <= 256 requests / 2^27 scalar products) and
    through per-request launches (1 lane, batches of 1)."""
    import spgemm_gb300 as sg
    pool = make_workload("served")
    products = [sg.scalar_products_host(a, b) for a, b in pool]
    dev = [(a.to_device(local), b.to_device(local)) for a, b in pool]
    modes = {"batched": dict(lanes=3, max_batch=256, max_batch_products=1 << 27),
             "per_request": dict(lanes=1, max_batch=1)}
    out = {}
    for mode, kw in modes.items():
        with sg.Server(local, hbm_budget_bytes=150 * 10**9, **kw) as srv:
            _serve_trace(srv, dev, products, np.zeros(len(pool)), np.arange(len(pool)))  # warm-up
            _, picks = _arrivals(1.0, requests, len(pool), seed=7)
            sat = _serve_trace(srv, dev, products, np.zeros(requests), picks)
            at, picks = _arrivals(rate, requests, len(pool), seed=int(rate))
            paced = _serve_trace(srv, dev, products, at, picks)
        out[mode] = {"saturation": sat, f"poisson_{int(rate)}_req_per_s": paced}
    return {"workload": WORKLOADS["served"], "pool": len(pool), "requests_per_trace": requests,
            "modes": modes, "by_mode": out,
            "batched_over_per_request": out["batched"]["saturation"]["req_per_s"]
            / out["per_request"]["saturation"]["req_per_s"],
            "timing": "server-side submit-to-ready latency; span on the host clock"}


def run_gpu_arm(args, rank, world, local):
    import torch
    import spgemm_gb300 as sg
    torch.cuda.set_device(local)
    pairs = make_workload(args.workload, args.rows)
    if world > 1:
        # row sharding: this rank's block of A's rows (about P / world scalar
        # products, cut by the prefix of the row products) against all of B
        import sharding
        sharded = []
        for a, b in pairs:
            first = sharding.partition_rows(a, b, world)
            sharded.append((sharding.slice_rows(a, int(first[rank]), int(first[rank + 1] - first[rank])), b))
        pairs = sharded
    eng = sg.Engine(local)
    dev_pairs = []
    for a, b in pairs:
        da = a.to_device(local)
        db = da if b is a else b.to_device(local)
        dev_pairs.append((da, db))

    # bin autotuner (untimed setup): per-bin team shape chosen by measured time on this workload
    tuned = None
    if not args.no_tune:
        da, db = dev_pairs[0]
        tuned = eng.tune(da, db, reps=2)

    m = device_measure(eng, pairs, dev_pairs, args.steps, args.warmup, local, world)
    products, c_nnz = m["products"], m["c_nnz"]
    t_ms, launches, last_phases, clocks = m["t_ms"], m["launches"], m["phases"], m["clocks"]
    flush, in_bytes = m["flush"], m["in_bytes"]
    t_max = all_max(t_ms, world)
    total_products = all_sum(products * args.steps, world)
    value = 2.0 * total_products / (t_max / 1e3) / 1e9

    # e2e: host (pinned) operands in, host (pinned) result out, through the C ABI
    e2e = None
    if not args.no_e2e:
        host_pairs = []
        for a, b in pairs:
            pa = _pinned_csr(a)
            pb = pa if b is a else _pinned_csr(b)
            host_pairs.append((pa, pb))
        outs = [(_pinned_like(a.rows + 1, torch.int64), _pinned_like(n, torch.int32), _pinned_like(n, torch.float64))
                for (a, _), n in zip(pairs, c_nnz)]
        h2d = sum(_csr_bytes(a) + (0 if b is a else _csr_bytes(b)) for a, b in pairs)
        d2h = sum(8 * (a.rows + 1) + 12 * n for (a, _), n in zip(pairs, c_nnz))

        def e2e_step():
            # spg_multiply_to_host: row blocks whose device->host copies overlap the later blocks
            for (pa, pb), (orp, oci, ova) in zip(host_pairs, outs):
                eng.multiply_to_host(pa, pb, orp, oci, ova)
            return float(ova[0].item()) if ova.numel() else 0.0

        for _ in range(max(1, args.warmup)):
            e2e_step()
        ke = max(1, min(args.steps, args.e2e_steps))
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ke):
            e2e_step()
        torch.cuda.synchronize()
        te = all_max(time.perf_counter() - t0, world)
        e2e = {"value": 2.0 * all_sum(products * ke, world) / te / 1e9, "unit": "GFLOP/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": ke}

    # plan replay: the same products with their structure phases done once and the
    # value phases (numeric, scan, compaction) replayed as one CUDA graph per step
    replay = None
    if not args.no_replay:
        with eng.plan(dev_pairs) as plan:
            for _ in range(args.warmup):
                plan.execute()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            dev_ms = 0.0
            for _ in range(args.steps):
                plan.execute()
                dev_ms += plan.last_ms
            wall = time.perf_counter() - t0
        replay = {"value": 2.0 * products * args.steps / wall / 1e9, "unit": "GFLOP/s",
                  "ms_per_step": 1e3 * wall / args.steps, "device_ms_per_step": dev_ms / args.steps,
                  "what": "spg_plan_execute: numeric + scan + compaction of the same products replayed as one "
                          "CUDA graph per step; row work, bins and allocation done once at plan time"}

    traffic = None
    tf = ROOT / "profiles" / f"traffic_{args.workload}.json"
    if tf.exists() and not args.rows and world == 1:
        traffic = json.loads(tf.read_text()).get("dram_bytes_per_step")
    roofline = dict(m["roofline"])
    roofline["traffic"] = traffic

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        impl, kind = cpu_reference()
        threads = os.cpu_count() or 1
        a, b = pairs[0]
        first, n = cpu_sample_rows(impl, kind, a, b, threads)
        t, p = time_cpu_slice(impl, kind, a, b, first, n, threads)
        cpu = {"value": 2.0 * p / t / 1e9, "unit": "GFLOP/s", "cores": threads, "kind": kind,
               "sample": f"rows [{first}, {first + n}) of A x B ({n} of {a.rows} rows, {p} products, {t:.2f} s)"}

    subs = None
    if rank == 0 and world == 1 and not args.no_sub and args.workload == "powerlaw" and not args.rows:
        eng.close()
        eng = None
        subs = {name: sub_record(name, min(args.steps, 10), args.warmup, local) for name in ("uniform", "galerkin")}
        subs["batched_subset"] = batched_subset_record(local)
        subs["served_subset"] = served_subset_record(local)

    if rank == 0:
        line = {
            "metric": "GFLOP/s", "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOADS[args.workload] + (f" [rows={args.rows}]" if args.rows else ""),
                       "name": args.workload,
                       "products_per_step": int(products), "c_nnz": int(sum(c_nnz)),
                       "l2": ("L2 flushed between timed steps (512 MiB write outside the events)" if flush
                              else f"inputs larger than L2 ({in_bytes / 1e6:.0f} MB, no flush)"),
                       "parallelism": (f"row sharding x{world} (rows cut by the prefix of their scalar products, "
                                       "B replicated, no collective in the timed region)") if world > 1
                                      else "single GPU",
                       "bin_variants": tuned["variants"] if tuned else None},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches), "clocks": clocks, "graph_replay": replay,
            "phases_ms_last_step": last_phases, "workloads": subs,
        }
        print(json.dumps(line))
    if eng is not None:
        eng.close()


def _wall(fn):
    """Seconds of fn() between device synchronisations (work spread over the
    server's streams has no single stream to put events on)."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return time.perf_counter() - t0, out


def run_batched(args, rank, world, local):
    """512 uneven products: all submitted to the serving loop at once (waves
    formed by admission under the 150 GB budget, one launch per bin and phase
    per wave) against the same products multiplied one call at a time."""
    import torch
    import spgemm_gb300 as sg
    torch.cuda.set_device(local)
    pairs = make_workload("batched")
    products = [sg.scalar_products_host(a, b) for a, b in pairs]
    total_p = sum(products)
    dev = [(a.to_device(local), b.to_device(local)) for a, b in pairs]
    in_bytes = sum(_csr_bytes(a) + _csr_bytes(b) for a, b in pairs)

    def served(srv):
        tickets = [srv.submit(a, b) for a, b in dev]
        nnz, batches, launches = 0, {}, 0
        for t in tickets:
            st, res, info = srv.poll(t)
            if st != "SPG_OK":
                raise SystemExit(f"batched request failed: {st} {info}")
            nnz += res.nnz
            batches[info["batch_id"]] = (info["batch_requests"], info["batch_launches"])
            res.free()
        return nnz, batches

    srv = sg.Server(local, lanes=2, max_batch=BATCH_PRODUCTS, hbm_budget_bytes=150 * 10**9,
                    max_batch_products=BATCH_MAX_PRODUCTS)
    for _ in range(args.warmup):
        c_nnz, _ = served(srv)
    times, waves, launches = [], [], 0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            t, (_, batches) = _wall(lambda: served(srv))
            times.append(t)
            waves.append(sorted(n for n, _ in batches.values()))
            launches += sum(l for _, l in batches.values())
    srv.close()
    t_batched = sum(times)
    value = 2.0 * total_p * args.steps / t_batched / 1e9

    eng = sg.Engine(local)

    def one_by_one():
        launches = 0
        for a, b in dev:
            r = eng.multiply(a, b, out="device")
            launches += eng.last_timings()["launches"]
            r.free()
        return launches

    one_by_one()
    k1 = max(1, min(args.steps, 2))
    t_single = 0.0
    for _ in range(k1):
        t, _ = _wall(one_by_one)
        t_single += t
    single = 2.0 * total_p * k1 / t_single / 1e9
    eng.close()

    c_bytes_alg = sum(sg.algorithmic_bytes(a, b, p, 0) for (a, b), p in zip(pairs, products)) + 12 * c_nnz
    pk = peaks()
    achieved = c_bytes_alg / (t_batched / args.steps) / 1e9
    line = {
        "metric": "GFLOP/s", "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_batched / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOADS["batched"], "name": "batched", "products": len(pairs),
                   "rows_total": int(sum(a.rows for a, _ in pairs)), "scalar_products_per_step": int(total_p),
                   "c_nnz": int(c_nnz), "l2": f"inputs larger than L2 ({in_bytes / 1e9:.1f} GB, no flush)",
                   "timing": "host wall clock between device synchronisations (two lanes, two streams)",
                   "server": {"lanes": 2, "max_batch": BATCH_PRODUCTS, "hbm_budget_bytes": 150 * 10**9,
                              "max_batch_products": BATCH_MAX_PRODUCTS},
                   "waves_per_step": [len(w) for w in waves], "wave_sizes_last_step": waves[-1]},
        "per_product_launches": {"value": single, "unit": "GFLOP/s", "steps": k1,
                                 "ms_per_step": 1e3 * t_single / k1,
                                 "what": "the same 512 products, one spg_multiply call each"},
        "batched_over_per_product": value / single,
        "roofline": {"bound": "hbm", "kernel": "whole batched step", "achieved": achieved, "peak": pk["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / pk["hbm_gbs"], "peak_source": pk["source"],
                     "traffic": None, "bytes_alg": int(c_bytes_alg)},
        "cpu_baseline": None, "e2e": None, "gpu_launches": int(launches), "clocks": clocks.summary(),
    }
    if rank == 0:
        print(json.dumps(line))


def _arrivals(rate: float, n: int, pool_size: int, seed: int):
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n)), rng.integers(0, pool_size, size=n)


def _serve_trace(srv, dev, products, at, picks):
    """Submits pool requests at the given arrival times (seconds) from one
    thread while another collects them; returns per-request (latency ms) and
    the span from first submit to last completion."""
    n = len(at)
    tickets = [None] * n
    submit_t = [0.0] * n
    ready = threading.Semaphore(0)

    def submitter():
        t0 = time.perf_counter()
        for i in range(n):
            d = t0 + at[i] - time.perf_counter()
            if d > 0:
                time.sleep(d)
            a, b = dev[picks[i]]
            submit_t[i] = time.perf_counter()
            tickets[i] = srv.submit(a, b)
            ready.release()

    th = threading.Thread(target=submitter)
    th.start()
    lat, done_t, batch_sizes, launches, seen = [], [], [], 0, set()
    for i in range(n):
        ready.acquire()
        st, res, info = srv.poll(tickets[i])
        if st != "SPG_OK":
            raise SystemExit(f"served request failed: {st} {info}")
        res.free()
        lat.append(info["latency_ms"])
        done_t.append(submit_t[i] + info["latency_ms"] / 1e3)
        batch_sizes.append(info["batch_requests"])
        if info["batch_id"] not in seen:
            seen.add(info["batch_id"])
            launches += info["batch_launches"]
    th.join()
    span = max(done_t) - min(submit_t)
    p = sum(products[j] for j in picks)
    lat = np.asarray(lat)
    return {"requests": n, "req_per_s": n / span, "gflops": 2.0 * p / span / 1e9,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_batch": float(np.mean(batch_sizes)), "span_s": span, "launches": int(launches)}


def run_served(args, rank, world, local):
    """The served stream: one Poisson trace per rate, served by continuous
    batching (3 lanes, batches of up to 256 requests / 2^27 scalar products)
    and by per-request launches
    (1 lane, batches of 1), plus both at saturation (every request queued at
    once)."""
    import torch
    import spgemm_gb300 as sg
    torch.cuda.set_device(local)
    pool = make_workload("served")
    products = [sg.scalar_products_host(a, b) for a, b in pool]
    dev = [(a.to_device(local), b.to_device(local)) for a, b in pool]
    modes = {"batched": dict(lanes=3, max_batch=256, max_batch_products=1 << 27),
             "per_request": dict(lanes=1, max_batch=1)}
    n_sat = 300
    table = {m: {} for m in modes}
    with ClockSampler(local) as clocks:
        for mode, kw in modes.items():
            with sg.Server(local, hbm_budget_bytes=150 * 10**9, **kw) as srv:
                for w in range(args.warmup):  # every pool entry once per warm-up pass
                    _serve_trace(srv, dev, products, np.zeros(len(pool)), np.arange(len(pool)))
                at, picks = _arrivals(1.0, n_sat, len(pool), seed=7)
                table[mode]["saturation"] = _serve_trace(srv, dev, products, np.zeros(n_sat), picks)
                for rate in SERVE_RATES:
                    n = int(min(400, max(100, 3 * rate)))
                    at, picks = _arrivals(rate, n, len(pool), seed=rate)
                    table[mode][str(rate)] = _serve_trace(srv, dev, products, at, picks)
    # the whole pool as one plan: all 24 requests per CUDA-graph replay
    eng = sg.Engine(local)
    with eng.plan(dev) as plan:
        for _ in range(3):
            plan.execute()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = 10
        for _ in range(reps):
            plan.execute()
        wall = time.perf_counter() - t0
    eng.close()
    replay = {"req_per_s": reps * len(pool) / wall, "gflops": 2.0 * sum(products) * reps / wall / 1e9,
              "what": "the 24 pool requests as one spg_plan: value phases replayed as one CUDA graph per "
                      "24 requests (structure phases at plan time)"}
    sat_b, sat_p = table["batched"]["saturation"], table["per_request"]["saturation"]
    line = {
        "metric": "served products/s", "value": sat_b["req_per_s"], "unit": "products/s", "n_gpus": world,
        "steps": 1, "warmup": args.warmup, "ms_per_step": 1e3 * sat_b["span_s"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOADS["served"], "name": "served", "pool": len(pool),
                   "pool_products": [int(p) for p in products], "rates_req_per_s": list(SERVE_RATES),
                   "saturation_requests": n_sat, "timing": "server-side submit-to-ready latency; span on the host clock",
                   "modes": modes, "hbm_budget_bytes": 150 * 10**9},
        "gflops_saturation": sat_b["gflops"],
        "per_request_launches": {"value": sat_p["req_per_s"], "unit": "products/s", "gflops": sat_p["gflops"],
                                 "p50_ms": sat_p["p50_ms"], "p99_ms": sat_p["p99_ms"]},
        "batched_over_per_request": sat_b["req_per_s"] / sat_p["req_per_s"],
        "p50_ms": sat_b["p50_ms"], "p99_ms": sat_b["p99_ms"],
        "by_rate": table, "graph_replay": replay, "roofline": None, "cpu_baseline": None, "e2e": None,
        "gpu_launches": int(sum(v["launches"] for m in table.values() for v in m.values())),
        "clocks": clocks.summary(),
    }
    if rank == 0:
        print(json.dumps(line))


def _pinned_like(n, dtype):
    import torch
    return torch.empty(max(int(n), 1), dtype=dtype, pin_memory=True)


def _pinned_csr(a):
    import torch
    import spgemm_gb300 as sg
    rp = torch.from_numpy(a.row_ptr).pin_memory()
    ci = torch.from_numpy(a.col).pin_memory()
    va = torch.from_numpy(a.val).pin_memory()
    m = sg.Csr(a.rows, a.cols, rp.numpy(), ci.numpy(), va.numpy())
    m._keep = (rp, ci, va)
    return m


def _csr_bytes(a) -> int:
    return 8 * (a.rows + 1) + 12 * a.nnz


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="powerlaw")
    ap.add_argument("--rows", type=int, default=0, help="power-law rows (default 1048576; profiling only)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-replay", action="store_true", help="skip the plan-replay (CUDA graph) sub-measurement")
    ap.add_argument("--no-tune", action="store_true", help="keep the default team shape in every bin")
    ap.add_argument("--no-sub", action="store_true",
                    help="skip the uniform, Galerkin, batched-subset and served-subset records of the default line")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_init()
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
    elif args.workload == "batched":
        run_batched(args, rank, world, local)
    elif args.workload == "served":
        run_served(args, rank, world, local)
    else:
        run_gpu_arm(args, rank, world, local)


if __name__ == "__main__":
    main()
