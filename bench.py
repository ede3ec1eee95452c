"""Benchmark of the GB300 FFT path (prints ONE JSON line on rank 0).

Headline workload (the configuration the headline metric is quoted on):
batched 1D complex FP32 FFTs, n = 4096, batch = 16384 (split re/im, 512 MiB
per array pair), inputs i.i.d. standard normal from a seed; one step = the
forward transform of the batch followed by the inverse transform.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config c2|c1|c3a|c3b|c3c|c4|c5] [--form plain|tc|f64]

On one GPU the default run also measures every other configuration at full
size and adds it to the same line under "configs" (c1, c3a, c3b, c3c, c4,
c5): its time per step and per forward launch, GFLOP/s, algorithmic GB/s and
fraction of the measured HBM peak, the per-pass fraction, accuracy against an
FP64 FFT on a sample, and the CPU baseline.  c4 adds the split-precision
tensor-core form on both of its input sets; c5 adds the tensor-core form of
the queue, its ratio to the plain form, both forms' worst-transform error
against FP64 on a fixed sample of transforms, and the end-to-end step.

value      GFLOP/s by afft's convention (5 N log2 N complex, 2.5 N log2 N
           real, testing.cpp:1027), inputs resident in HBM, CUDA events on
           the launching stream, max over ranks.
e2e        the same metric through the C ABI with pinned HOST buffers: each
           call moves its input to the device and its result back (staged
           copies, or the kernels' own accesses over the host link when the
           plan touches each array once in wide segments).
roofline   the forward plan's algorithmic bytes (one read + one write of the
           data) / its time (CUDA events), against the measured HBM copy
           peak; "passes" divides the same time into what the plan's launches
           must move between them (each reads its input and writes its output
           once), i.e. how close multi-pass plans run to the peak per pass.
cpu_baseline  afft itself (the reference library built from its sources on
           this host: its best SIMD backend on x86-64, its scalar backend on
           Arm, where afft builds no other) through its own C API on all host
           threads, one plan per thread, over a bounded sample of the same
           workload; the oracle's FP32 port of afft where the library is not
           built.
--impl reference  times that CPU path alone (all host threads), same metric
           and the same config record.

Multi-GPU (torchrun): each rank transforms its own batch (no collective);
scaling is weak.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "GFLOP/s (5N·log2N) & HBM GB/s: TC-split+batched vs plain FP32 at rel-L2≤5e-6"

CONFIGS = {
    # name: (kind, dims, batch, description, inverse_too, input distribution)
    "c1": ("c", [1024], 1, "1D c2c n=1024 fwd + inv (latency)", True, "uniform"),
    "c2": ("c", [4096], 16384, "batched 1D c2c n=4096 x 16384, fwd + inv", True, "normal"),
    "c3a": ("c", [256, 256, 256], 1, "3D c2c 256^3 fwd + inv", True, "uniform"),
    "c3b": ("r", [4096, 4096], 1, "2D r2c 4096^2 + c2r", True, "normal"),
    "c3c": ("r", [1 << 20], 64, "64 x 1D r2c n=2^20 + c2r", True, "normal"),
    "c4": ("c", [65536], 4096, "batched 1D c2c n=65536 x 4096 fwd", False, "uniform"),
    "c5": ("queue", None, 10000, "uneven batch: 10000 transforms, 1D 2^6-2^18 / 2D 2^6-2^11 / 3D 2^5-2^8, "
           "50% real, 50% inverse, one graph-captured queue", False, "normal"),
}
SUB_ORDER = ["c1", "c3a", "c3b", "c3c", "c4", "c5"]
DATA = "synthetic: seeded inputs with the configuration's shape and distribution (config.inputs)"
DIST_TEXT = {"uniform": "seeded uniform[-1,1)", "normal": "seeded standard normal",
             "spread": "seeded log-uniform magnitudes over 1e-4..1, uniform phase"}

FORMS = {"plain": "plain FP32 Stockham",
         "tc": "split-precision tensor cores (tcgen05 DFT-16, FP16 hi+lo, FP32 accumulate) where eligible",
         "f64": "FP64 data and arithmetic (afft_64_*): radix-8 Stockham FP64 kernels"}

# GB300's nominal FP64 rate (GFLOP/s); MEASURED_PEAKS.json has no FP64 figure
FP64_NOMINAL_GFLOPS = 1250.0
# GB300 L2 capacity (bytes)
L2_BYTES = 129e6


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(cfg):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/traffic.json) and how it was taken, or (None, None)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            d = json.load(f)[cfg]
        return d["dram_bytes_per_launch"], "committed ncu capture (profiles/traffic.json): " + d["how"]
    except Exception:
        return None, None


def flops_of(kind, dims, batch):
    n = int(np.prod(dims))
    c = 5.0 if kind in ("c", "ci") else 2.5
    return c * n * math.log2(n) * batch if n > 1 else 0.0


def bytes_of(kind, dims, batch, esize=4):
    """Algorithmic bytes of one transform pass: one read + one write
    (esize bytes per real value: 4 for FP32, 8 for FP64)."""
    n = int(np.prod(dims))
    d = [x for x in dims if x != 1] or [1]
    h = (d[0] // 2 + 1) * (n // d[0])
    if kind in ("c", "ci"):
        return 4 * esize * n * batch
    return (esize * n + 2 * esize * h) * batch


def config_record(cfg, args, world=1):
    """The config dict of a bench line; both arms print the same one."""
    kind, dims, batch, desc, with_inv, dist = CONFIGS[cfg]
    if args.batch and kind != "queue":
        batch = args.batch
        desc = desc + " (batch overridden to %d)" % batch
    if kind == "queue":
        return {"workload": desc, "transforms": args.batch or batch, "form": FORMS[args.form],
                "inputs": DIST_TEXT[dist], "parallelism": "dp%d (independent batches)" % world}
    esize = 8 if args.form == "f64" else 4
    sb = bytes_of(kind, dims, batch, esize) * (2 if with_inv else 1)
    return {"workload": desc, "kind": kind, "dims": dims, "batch_per_gpu": batch, "form": FORMS[args.form],
            "inputs": DIST_TEXT[dist],
            "l2": "L2 flushed before each timed step (512 MiB write, outside the step's events)"
            if sb < 3 * L2_BYTES else "inputs larger than L2 (%d MiB per array pair)"
            % (bytes_of(kind, dims, batch, esize) // 2 >> 20),
            "parallelism": "dp%d (independent batches)" % world}


class ClockSampler:
    """nvidia-smi sampled every 100 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
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
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def rank_seed(rank):
    """Each rank transforms its own batch: a distinct input seed per rank."""
    return 1234 + rank


def fp64_reference(kind, dims, a, b=None):
    """numpy's float64 FFT with afft's conventions for one transform
    (unnormalised inverses; real transforms halve dims[0]; the real inverse
    reads the real parts of planes 0 and d0/2 only, as pocketfft's c2r does
    after the inverse transform of the other axes)."""
    d = [x for x in dims if x != 1] or [1]
    nd = len(d)
    n = int(np.prod(d))
    axes = list(range(1, nd)) + [0]     # the halved axis last, as numpy's real FFTs want
    if kind in ("c", "ci"):
        x = (a + 1j * b).reshape(d)
        y = np.fft.fftn(x) if kind == "c" else np.fft.ifftn(x) * n
        return y.reshape(-1)
    if kind == "r":
        return np.fft.rfftn(a.reshape(d), axes=axes).reshape(-1)
    h = [d[0] // 2 + 1] + d[1:]
    x = (a + 1j * b).reshape(h)
    s = [d[i] for i in axes]
    return np.fft.irfftn(x, s=s, axes=axes).reshape(-1) * n


def errors(y, ref):
    return {"rel_l2": float(np.linalg.norm(y - ref) / max(np.linalg.norm(ref), 1e-300)),
            "max_err": float(np.abs(y - ref).max() / max(np.abs(ref).max(), 1e-300))}


def accuracy(kind, dims, batch, src, mid, back, with_inv):
    """Relative L2 and max error (max |y - ref| / max |ref|) of the forward
    outputs of a sample of the batch against numpy's float64 FFT, and of the
    unnormalised round trip inverse(forward(x)) / n against x."""
    n = int(np.prod(dims))
    d = [x for x in dims if x != 1] or [1]
    h = (d[0] // 2 + 1) * (n // d[0])
    k = max(1, min(batch, (1 << 22) // max(n, 1)))   # transforms in the sample
    x = src[0][:k * n].double().cpu().numpy()
    if kind == "c":
        x = x + 1j * src[1][:k * n].double().cpu().numpy()
    shape = [k] + list(d)
    ref = np.fft.fftn(x.reshape(shape), axes=list(range(1, len(shape))))
    if kind != "c":
        ref = ref[:, :d[0] // 2 + 1]
    m = h if kind != "c" else n
    y = mid[0][:k * m].double().cpu().numpy() + 1j * mid[1][:k * m].double().cpu().numpy()
    ref = ref.reshape(-1)
    # afft's own harness metric (testing.cpp:1113-1129) beside the standard ones
    afft_metric = float(np.sqrt(np.sum(np.abs(y - ref) ** 2) / np.sum(np.abs(y) ** 2 + np.abs(ref) ** 2)))
    out = dict(sample="%d of %d transforms" % (k, batch), reference="numpy float64 FFT", **errors(y, ref),
               afft_metric=afft_metric, afft_bound=1.2e-7 * math.sqrt(max(math.log2(int(np.prod(d))), 1.0)))
    if with_inv:
        xb = back[0][:k * n].double().cpu().numpy()
        if kind == "c":
            xb = xb + 1j * back[1][:k * n].double().cpu().numpy()
        xb = xb / n
        out["round_trip_rel_l2"] = float(np.linalg.norm(xb - x) / np.linalg.norm(x))
    return out


def fill(t, dist, g):
    import torch
    if dist == "uniform":
        t.uniform_(-1.0, 1.0, generator=g)
    elif dist == "normal":
        t.normal_(generator=g)
    else:
        raise ValueError(dist)
    return t


def make_inputs(kind, dims, batch, seed, dev, dtype=None, dist="normal"):
    import torch
    dtype = dtype or torch.float32
    n = int(np.prod(dims))
    d = [x for x in dims if x != 1] or [1]
    h = (d[0] // 2 + 1) * (n // d[0])
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    m = n * batch
    E = lambda k: torch.empty(k, device=dev, dtype=dtype)
    if kind == "c":
        a = fill(E(m), dist, g)
        b = fill(E(m), dist, g)
        return (a, b), (E(m), E(m)), (E(m), E(m))
    # real: x -> half spectrum -> x
    a = fill(E(m), dist, g)
    return (a,), (E(h * batch), E(h * batch)), (E(m),)


def spread_inputs(m, seed, dev):
    """C4's second input set: magnitudes 10^U(-4,0), phases U(0, 2 pi)."""
    import torch
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    mag = torch.pow(10.0, torch.empty(m, device=dev).uniform_(-4.0, 0.0, generator=g))
    ph = torch.empty(m, device=dev).uniform_(0.0, 2 * math.pi, generator=g)
    return (mag * torch.cos(ph)).contiguous(), (mag * torch.sin(ph)).contiguous()


# ---------------------------------------------------------------- CPU legs

def cpu_rate(kind, dims, batch_total, threads, budget_s, f64=False):
    """GFLOP/s of the CPU path on `threads` host threads over a bounded
    sample of the workload (forward + inverse per transform): afft itself
    when its library is built here, else the oracle's port of afft.
    Returns (rate, sample text, threads used, kind, description)."""
    from oracle import oracle as O
    vt = np.float64 if f64 else np.float32
    ref = None if f64 else O.ref_bench_lib()
    if ref is not None:
        fwd = O.RefBatch(kind, dims, threads)
        inv = O.RefBatch("ci" if kind == "c" else "ri", dims, threads)
        what, ck = ref[2], "reference"
    else:
        Port = O.Port64 if f64 else O.Port32
        fwd = Port(kind, dims)
        inv = Port("ci" if kind == "c" else "ri", dims)
        what, ck = ("FP64" if f64 else "FP32") + " port of afft (oracle/afft_port.inc)", "port"
    rng = np.random.default_rng(0)
    # sample size: grow until a pass takes >= budget/4, capped by the workload
    # (a single transform runs on one thread, as afft's own calls do)
    sample = max(1, min(threads, batch_total))
    while True:
        a = rng.standard_normal(fwd.in_elems * sample).astype(vt)
        b = None if kind == "r" else rng.standard_normal(fwd.in_elems * sample).astype(vt)
        used = min(threads, sample)
        t0 = time.perf_counter()
        out = fwd(a, b, batch=sample, threads=used)
        inv(out[0], out[1], batch=sample, threads=used)
        dt = time.perf_counter() - t0
        if dt >= budget_s / 4 or sample >= batch_total:
            break
        sample = min(batch_total, sample * 4)
    # timed repeats filling the budget
    reps = max(1, int(budget_s / max(dt, 1e-6)))
    t0 = time.perf_counter()
    for _ in range(reps):
        out = fwd(a, b, batch=sample, threads=used)
        inv(out[0], out[1], batch=sample, threads=used)
    dt = time.perf_counter() - t0
    fl = 2 * flops_of(kind, dims, sample) * reps
    return (fl / dt / 1e9, "%d of %d transforms (fwd+inv) x %d reps, %.1f s" % (sample, batch_total, reps, dt),
            used, ck, what)


def cpu_mixed_rate(items, threads, budget_s, seed=0):
    """GFLOP/s of the CPU path over a bounded random sample of the mixed
    batch, each transform its own call, host threads taking them in turn:
    afft itself when built here, else the oracle's FP32 port."""
    from oracle import oracle as O
    from fft_gb300 import uneven as U
    rng = np.random.default_rng(seed)
    order = [int(j) for j in rng.permutation(len(items))]
    ref = O.ref_bench_lib()
    work, nbytes = [], 0

    def add(j):
        nonlocal nbytes
        kind, dims = items[j]
        i, o = U.elems(kind, dims)
        a = rng.standard_normal(i).astype(np.float32)
        b = None if kind == "r" else rng.standard_normal(i).astype(np.float32)
        oa = np.empty(o, np.float32)
        ob = None if kind == "ri" else np.empty(o, np.float32)
        nbytes += U.bytes_moved(kind, dims)
        work.append((kind, dims, a, b, oa, ob))

    if ref is not None:
        runner = O.RefMixed(threads)
        what, ck = ref[2], "reference"

        def run():
            runner.prepare(work)
            t0 = time.perf_counter()
            runner.run()
            return time.perf_counter() - t0
    else:
        from concurrent.futures import ThreadPoolExecutor
        plans = {}
        pool = ThreadPoolExecutor(threads)
        what, ck = "FP32 port of afft (oracle/afft_port.inc)", "port"

        def run():
            for w in work:
                if (w[0], tuple(w[1])) not in plans:
                    plans[(w[0], tuple(w[1]))] = O.Port32(w[0], w[1])
            t0 = time.perf_counter()
            list(pool.map(lambda w: plans[(w[0], tuple(w[1]))](w[2], w[3], out=(w[4], w[5])), work))
            return time.perf_counter() - t0
    # grow the sample until one pass takes >= budget/4 (or 2 GB of data, or all)
    while True:
        for j in order[len(work):len(work) + 64]:
            add(j)
        dt = run()
        if dt >= budget_s / 4 or nbytes > 2e9 or len(work) >= len(items):
            break
    reps = max(1, int(budget_s / max(dt, 1e-6)))
    dt = sum(run() for _ in range(reps))
    fl = sum(U.flops(w[0], w[1]) for w in work) * reps
    return (fl / dt / 1e9, "%d of %d transforms (random sample, seed %d) x %d reps, %.1f s" % (
        len(work), len(items), seed, reps, dt), threads, ck, what)


def cpu_record(rate, sample, used, ck, what):
    return {"value": round(rate, 3), "unit": "GFLOP/s", "cores": used, "kind": ck, "impl": what, "sample": sample}


def run_reference(args, cfg):
    world, rank, _ = dist_env()
    kind, dims, batch, desc, _, _ = CONFIGS[cfg]
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # bounded: each step is a sample of the workload sized to ~1-3 s
    rates = []
    f64 = args.form == "f64"
    for i in range(args.warmup + args.steps):
        if kind == "queue":
            from fft_gb300 import uneven as U
            r = cpu_mixed_rate(U.uneven_batch(args.batch or batch, seed=5), threads, budget_s=1.5)
        else:
            r = cpu_rate(kind, dims, args.batch or batch, threads, budget_s=1.5, f64=f64)
        if i >= args.warmup:
            rates.append(r[0])
    value = statistics.median(rates)
    line = {"metric": METRIC, "value": round(value, 3), "unit": "GFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if f64 else "f32", "data": DATA, "impl": "reference",
            "config": config_record(cfg, args, world),
            "cpu_baseline": cpu_record(value, r[1], r[2], r[3], r[4]),
            "e2e": {"value": round(value, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU legs

def measure_plan(args, cfg, dev, stream, world=1, rank=0, steps=None, soak=None, batch=None, headline=False):
    """One configuration's batched plans, timed with CUDA events on `stream`.
    Returns a record with the timings, roofline, accuracy and (headline
    only) the timed buffers for the further legs."""
    import torch
    import fft_gb300 as G
    kind, dims, cbatch, desc, with_inv, dist = CONFIGS[cfg]
    batch = batch or cbatch
    steps = steps or args.steps
    soak = args.soak if soak is None else soak
    form = None if args.form == "plain" else args.form
    f64 = args.form == "f64"
    dtype = torch.float64 if f64 else torch.float32
    esize = 8 if f64 else 4
    fwd = G.BatchPlan(kind, dims, batch, form=form)
    inv = G.BatchPlan("ci" if kind == "c" else "ri", dims, batch, form=form) if with_inv else None
    src, mid, back = make_inputs(kind, dims, batch, rank_seed(rank), dev, dtype, dist)
    torch.cuda.synchronize()

    def launch_fwd():
        if kind == "c":
            fwd.launch(src[0], src[1], mid[0], mid[1], stream)
        else:
            fwd.launch(src[0], None, mid[0], mid[1], stream)

    def launch_inv():
        if kind == "c":
            inv.launch(mid[0], mid[1], back[0], back[1], stream)
        else:
            inv.launch(mid[0], mid[1], back[0], None, stream)

    def step():
        launch_fwd()
        if inv:
            launch_inv()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 3)):
        step()
    barrier()
    # a step whose data is not several times larger than L2 would run from L2:
    # write a 512 MiB buffer on the same stream before every timed step,
    # outside the step's own events
    sb = bytes_of(kind, dims, batch, esize) * (2 if inv else 1)
    flush = torch.empty((512 << 20) // 4, dtype=torch.float32, device=dev) if sb < 3 * L2_BYTES else None
    # timed region: events around every launch of the dominant (forward) plan,
    # around every step, and around the whole region
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    es = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        # untimed soak of the same steps so the 100 ms clock samples cover the
        # load state of the timed region (which may last only milliseconds)
        time.sleep(0.3)
        t_soak = time.perf_counter()
        while time.perf_counter() - t_soak < soak:
            for _ in range(10):
                step()
            torch.cuda.synchronize()
        barrier()
        t_start.record(stream)
        for i in range(steps):
            if flush is not None:
                with torch.cuda.stream(stream):
                    flush.fill_(float(i))
            es[i][0].record(stream)
            ev[i][0].record(stream)
            launch_fwd()
            ev[i][1].record(stream)
            if inv:
                launch_inv()
            es[i][1].record(stream)
        t_end.record(stream)
        barrier()
    # with flushes, the steps' own events; else the whole region
    total_ms = sum(a.elapsed_time(b) for a, b in es) if flush is not None else t_start.elapsed_time(t_end)
    fwd_ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_step = total_ms / steps
    per_step_flops = flops_of(kind, dims, batch) * (2 if inv else 1)
    value = per_step_flops * world / (ms_step / 1e3) / 1e9
    torch.cuda.synchronize()
    acc = accuracy(kind, dims, batch, src, mid, back, inv is not None) if rank == 0 else None
    hbm, peak_src = peaks()
    alg_bytes = bytes_of(kind, dims, batch, esize)
    achieved = alg_bytes / (fwd_ms / 1e3) / 1e9
    # the same time against what the plan's passes must move between them
    # (each launch reads its input and writes its output once)
    pb = G.pass_bytes(G.describe(kind, dims, batch, G.FORM_F64 if f64 else 0)) * esize // 4
    passes = {"launches": fwd.launches, "bytes": pb, "achieved": round(pb / (fwd_ms / 1e3) / 1e9, 1),
              "frac": round(pb / (fwd_ms / 1e3) / 1e9 / hbm, 4), "unit": "GB/s"}
    kernel = "forward plan (%d launch%s), %.4f ms per launch" % (fwd.launches, "es" if fwd.launches > 1 else "",
                                                                  fwd_ms / fwd.launches)
    if f64:
        # FP64 arithmetic, not HBM, bounds the FP64 kernels on GB300
        fwd_gflops = flops_of(kind, dims, batch) / (fwd_ms / 1e3) / 1e9
        roofline = {"bound": "fp64", "achieved": round(fwd_gflops, 1), "peak": FP64_NOMINAL_GFLOPS,
                    "unit": "GFLOP/s", "frac": round(fwd_gflops / FP64_NOMINAL_GFLOPS, 4), "traffic": None,
                    "peak_source": "nominal (no measured FP64 figure)", "kernel": kernel,
                    "hbm": {"achieved": round(achieved, 1), "peak": hbm, "frac": round(achieved / hbm, 4),
                            "unit": "GB/s"},
                    "passes": passes}
    else:
        roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(achieved / hbm, 4), "traffic": None, "peak_source": peak_src,
                    "kernel": kernel, "passes": passes}
    rec = {"value": round(value, 2), "unit": "GFLOP/s", "ms_per_step": round(ms_step, 4),
           "ms_per_launch": round(fwd_ms / fwd.launches, 5), "fwd_ms": round(fwd_ms, 5),
           "gbs_algorithmic": round(achieved, 1), "roofline": roofline, "accuracy": acc,
           "gpu_launches": (fwd.launches + (inv.launches if inv else 0)) * steps,
           "clocks": dict(clk.summary(), window="soak %.1f s + timed region" % soak)}
    if cfg == "c1":
        rec["us_per_launch"] = round(1e3 * fwd_ms / fwd.launches, 2)
    if headline:
        rec["_bufs"] = (src, mid, back, per_step_flops, ms_step, with_inv, form, dtype)
    return rec


def tc_form_rate(kind, dims, batch, with_inv, src, mid, back, stream, per_step_flops, plain_ms, steps=20):
    """Same steps with the split-precision tensor-core form (AFFT_GB300_FORM_TC):
    its rate, its ratio to the plain form, and its accuracy against numpy's
    float64 FFT on a sample of transforms."""
    import torch
    import fft_gb300 as G
    if kind != "c":
        return None
    fwd = G.BatchPlan("c", dims, batch, form="tc")
    inv = G.BatchPlan("ci", dims, batch, form="tc") if with_inv else None

    def step():
        fwd.launch(src[0], src[1], mid[0], mid[1], stream)
        if inv:
            inv.launch(mid[0], mid[1], back[0], back[1], stream)
    for _ in range(3):
        step()
    torch.cuda.synchronize()
    acc = accuracy(kind, dims, batch, src, mid, back, with_inv)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"value": round(per_step_flops / (ms / 1e3) / 1e9, 2), "unit": "GFLOP/s", "ms_per_step": round(ms, 4),
            "ratio_to_plain": round(plain_ms / ms, 3), "accuracy": acc,
            "launches_per_step": fwd.launches + (inv.launches if inv else 0),
            "note": "tcgen05 DFT-16 stages, FP16 hi+lo operands, FP32 accumulation in TMEM; "
                    "tensor-pipe utilisation in profiles/line_fft_256_cols_tc_c4.md"}


def e2e_rate(args, kind, dims, batch, src, world, form=None, dtype=None):
    """Same metric through the C ABI's synchronous calls with pinned host
    buffers: every call copies its input to the device and its result back."""
    import torch
    import fft_gb300 as G
    dtype = dtype or torch.float32
    es = 8 if dtype == torch.float64 else 4
    fwd = G.BatchPlan(kind, dims, batch, form=form)
    inv = G.BatchPlan("ci" if kind == "c" else "ri", dims, batch, form=form)
    n = int(np.prod(dims))
    d = [x for x in dims if x != 1] or [1]
    h = (d[0] // 2 + 1) * (n // d[0])
    m = n * batch
    pin = lambda k: torch.empty(k, dtype=dtype).pin_memory()
    if kind == "c":
        a, b = pin(m), pin(m)
        a.copy_(src[0].cpu())
        b.copy_(src[1].cpu())
        o1, o2, r1, r2 = pin(m), pin(m), pin(m), pin(m)

        def step():
            fwd(a, b, o1, o2)
            inv(o1, o2, r1, r2)
        h2d = 2 * (2 * m * es)
        d2h = 2 * (2 * m * es)
    else:
        a = pin(m)
        a.copy_(src[0].cpu())
        o1, o2, r1 = pin(h * batch), pin(h * batch), pin(m)

        def step():
            fwd(a, o1, o2)
            inv(o1, o2, r1)
        h2d = es * m + 2 * es * h * batch
        d2h = 2 * es * h * batch + es * m
    steps = max(2, min(args.steps, 5))
    step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    dt = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([dt], device=torch.device("cuda", torch.cuda.current_device()))
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dt = float(t.item())
    val = 2 * flops_of(kind, dims, batch) * world * steps / dt / 1e9
    return {"value": round(val, 2), "unit": "GFLOP/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": steps}


def queue_accuracy(items, buf, offs, sample_idx):
    """Worst-transform and overall rel-L2 / max error of a queue's outputs
    against numpy's float64 FFT over the transforms in sample_idx."""
    from fft_gb300 import uneven as U
    worst_l2, worst_max, num, den = 0.0, 0.0, 0.0, 0.0
    for j in sample_idx:
        kind, dims = items[j]
        rec = offs[j]
        i, o = U.elems(kind, dims)
        a = buf[rec[0]:rec[0] + i].double().cpu().numpy()
        b = None if rec[1] is None else buf[rec[1]:rec[1] + i].double().cpu().numpy()
        ref = fp64_reference(kind, dims, a, b)
        y = buf[rec[2]:rec[2] + o].double().cpu().numpy()
        if rec[3] is not None:
            y = y + 1j * buf[rec[3]:rec[3] + o].double().cpu().numpy()
        e = errors(y, ref)
        worst_l2 = max(worst_l2, e["rel_l2"])
        worst_max = max(worst_max, e["max_err"])
        num += float(np.sum(np.abs(y - ref) ** 2))
        den += float(np.sum(np.abs(ref) ** 2))
    return {"transforms": len(sample_idx), "reference": "numpy float64 FFT, transform by transform",
            "worst_transform_rel_l2": worst_l2, "worst_transform_max_err": worst_max,
            "rel_l2": (num / den) ** 0.5}


def measure_queue(args, cfg, dev, steps=None, soak=None, cpu=True, e2e=True, tc=True):
    """The mixed batch as one queue run per step (device-resident data)."""
    import torch
    import fft_gb300 as G
    from fft_gb300 import uneven as U
    steps = steps or args.steps
    soak = args.soak if soak is None else soak
    items = U.uneven_batch(args.batch or CONFIGS[cfg][2], seed=5)
    buf, offs, boundary = U.allocate(items, dev, io_regions=True)
    q = G.Queue(U.descs(items, buf, offs), form=None if args.form == "plain" else args.form)
    stream = torch.cuda.Stream(device=dev)
    for _ in range(max(args.warmup, 3)):
        q.run(stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        time.sleep(0.3)
        t_soak = time.perf_counter()
        while time.perf_counter() - t_soak < soak:
            q.run(stream)
            torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            q.run(stream)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    fl = sum(U.flops(k, d) for k, d in items)
    by = sum(U.bytes_moved(k, d) for k, d in items)
    hbm, peak_src = peaks()
    # a fixed sample of transforms (seeded), checked against FP64 for both forms
    sample_idx = sorted(int(j) for j in np.random.default_rng(77).choice(len(items), min(256, len(items)),
                                                                          replace=False))
    acc = queue_accuracy(items, buf, offs, sample_idx)

    # the split-precision tensor-core form of the same queue on the same data
    tcrec = None
    if tc and args.form == "plain":
        qt = G.Queue(U.descs(items, buf, offs), form="tc")
        for _ in range(3):
            qt.run(stream)
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(steps):
            qt.run(stream)
        t1.record(stream)
        torch.cuda.synchronize()
        ms_tc = t0.elapsed_time(t1) / steps
        tcrec = {"value": round(fl / (ms_tc / 1e3) / 1e9, 2), "unit": "GFLOP/s", "ms_per_step": round(ms_tc, 4),
                 "transforms_per_s": round(len(items) / (ms_tc / 1e3), 1), "ratio_to_plain": round(ms / ms_tc, 3),
                 "accuracy": queue_accuracy(items, buf, offs, sample_idx), "launches_per_step": qt.launches,
                 "note": "tcgen05 DFT-16 stages where eligible (radix-16 stages of 256- and 4096-point passes), "
                         "FP16 hi+lo operands, FP32 accumulation in TMEM; other passes plain FP32"}
        del qt
        q.run(stream)           # leave the plain form's outputs in place
        torch.cuda.synchronize()

    # the same queue with the autotuner's per-shape choices (each distinct
    # shape tuned on this device when the queue is created)
    tunedrec = None
    if tc and args.form == "plain" and not args.no_tune:
        t0 = time.perf_counter()
        qq = G.Queue(U.descs(items, buf, offs), tuned=True)
        tune_s = time.perf_counter() - t0
        for _ in range(3):
            qq.run(stream)
        torch.cuda.synchronize()
        t0e, t1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0e.record(stream)
        for _ in range(steps):
            qq.run(stream)
        t1e.record(stream)
        torch.cuda.synchronize()
        ms_tuned = t0e.elapsed_time(t1e) / steps
        tunedrec = {"ms_per_step": round(ms_tuned, 4), "transforms_per_s": round(len(items) / (ms_tuned / 1e3), 1),
                    "untuned_ms_per_step": round(ms, 4), "ratio_to_untuned": round(ms / ms_tuned, 3),
                    "tuning_s": round(tune_s, 1), "launches_per_step": qq.launches,
                    "accuracy": queue_accuracy(items, buf, offs, sample_idx),
                    "note": "each distinct (kind, shape) tuned at a batch of about 2^24 elements: four-step split, "
                            "real pre-pass placement, TMA or LSU tile loads, cols tile width, plain or "
                            "tensor-core form"}
        del qq
        q.run(stream)           # leave the plain form's outputs in place
        torch.cuda.synchronize()

    # end to end: every step copies all inputs from pinned host memory, runs
    # the queue and copies all outputs back (one copy each way: the inputs
    # and the outputs occupy two contiguous regions).  Steps are pipelined the
    # way a stream of batches runs: the copy in of step i (after queue i-1 has
    # read the inputs) overlaps the copy out of step i-1, on their own streams
    # (the host link carries both directions at once); queue i waits for both.
    e2erec = None
    if e2e:
        in_host = torch.empty(boundary, dtype=torch.float32).pin_memory()
        out_host = torch.empty(buf.numel() - boundary, dtype=torch.float32).pin_memory()
        in_host.copy_(buf[:boundary])
        esteps = max(2, min(steps, 4))
        s_in, s_out = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)

        def e2e_run(n):
            q_done = torch.cuda.Event()
            q_done.record(stream)
            for i in range(n):
                s_in.wait_event(q_done)                  # queue i-1 has read the inputs
                with torch.cuda.stream(s_in):
                    buf[:boundary].copy_(in_host, non_blocking=True)
                in_done = torch.cuda.Event()
                in_done.record(s_in)
                stream.wait_event(in_done)
                stream.wait_stream(s_out)                # copy out of step i-1 is done
                q.run(stream)
                q_done = torch.cuda.Event()
                q_done.record(stream)
                s_out.wait_event(q_done)
                with torch.cuda.stream(s_out):
                    out_host.copy_(buf[boundary:], non_blocking=True)
            torch.cuda.synchronize()
        e2e_run(1)
        t0 = time.perf_counter()
        e2e_run(esteps)
        dt = (time.perf_counter() - t0) / esteps
        e2erec = {"value": round(fl / dt / 1e9, 2), "unit": "GFLOP/s", "h2d_bytes_per_step": 4 * boundary,
                  "d2h_bytes_per_step": 4 * (buf.numel() - boundary), "steps": esteps,
                  "ms_per_step": round(dt * 1e3, 3),
                  "note": "steps pipelined: copy in of step i overlaps copy out of step i-1"}
        del in_host, out_host
    cpurec = None
    if cpu:
        cpurec = cpu_record(*cpu_mixed_rate(items, os.cpu_count() or 1, args.sub_cpu_budget))
    rec = {"value": round(fl / (ms / 1e3) / 1e9, 2), "unit": "GFLOP/s", "ms_per_step": round(ms, 4),
           "transforms_per_s": round(len(items) / (ms / 1e3), 1), "algorithmic_bytes": by,
           "gbs_algorithmic": round(by / (ms / 1e3) / 1e9, 1), "queue_launches": q.launches,
           "roofline": {"bound": "hbm", "achieved": round(by / (ms / 1e3) / 1e9, 1), "peak": hbm, "unit": "GB/s",
                        "frac": round(by / (ms / 1e3) / 1e9 / hbm, 4), "traffic": None, "peak_source": peak_src,
                        "kernel": "whole queue (graph of %d launches)" % q.launches},
           "accuracy": acc, "tc_split_form": tcrec, "autotuned": tunedrec, "e2e": e2erec, "cpu_baseline": cpurec,
           "gpu_launches": q.launches * steps,
           "clocks": dict(clk.summary(), window="soak %.1f s + timed region" % soak)}
    del q, buf
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return rec


def sub_record(args, cfg, dev):
    """One configuration at full size for the "configs" part of the line."""
    import torch
    steps = min(args.steps, 20)
    if CONFIGS[cfg][0] == "queue":
        rec = measure_queue(args, cfg, dev, steps=steps, soak=0.5)
    else:
        stream = torch.cuda.Stream(device=dev)
        rec = measure_plan(args, cfg, dev, stream, steps=steps, soak=0.5, headline=(cfg == "c4"))
        kind, dims, batch, _, with_inv, _ = CONFIGS[cfg]
        if cfg == "c4" and args.form == "plain":
            # the split-precision form on C4's two input sets: uniform[-1,1)
            # (the plain run's inputs) and magnitudes spread over 1e-4
            import fft_gb300 as G
            src, mid, back, psf, ms_step, _, _, _ = rec.pop("_bufs")
            tcr = tc_form_rate(kind, dims, batch, with_inv, src, mid, back, stream, psf, ms_step, steps=steps)
            a, b = spread_inputs(src[0].numel(), 4, dev)
            src[0].copy_(a)
            src[1].copy_(b)
            del a, b
            for where, form in ((rec, None), (tcr, "tc")):
                G.BatchPlan("c", dims, batch, form=form).launch(src[0], src[1], mid[0], mid[1], stream)
                torch.cuda.synchronize()
                where["accuracy_spread_set"] = accuracy(kind, dims, batch, src, mid, back, False)
            rec["tc_split_form"] = tcr
            del src, mid, back
        rec.pop("_bufs", None)
        if not args.no_cpu:
            rec["cpu_baseline"] = cpu_record(*cpu_rate(kind, dims, batch, os.cpu_count() or 1, args.sub_cpu_budget))
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    rec["config"] = config_record(cfg, args)
    return rec


def run_ours(args, cfg):
    import torch

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)

    if CONFIGS[cfg][0] == "queue":
        rec = measure_queue(args, cfg, dev, cpu=not args.no_cpu, e2e=not args.no_e2e, tc=not args.no_tc)
        line = {"metric": METRIC, "value": rec["value"], "unit": "GFLOP/s", "n_gpus": 1, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": rec["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": DATA,
                "config": config_record(cfg, args), "roofline": rec["roofline"], "cpu_baseline": rec["cpu_baseline"],
                "e2e": rec["e2e"], "accuracy": rec["accuracy"], "tc_split_form": rec["tc_split_form"],
                "autotuned": rec["autotuned"],
                "transforms_per_s": rec["transforms_per_s"], "queue_launches": rec["queue_launches"],
                "gpu_launches": rec["gpu_launches"], "clocks": rec["clocks"]}
        print(json.dumps(line), flush=True)
        return

    kind, dims, batch, desc, with_inv, _ = CONFIGS[cfg]
    stream = torch.cuda.Stream(device=dev)   # our kernels and the events share it
    head = measure_plan(args, cfg, dev, stream, world, rank, batch=args.batch or None, headline=True)
    batch = args.batch or batch
    src, mid, back, per_step_flops, ms_step, with_inv, form, dtype = head.pop("_bufs")
    f64 = args.form == "f64"

    # the split-precision tensor-core form on the same workload, same stream
    tc_form = None
    if args.form == "plain" and not args.no_tc and world == 1:
        tc_form = tc_form_rate(kind, dims, batch, with_inv, src, mid, back, stream, per_step_flops, ms_step)

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        e2e = e2e_rate(args, kind, dims, batch, src, world, form=form, dtype=dtype)
    del src, mid, back
    torch.cuda.synchronize()
    torch.cuda.empty_cache()

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        cpu = cpu_record(*cpu_rate(kind, dims, batch, threads, budget_s=args.cpu_budget, f64=f64))
        if cpu["cores"] > 1:
            # the same CPU path on one thread (a bounded sample), beside all host threads
            r1 = cpu_rate(kind, dims, batch, 1, budget_s=max(1.0, args.cpu_budget / 4), f64=f64)
            cpu["single_thread"] = {"value": round(r1[0], 3), "cores": 1, "sample": r1[1]}
    roofline = head["roofline"]
    if not f64 and not args.batch and args.form == "plain":
        tr, how = committed_traffic(cfg)
        if tr is not None:
            roofline["traffic"] = tr
            roofline["traffic_source"] = how
    line = {
        "metric": METRIC, "value": head["value"], "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": head["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if f64 else "f32",
        "data": DATA,
        "config": config_record(cfg, args, world),
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "accuracy": head["accuracy"],
        "tc_split_form": tc_form,
        "gpu_launches": head["gpu_launches"],
        "clocks": head["clocks"],
    }
    # every other configuration at full size, on one GPU only
    if world == 1 and not args.no_sub and not args.batch and args.form == "plain":
        subs = {}
        for c in SUB_ORDER:
            if c != cfg:
                subs[c] = sub_record(args, c, dev)
        line["configs"] = subs
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=sorted(CONFIGS))
    ap.add_argument("--batch", type=int, default=0, help="override the batch (profiling a smaller case)")
    ap.add_argument("--form", default="plain", choices=["plain", "tc", "f64"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tc", action="store_true", help="skip timing the tensor-core form beside the plain one")
    ap.add_argument("--no-sub", action="store_true", help="headline configuration only (no \"configs\" records)")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuned queue beside the default one")
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--sub-cpu-budget", type=float, default=3.0,
                    help="seconds of CPU baseline per configuration record")
    ap.add_argument("--soak", type=float, default=1.5, help="seconds of untimed load before the timed region")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args, args.config)
    else:
        run_ours(args, args.config)


if __name__ == "__main__":
    main()
