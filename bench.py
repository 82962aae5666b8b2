"""Benchmark of the BCSR SpMM hot path on GB300 (one JSON line on stdout).

Workload (the mixed-precision configuration the headline metric is quoted on):
  A 16384 x 16384 with 64x16 blocks, random block pattern at 2 % block density,
  block values N(0,1) x 10^u (u ~ U[-3, 3] per block); B 16384 x 512 N(0,1);
  C = A B in fp32. Synthetic, seeded.
  One step = one SpMM over one problem. Six copies of the problem (inputs and
  output, ~370 MB > 2.5 x L2) are used round-robin so no step reads another
  step's data from L2.

Arms:
  (default) this library: for every precision (fp16, bf16, e4m3 + per-block
            scales, split fp16 hi+lo) the learned cost model picks the entry of
            the tuner table that runs (kernel configurations and per-matrix
            plans); the exhaustive sweep over the whole table, timed the same
            way (back to back over the rotating copies, graph-replayed, plans
            chained with the inputs-ready flag), is reported beside it as the
            model's regret. The headline `value` is the fastest precision whose
            measured error on this workload (max-relative against an FP64
            product of the fp32 inputs, on sampled block rows) is <= 1e-2.
            Plain fp16 (the library's default configuration, no tuning, no
            plan) is reported beside it.
            The line also carries the batched workload: 64 uneven products in one
            persistent launch replayed from a CUDA graph, against 64 sequential
            launches.
  --impl reference: the reference's host multiply (cpu_matmul_ref,
            nvbench_main.cu:78-91, restated in oracle/) on all host cores, over a
            bounded row sample per step, in the same unit.
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

M = K = 16384
N = 512
BR = 64
DENSITY = 0.02
SEED = 20240
WORKLOAD = ("A 16384x16384, 64x16 blocks, random 2% block density, values N(0,1)*10^U[-3,3] "
            "per block; B 16384x512 N(0,1); C fp32")
METRIC = "BCSR SpMM TFLOP/s (nonzero-block FLOPs), tuned mixed precision vs plain FP16"
# Problem copies used round-robin by the GPU arms: 6 x 60.8 MB = 365 MB, over
# 2.5x the 129 MB L2, so no step reads another step's inputs from L2.
COPIES = 6
DATA = "synthetic (seeded generators)"
# The workload, the same in both arms (how each arm runs it is in its own keys).
CONFIG = {"workload": WORKLOAD,
          "l2": "GPU steps rotate over %d problem copies (365 MB, > 2.5x L2); the CPU arm's sample "
                "is its own" % COPIES}
# Documented normwise error bars vs FP64 (tests/test_gpu_precision.py).
ERROR_BAR = {"f16": 2e-3, "bf16": 1e-2, "f16_split": 2e-6, "e4m3": 8e-2}
TARGET_ERR = 1e-2


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def make_structure():
    import matrixmultiplicationcuda_gb300 as m
    rp, ci = m.gen_structure(M, K, BR, m.PATTERN_RANDOM, DENSITY, 0, seed=SEED)
    return rp, ci


def fp64_rows(rp, ci, vals, Bf, rows):
    """FP64 product of block rows `rows` of A (fp32 block values) and B (fp32)."""
    blocks = vals.reshape(-1, BR, 16).astype(np.float64)
    Bd = Bf.astype(np.float64)
    out = []
    for r in rows:
        acc = np.zeros((BR, N))
        for k in range(rp[r], rp[r + 1]):
            acc += blocks[k] @ Bd[ci[k] * 16:(ci[k] + 1) * 16]
        out.append(acc)
    return np.concatenate(out)


def work_units(rp, ci):
    nnzb = len(ci)
    flops = 2.0 * nnzb * BR * 16 * N
    cols_touched = len(np.unique(ci))
    return nnzb, flops, cols_touched


# bytes per stored element of A and of B, and per-block scale bytes, by precision
STORAGE = {"f16": (2, 2, 0), "bf16": (2, 2, 0), "e4m3": (1, 1, 4), "f16_split": (4, 4, 0)}


def algorithmic_bytes(nnzb, cols_touched, prec="f16"):
    """Compulsory bytes of one SpMM: A values (+ e4m3 block scales) + col_idx +
    row_ptr + the B rows that are referenced + the fp32 C write."""
    a_es, b_es, sc = STORAGE[prec]
    return (nnzb * BR * 16 * a_es + nnzb * sc + 4 * nnzb + 4 * (M // BR + 1) +
            cols_touched * 16 * N * b_es + M * N * 4)


# ------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples (SM clock, throttle reasons) in the background."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.samples = []
        self.proc = None
        self.marks = {}

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.samples.append((time.time(), parts))

    def mark(self, name):
        self.marks[name] = time.time()

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        t0, t1 = self.marks.get("timed_start", 0), self.marks.get("timed_end", 1e30)
        w0 = self.marks.get("load_start", 0)
        timed = [s for t, s in self.samples if t0 <= t <= t1]
        window = "timed"
        if len(timed) < 3:   # a short timed region: add the sustained load just before it
            timed = [s for t, s in self.samples if w0 <= t <= t1]
            window = "warmup+timed"
        if not timed:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [num(s[1]) for s in timed if num(s[1])]
        mx = [num(s[2]) for s in timed if num(s[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in timed for i in range(4) if s[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(timed), "window": window}


# ------------------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_tflops(flops_per_step, ms_per_step_max, world):
    """Replicas: every rank runs the same product, so the job's throughput is
    world x one product's FLOPs over the slowest rank's time per step."""
    return world * flops_per_step / (ms_per_step_max * 1e-3) / 1e12


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_sample_rows(rp, ci, vals_f32, rows, row0):
    """Dense fp16 rows [row0, row0+rows) of A (what the reference host multiply reads)."""
    A = np.zeros((rows, K), np.float16)
    br0, br1 = row0 // BR, (row0 + rows + BR - 1) // BR
    blocks = vals_f32.reshape(-1, BR, 16)
    for br in range(br0, br1):
        for k in range(rp[br], rp[br + 1]):
            r_lo = max(br * BR, row0)
            r_hi = min((br + 1) * BR, row0 + rows)
            A[r_lo - row0:r_hi - row0, ci[k] * 16:(ci[k] + 1) * 16] = blocks[k][r_lo - br * BR:r_hi - br * BR]
    return A


def useful_flops_rows(rp, row0, rows):
    """Nonzero-block FLOPs of output rows [row0, row0+rows)."""
    f = 0.0
    for br in range(row0 // BR, (row0 + rows + BR - 1) // BR):
        lo, hi = max(br * BR, row0), min((br + 1) * BR, row0 + rows)
        f += 2.0 * (rp[br + 1] - rp[br]) * 16 * (hi - lo) * N
    return f


def cpu_reference_rate(rp, ci, vals, Bbits, rows, threads, min_seconds=0.0, row0=0):
    """TFLOP/s (nonzero-block) of the restated reference host multiply on `rows` rows."""
    from oracle import oracle
    A = cpu_sample_rows(rp, ci, vals, rows, row0)
    done, t = 0.0, 0.0
    while True:
        t0 = time.perf_counter()
        oracle.cpu_matmul_ref(A.view(np.uint16), Bbits, threads=threads)
        t += time.perf_counter() - t0
        done += useful_flops_rows(rp, row0, rows)
        if t >= min_seconds:
            break
    return done / t / 1e12, t


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


# ------------------------------------------------------------------------------------
def run_reference(args, world, rank):
    """The reference's host multiply (cpu_matmul_ref, nvbench_main.cu:78-91, in the
    oracle's restatement) on every host thread, over a bounded sample of output
    rows per step. Its inputs come from the oracle's restatement of the synthetic
    generators (bit-identical to the library's, pinned by the CPU tests), so this
    arm loads nothing of the library."""
    if rank != 0:
        return
    from oracle import oracle
    rp, ci = oracle.gen_structure(M, K, BR, oracle.PATTERN_RANDOM, DENSITY, 0, seed=SEED)
    nnzb = len(ci)
    vals = oracle.gen_values(nnzb, BR, 16, oracle.DIST_SCALED_NORMAL, seed=SEED + 1)
    vals = vals.astype(np.float16).astype(np.float32)
    B = oracle.gen_dense(K, N, oracle.DIST_NORMAL, seed=SEED + 2).astype(np.float16)
    threads = host_threads()
    rows = 64 * threads          # bounded sample per step: about 0.4 s on 16 Arm cores
    for i in range(args.warmup):
        r0 = (i * 977) % (M - rows)
        r0 -= r0 % BR
        cpu_reference_rate(rp, ci, vals, B.view(np.uint16), min(rows, 256), threads, row0=r0)
    t_total, f_total = 0.0, 0.0
    for i in range(args.steps):
        r0 = (i * 1931) % (M - rows)
        r0 -= r0 % BR
        A = cpu_sample_rows(rp, ci, vals, rows, r0)
        t0 = time.perf_counter()
        oracle.cpu_matmul_ref(A.view(np.uint16), B.view(np.uint16), threads=threads)
        t_total += time.perf_counter() - t0
        f_total += useful_flops_rows(rp, r0, rows)
    value = f_total / t_total / 1e12
    wmma = None if args.no_wmma else reference_wmma_gpu(rp, ci, vals, B)
    sample = ("%d of %d output rows per step (rows [r0, r0 + %d), r0 moving over the matrix), the "
              "reference host multiply (dense i-k-j over all K, fp32, zeros multiplied too) split by rows "
              "over %d threads; the rate counts the sample's nonzero-block FLOPs" % (rows, M, rows, threads))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": DATA, "config": dict(CONFIG),
            "us_per_output_row": 1e6 * t_total / (args.steps * rows),
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0,
            "reference_wmma_gpu": wmma}
    print(json.dumps(line))


def reference_wmma_gpu(rp, ci, vals, B, reps=20):
    """Context beside the CPU rate: the reference's own WMMA kernel for 64x16 blocks
    (sparseMatrixMulTensor64x16, src/cuda_kernels.cu:618-695, built unmodified for
    sm_103a), launched with the reference harness's grid on the same product: timed
    alone after an L2 flush (the reference harness's cold timing) and back to back
    over six rotating copies (the timing of the library's own step). None when no
    GPU or no reference build is present."""
    try:
        import torch
        from oracle import oracle
        if not torch.cuda.is_available() or not oracle.ref_wmma_available():
            return None
    except ImportError:
        return None
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    st = torch.cuda.current_stream().cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def cold(launch):
        for _ in range(3):
            launch(0)
        ts = []
        for k in range(reps):
            flush.fill_(k & 0xff)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            launch(0)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e3)
        return float(np.mean(ts))

    copies = [[t(rp), t(ci), t(vals.astype(np.float16)), t(B), torch.empty((M, N), dtype=torch.float32, device=dev)]
              for _ in range(COPIES)]
    launch = lambda i: oracle.ref_wmma_launch("sparseMatrixMulTensor64x16", *[x.data_ptr() for x in copies[i % COPIES]],
                                              M, N, st)
    us = cold(launch)
    for i in range(COPIES):
        launch(i)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    loops = 60
    e0.record()
    for i in range(loops):
        launch(i)
    e1.record()
    torch.cuda.synchronize()
    us_b2b = e0.elapsed_time(e1) * 1e3 / loops
    flops = 2.0 * len(ci) * BR * 16 * N
    out = {"kernel": "sparseMatrixMulTensor64x16", "us": us, "tflops": flops / (us * 1e-6) / 1e12,
           "back_to_back_us": us_b2b, "back_to_back_tflops": flops / (us_b2b * 1e-6) / 1e12,
           "grid": "(N/32, M/64) warps of 32 threads, as the reference harness launches it"}
    del copies
    # the 1024^2 16x16 case through the reference generator and BCSR build (restated)
    A1 = oracle.generate_matrix(1024, 1024, 0.9, "blockrandom", 16, 123)
    B1 = oracle.f32_to_f16(oracle.generate_matrix(1024, 1024, 0.0, "random", 16, 456))
    hdr, idx, data = oracle.bcsr(oracle.f32_to_f16(A1), 16, 16)
    d1 = [t(hdr), t(idx), t(data), t(B1), torch.empty((1024, 1024), dtype=torch.float32, device=dev)]
    launch1 = lambda i: oracle.ref_wmma_launch("sparseMatrixMulTensor", *[x.data_ptr() for x in d1], 1024, 1024, st)
    us1 = cold(launch1)
    f1 = 2.0 * len(idx) * 16 * 16 * 1024
    return {"A16384_64x16_N512": out,
            "A1024_16x16_N1024": {"kernel": "sparseMatrixMulTensor", "us": us1, "tflops": f1 / (us1 * 1e-6) / 1e12,
                                  "nnzb": int(len(idx)), "grid": "(N/16, M/16) warps, as the reference harness"}}


def run_ours(args, world, rank, local):
    import torch
    import matrixmultiplicationcuda_gb300 as m
    from matrixmultiplicationcuda_gb300 import DType
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    hbm_peak, tensor_peak, peak_kind = peaks()

    rp, ci = make_structure()
    nnzb, flops, cols_touched = work_units(rp, ci)
    vals = m.gen_values(nnzb, BR, 16, m.DIST_SCALED_NORMAL, seed=SEED + 1)
    Bf = m.gen_dense(K, N, m.DIST_NORMAL, seed=SEED + 2)

    # device copies of the problem (six, round-robin) per precision
    l2 = torch.cuda.get_device_properties(dev).L2_cache_size
    per_copy = algorithmic_bytes(nnzb, cols_touched, "f16")
    copies = COPIES
    assert copies * per_copy > 2.5 * l2, "problem copies no longer exceed 2.5x L2"
    rp_d = torch.from_numpy(rp).to(dev)
    ci_d = torch.from_numpy(ci).to(dev)
    v32 = torch.from_numpy(vals).to(dev)
    B32 = torch.from_numpy(Bf).to(dev)

    precs = {"f16": DType.F16, "bf16": DType.BF16, "e4m3": DType.E4M3, "f16_split": DType.F16_SPLIT}
    if args.precision != "auto":
        precs = {args.precision: precs[args.precision], "f16": DType.F16}

    def prepare(dt):
        out = []
        for c in range(copies):
            qv, qlo, qs = m.quantize(v32, dt, block_elems=BR * 16)
            Bq, Blo, Bs = m.quantize(B32.reshape(-1), dt)
            A = m.BCSR(M, K, BR, 16, rp_d.clone(), ci_d.clone(), qv, dt, qlo, qs)
            C = torch.empty((M, N), dtype=torch.float32, device=dev)
            out.append((A, Bq.view(K, N), Blo.view(K, N) if Blo is not None else None,
                        float(Bs[0]) if Bs is not None else 1.0, C))
        return out

    def launch(prob, cfg, stream=None, inputs_ready=True):
        """One product on a configuration, or on a per-matrix plan (m.BcsrPlan).
        A plan run in the timed loops says inputs_ready: every copy's A and B were
        written and synchronised before the loops, and no kernel in them writes an
        input, so a launch may start copying its first items while the one before
        it finishes. The end-to-end leg, which copies fresh inputs every step,
        passes inputs_ready=False."""
        A, Bq, Blo, bs, C = prob
        if isinstance(cfg, m.BcsrPlan):
            cfg.run(A, Bq, C=C, B_lo=Blo, b_scale=bs, stream=stream, inputs_ready=inputs_ready)
        else:
            m.spmm(A, Bq, N=N, C=C, cfg=cfg, B_lo=Blo, b_scale=bs, stream=stream)

    def cfg_name(c):
        if isinstance(c, m.BcsrPlan):
            items, groups, pc = c.info()
            return "plan %s (%d rows split)" % (tuner.config_name(pc), groups)
        return tuner.config_name(c)

    stream = torch.cuda.current_stream()
    graph_note = {"ok": True, "why": ""}

    def capture(probs, cfg, steps):
        """`steps` launches captured in one CUDA graph, or None if capture fails.
        Replaying it issues the launches with no host work between them, so a
        loop of launches a few microseconds long is not bound by the Python
        call that issues each one."""
        if not graph_note["ok"]:
            return None
        try:
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                for i in range(3):   # warm-up on a side stream, as capture wants
                    launch(probs[i % len(probs)], cfg, stream=side)
            torch.cuda.current_stream().wait_stream(side)
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="relaxed"):
                cs = torch.cuda.current_stream()
                for i in range(steps):
                    launch(probs[i % len(probs)], cfg, stream=cs)
            g.replay()   # first replay uploads the graph
            torch.cuda.synchronize()
            return g
        except Exception as e:   # time eager launches from here on
            graph_note.update(ok=False, why=str(e).splitlines()[0][:200])
            sys.stderr.write("graph capture failed (%s); timing eager launches\n" % graph_note["why"])
            torch.cuda.synchronize()
            return None

    def hold_gpu():
        """A ~0.1 ms spin kernel ahead of a start event: the GPU stays busy while
        the host records the event and submits the timed launches, so the
        device-timed region holds the launches and not the host's submission
        gap (about 5 us, 0.2 us per step of a 20-step loop)."""
        torch.cuda._sleep(200_000)

    def time_loop(probs, cfg, steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g = capture(probs, cfg, steps)
        hold_gpu()
        e0.record(stream)
        if g is not None:
            g.replay()
        else:
            for i in range(steps):
                launch(probs[i % len(probs)], cfg)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / steps

    # Per precision: the learned cost model's pick, timed; the exhaustive sweep
    # beside it (its best, and the model's regret against it).
    from matrixmultiplicationcuda_gb300 import costmodel, tuner
    model = costmodel.CostModel.load(os.path.join(ROOT, "matrixmultiplicationcuda_gb300", "data", "costmodel.npz"))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    table = tuner.configs()
    results = {}
    prepared = {}
    sampler = ClockSampler(local)
    sampler.start()
    sampler.mark("load_start")
    def realize(c, A0):
        """A table entry as something launch() runs: a plan entry becomes its
        per-matrix plan (built once, outside every timed region)."""
        return m.BcsrPlan(A0, N, c) if tuner.is_plan(c) else c

    for name, dt in precs.items():
        probs = prepare(dt)
        prepared[name] = probs
        A0, Bq0, Blo0, bs0, C0 = probs[0]
        # The learned cost model picks the configuration that runs; the
        # exhaustive sweep over the whole table, in the same regime (launches
        # back to back over the rotating copies, replayed from a CUDA graph,
        # plans chained with the inputs-ready flag), is its judge and fallback.
        ms_sweep = tuner.sweep_b2b([(A, Bq, C, Blo, bs) for (A, Bq, Blo, bs, C) in probs], launches=30, warmup=2)
        m.device_error_check()
        pick_model = model.select(A0, N)
        pick_sweep = table[int(np.argmin(ms_sweep))]
        cfg_model = realize(pick_model, A0)
        cfg_sweep = cfg_model if tuner.config_key(pick_sweep) == tuner.config_key(pick_model) else realize(pick_sweep, A0)
        time_loop(probs, cfg_model, 3)
        t_model = time_loop(probs, cfg_model, 30)
        if cfg_sweep is cfg_model:
            t_sweep = t_model
        else:
            time_loop(probs, cfg_sweep, 3)
            t_sweep = time_loop(probs, cfg_sweep, 30)
        m.device_error_check()
        cands = {cfg_name(cfg_model): cfg_model, cfg_name(cfg_sweep): cfg_sweep}
        sys.stderr.write("%s: model pick %s %.2f us, sweep best %s %.2f us (in the sweep %.2f us)\n" % (
            name, tuner.config_name(pick_model), t_model * 1e3, tuner.config_name(pick_sweep), t_sweep * 1e3,
            float(np.min(ms_sweep)) * 1e3))
        results[name] = {"ms": t_model, "cfg": cfg_model, "model_cfg": pick_model, "model_ms": t_model,
                         "cands": cands, "tflops": flops / t_model / 1e9, "sweep_ms": t_sweep, "sweep_cfg": pick_sweep,
                         "sweep_table_ms": {tuner.config_name(c): float(t) for c, t in zip(table, ms_sweep)
                                            if np.isfinite(t)},
                         "err_bar": ERROR_BAR[name], "bytes": algorithmic_bytes(nnzb, cols_touched, name)}
    model.close()
    # error of every precision against an FP64 product of the exact fp32 inputs,
    # on sampled block rows
    sample_rows = [0, (M // BR) // 3, 2 * (M // BR) // 3, M // BR - 1]
    ref = fp64_rows(rp, ci, vals, Bf, sample_rows)
    for name in results:
        A0, Bq0, Blo0, bs0, C0 = prepared[name][0]
        launch(prepared[name][0], results[name]["cfg"])
        torch.cuda.synchronize()
        got = np.concatenate([C0[r * BR:(r + 1) * BR].cpu().numpy() for r in sample_rows])
        d = got.astype(np.float64) - ref
        results[name]["max_rel"] = float(np.abs(d).max() / np.abs(ref).max())
        results[name]["fro_rel"] = float(np.linalg.norm(d) / np.linalg.norm(ref))
    # plain fp16: the library's default configuration, no tuning
    time_loop(prepared["f16"], None, 3)
    plain_ms = time_loop(prepared["f16"], None, 30)
    # the headline precision: the fastest whose measured error on this workload
    # is within the target (max-relative against FP64)
    ok = {k: v for k, v in results.items() if v["max_rel"] <= TARGET_ERR} or {"f16": results["f16"]}
    tuned = min(ok, key=lambda k: results[k]["ms"])
    probs, cfg = prepared[tuned], results[tuned]["cfg"]
    if args.pick_from:
        # run what an earlier run's line names (its precision and configuration,
        # among this run's candidates): a profiler's timings must not change the pick
        prev = json.loads(open(args.pick_from).read().strip().splitlines()[-1])
        tuned = prev["dtype"]
        cfg = results[tuned]["cands"][prev["run"]["kernel_config"]]
        probs = prepared[tuned]

    # warm-up, then exactly K timed steps on the tuned configuration: the K
    # launches are captured in one CUDA graph beforehand and replayed once
    t_warm = time.time()
    w = 0
    while w < args.warmup or time.time() - t_warm < 1.0:
        launch(probs[w % len(probs)], cfg)
        w += 1
    torch.cuda.synchronize()
    timed_graph = capture(probs, cfg, args.steps)
    barrier(world)
    torch.cuda.synchronize()
    sampler.mark("timed_start")
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # NVTX range "bench_timed": a profiler can capture exactly the timed launches
    # (ncu --nvtx --nvtx-include "bench_timed/")
    torch.cuda.nvtx.range_push("bench_timed")
    hold_gpu()
    g0.record(stream)
    if timed_graph is not None:
        timed_graph.replay()
    else:
        for i in range(args.steps):
            launch(probs[i % len(probs)], cfg)
    g1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    sampler.mark("timed_end")
    barrier(world)
    m.device_error_check()
    total_ms = g0.elapsed_time(g1)
    kern_ms = total_ms / args.steps          # average launch duration, launch gaps included
    total_ms = max_over_ranks(total_ms, world)
    ms_step = total_ms / args.steps
    value = whole_job_tflops(flops, ms_step, world)

    # End to end through the public API with host buffers (pinned), tuned precision:
    # every step copies its inputs host -> device, multiplies, and reads C back.
    # Three device buffer sets rotate through three streams -- uploads, products,
    # downloads -- ordered by events, so the host link carries one step's inputs
    # in while an earlier step's C comes out (the copy engines run both
    # directions at once) and no stream's next upload waits behind its own
    # download.
    A0, Bq0, Blo0, bs0, C0 = probs[0]
    hA = [t.cpu().pin_memory() for t in (A0.row_ptr, A0.col_idx, A0.vals)]
    hx = [t.cpu().pin_memory() for t in (A0.vals_lo, A0.scales) if t is not None]
    hB = [t.cpu().pin_memory() for t in (Bq0, Blo0) if t is not None]
    nsets = 3
    hC = [torch.empty((M, N), dtype=torch.float32).pin_memory() for _ in range(nsets)]
    h2d = sum(t.numel() * t.element_size() for t in hA + hx + hB)
    d2h = hC[0].numel() * 4
    up, comp, down = (torch.cuda.Stream(device=dev) for _ in range(3))
    sets = []
    for k in range(nsets):
        dA = [torch.empty_like(t, device=dev) for t in hA]
        dx = [torch.empty_like(t, device=dev) for t in hx]
        dB = [torch.empty_like(t, device=dev) for t in hB]
        Ae = m.BCSR(M, K, BR, 16, dA[0], dA[1], dA[2], A0.dtype,
                    dx[0] if A0.vals_lo is not None else None,
                    dx[-1] if A0.scales is not None else None)
        sets.append((dA + dx + dB, Ae, dB, torch.empty((M, N), dtype=torch.float32, device=dev)))
    ev_in = [torch.cuda.Event() for _ in range(nsets)]     # set k's inputs are on the device
    ev_done = [torch.cuda.Event() for _ in range(nsets)]   # set k's product is in its C
    ev_free = [torch.cuda.Event() for _ in range(nsets)]   # set k's C has reached the host
    used = [False] * nsets

    def e2e_step(i):
        k = i % nsets
        dev_bufs, Ae, dB, Cd = sets[k]
        if used[k]:
            up.wait_event(ev_free[k])       # the set's last C has left before it is refilled
        with torch.cuda.stream(up):
            for d, h in zip(dev_bufs, hA + hx + hB):
                d.copy_(h, non_blocking=True)
            ev_in[k].record(up)
        comp.wait_event(ev_in[k])
        launch((Ae, dB[0], dB[1] if len(dB) > 1 else None, bs0, Cd), cfg, stream=comp, inputs_ready=False)
        ev_done[k].record(comp)
        down.wait_event(ev_done[k])
        with torch.cuda.stream(down):
            hC[k].copy_(Cd, non_blocking=True)
            ev_free[k].record(down)
        used[k] = True

    e2e_steps = max(4, min(args.steps, 50))
    for i in range(4):
        e2e_step(i)
    torch.cuda.synchronize()
    barrier(world)
    q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    q0.record(stream)
    for st in (up, comp, down):
        st.wait_event(q0)
    for i in range(e2e_steps):
        e2e_step(i)
    for st in (up, comp, down):
        ev = torch.cuda.Event()
        ev.record(st)
        stream.wait_event(ev)
    q1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(q0.elapsed_time(q1) / e2e_steps, world)
    m.device_error_check()

    # What bounds the step, measured the same way (30 launches replayed from a
    # graph, back to back): writing C alone (torch's fill kernel over the
    # rotating copies' C, 33.5 MB per launch), a one-element kernel (the launch
    # floor of such a loop), and the tuned configuration with every launch on
    # the same copy, so that A, B and C stay in L2 and no launch touches DRAM.
    def time_graph(fn, steps=30):
        side = torch.cuda.Stream()
        side.wait_stream(stream)
        with torch.cuda.stream(side):
            for i in range(3):
                fn(i)
        stream.wait_stream(side)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for i in range(steps):
                fn(i)
        g.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        hold_gpu()
        e0.record(stream)
        g.replay()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / steps

    one = torch.zeros(1, device=dev)
    write_c_ms = time_graph(lambda i: probs[i % len(probs)][4].fill_(0.0))
    floor_ms = time_graph(lambda i: one.fill_(float(i)))
    time_loop([probs[0]], cfg, 3)
    l2_warm_ms = time_loop([probs[0]], cfg, 30)
    bounds = {"c_write_us": write_c_ms * 1e3, "c_write_tbs": M * N * 4 / (write_c_ms * 1e-3) / 1e12,
              "launch_floor_us": floor_ms * 1e3, "l2_resident_step_us": l2_warm_ms * 1e3,
              "note": ("per launch, 30 graph-replayed launches back to back: writing the 33.5 MB of C alone "
                       "(torch fill over the rotating copies' C); a one-element kernel; the tuned "
                       "configuration on one copy only (A, B, C resident in L2, no DRAM traffic)")}
    m.device_error_check()
    sampler.stop()
    clocks = sampler.summary()

    batched = None if args.no_batch else bench_batched(m, torch, dev, flush, hbm_peak)

    # CPU baseline (reference host multiply, restated), rank 0 only, bounded sample
    cpu = cpu_sparse = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        vh = vals.astype(np.float16).astype(np.float32)
        Bh = Bf.astype(np.float16).view(np.uint16)
        rate, secs = cpu_reference_rate(rp, ci, vh, Bh, 192, 1, min_seconds=10.0, row0=4096)
        cpu = {"value": rate, "unit": "TFLOP/s", "cores": 1, "kind": "port",
               "sample": "192 of %d output rows, reference host multiply (dense i-k-j, fp32, "
                         "one thread), repeated for %.1f s" % (M, secs)}
        # beside it, a block-sparse fp32 host multiply on every host core: a
        # baseline only, not the reference's algorithm
        from oracle import oracle
        threads = os.cpu_count() or 1
        vbits = vals.astype(np.float16).view(np.uint16)
        Bq = Bf.astype(np.float16).astype(np.float32).reshape(K, N)
        t0, runs = time.perf_counter(), 0
        while True:
            oracle.bcsr_matmul_f32_mt(rp, ci, vbits, BR, Bq, threads=threads)
            runs += 1
            if time.perf_counter() - t0 >= 3.0:
                break
        secs_s = time.perf_counter() - t0
        cpu_sparse = {"value": runs * flops / secs_s / 1e12, "unit": "TFLOP/s", "cores": threads,
                      "kind": "block-sparse host multiply (baseline only)",
                      "sample": "the whole product, %d runs in %.1f s, fp32, split by block rows" % (runs, secs_s)}

    tr = results[tuned]
    bytes_launch = tr["bytes"]
    achieved = bytes_launch / (kern_ms * 1e-3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(tp):
        traffic = json.load(open(tp)).get(tuned)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": tuned, "data": DATA, "config": dict(CONFIG),
            "us_per_output_row": 1e3 * ms_step / M,
            "run": {"precision": tuned,
                    "kernel_config": cfg_name(cfg),
                    "picked_by": ("the learned cost model's pick (spmm_cost_model_select); the exhaustive "
                                  "back-to-back sweep over the tuner table is its judge (model_regret)")
                    if not args.pick_from else "pinned to the line in %s" % os.path.basename(args.pick_from),
                    "parallelism": "replicas" if world > 1 else "single GPU",
                    "copies_mb": copies * per_copy / 1e6,
                    "nnzb": nnzb,
                    "timed_loop": ("the K launches captured in one CUDA graph before the timed region and "
                                   "replayed once (the candidates' loops likewise)") if graph_note["ok"]
                    else "eager launches (graph capture failed: %s)" % graph_note["why"],
                    "inputs_ready": ("plan runs with SPMM_RUN_INPUTS_READY: no kernel in the timed loop writes "
                                     "A or B, so a launch copies and multiplies its first items while the "
                                     "previous step finishes, and waits for it before claiming queued work "
                                     "or writing C") if isinstance(cfg, m.BcsrPlan) else None},
            "plain_fp16": {"tflops": flops / plain_ms / 1e9, "ms": plain_ms,
                           "kernel_config": "library default (no tuning)"},
            "tuned_vs_plain_fp16": plain_ms / tr["ms"],
            "precisions": {k: {"tflops": v["tflops"], "ms": v["ms"], "err_bar": v["err_bar"],
                               "model_pick": tuner.config_name(v["model_cfg"]), "run_as": cfg_name(v["cfg"]),
                               "model_pick_ms": v["model_ms"],
                               "sweep_best": tuner.config_name(v["sweep_cfg"]), "sweep_best_ms": v["sweep_ms"],
                               "model_regret": v["model_ms"] / v["sweep_ms"] - 1.0,
                               "sweep_b2b_ms": v["sweep_table_ms"],
                               "max_rel_err": v["max_rel"], "fro_rel_err": v["fro_rel"]}
                           for k, v in results.items()},
            "error_sample": "block rows %s, against an FP64 product of the fp32 inputs" % sample_rows,
            "batched": batched,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": traffic,
                         "algorithmic_bytes": bytes_launch, "peak_source": peak_kind,
                         "tensor_frac": (flops / (kern_ms * 1e-3) / 1e12) / tensor_peak},
            "bounds": bounds,
            "cpu_baseline": cpu,
            "cpu_baseline_block_sparse": cpu_sparse,
            "e2e": {"value": world * flops / (e2e_ms * 1e-3) / 1e12, "unit": "TFLOP/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
            "gpu_launches": args.steps,
            "clocks": clocks,
        }
        print(json.dumps(line))


def bench_batched(m, torch, dev, flush, hbm_peak, reps=20):
    """64 uneven fp16 products (workloads.uneven_batch_specs): one persistent
    launch replayed from a CUDA graph against 64 sequential single-product
    launches (eager and graph-captured), L2 flushed before every timed run."""
    specs = m.uneven_batch_specs(64, seed=2024)
    probs, flops, nbytes = [], 0.0, 0.0
    for sp in specs:
        rp, ci, vals, Bf = m.make_problem(sp)
        A = m.BCSR.from_host(sp["M"], sp["K"], sp["bR"], rp, ci, vals, m.DType.F16, device=dev)
        B = torch.from_numpy(Bf).to(dev).half()
        C = torch.empty((sp["M"], sp["N"]), dtype=torch.float32, device=dev)
        probs.append((A, B, C))
        flops += 2.0 * len(ci) * sp["bR"] * 16 * sp["N"]
        nbytes += (len(ci) * (sp["bR"] * 32 + 4) + 4 * (sp["M"] // sp["bR"] + 1) +
                   len(np.unique(ci)) * 16 * sp["N"] * 2 + sp["M"] * sp["N"] * 4)
    plan = m.BatchPlan(probs)
    side = torch.cuda.Stream(device=dev)
    side.wait_stream(torch.cuda.current_stream())
    plan.run()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        plan.run()

    def seq():
        for A, B, C in probs:
            m.spmm(A, B, C=C)

    g2 = torch.cuda.CUDAGraph()
    seq()
    torch.cuda.synchronize()
    with torch.cuda.graph(g2, stream=side):
        seq()

    def timed(fn):
        ts = []
        for k in range(reps + 3):
            flush.fill_(k & 0xff)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            if k >= 3:
                ts.append(e0.elapsed_time(e1) * 1e3)
        return float(np.mean(ts))   # event timestamps advance in ~2 us steps: the mean averages them out

    t_batch = timed(g.replay)
    t_seq = timed(seq)
    t_seq_graph = timed(g2.replay)
    m.device_error_check()
    plan.close()
    return {"workload": "64 products, M=K in [512, 8192], bR in {16,32,64}, random/band/blockdiag, "
                        "density log-uniform [0.5%, 25%], N in {128,256,512}, fp16",
            "gflop": flops / 1e9, "algorithmic_mb": nbytes / 1e6,
            "batched_graph_us": t_batch, "sequential_eager_us": t_seq, "sequential_graph_us": t_seq_graph,
            "speedup_vs_sequential": t_seq / t_batch, "speedup_vs_sequential_graph": t_seq_graph / t_batch,
            "batched_tflops": flops / (t_batch * 1e-6) / 1e12,
            "roofline_frac": (nbytes / (t_batch * 1e-6) / 1e9) / hbm_peak}


def run_profile(args):
    """One problem copy, `--launches` launches of one precision / configuration and
    nothing else: the command the ncu captures in profiles/ run."""
    import torch
    import matrixmultiplicationcuda_gb300 as m
    from matrixmultiplicationcuda_gb300 import DType
    dev = torch.device("cuda", 0)
    rp, ci = make_structure()
    nnzb = len(ci)
    vals = m.gen_values(nnzb, BR, 16, m.DIST_SCALED_NORMAL, seed=SEED + 1)
    Bf = m.gen_dense(K, N, m.DIST_NORMAL, seed=SEED + 2)
    dt = {"f16": DType.F16, "bf16": DType.BF16, "e4m3": DType.E4M3, "f16_split": DType.F16_SPLIT}[args.profile]
    qv, qlo, qs = m.quantize(torch.from_numpy(vals).to(dev), dt, block_elems=BR * 16)
    Bq, Blo, Bs = m.quantize(torch.from_numpy(Bf).to(dev).reshape(-1), dt)
    A = m.BCSR(M, K, BR, 16, torch.from_numpy(rp).to(dev), torch.from_numpy(ci).to(dev), qv, dt, qlo, qs)
    C = torch.empty((M, N), dtype=torch.float32, device=dev)
    cfg = m.Config(kernel=args.kernel, n_tile=args.n_tile, stages=args.stages, acc_buffers=args.acc)
    for _ in range(args.launches):
        m.spmm(A, Bq.view(K, N), N=N, C=C, cfg=cfg, B_lo=Blo.view(K, N) if Blo is not None else None,
               b_scale=float(Bs[0]) if Bs is not None else 1.0)
    torch.cuda.synchronize()
    m.device_error_check()
    print("profile: %s nnzb=%d launches=%d" % (args.profile, nnzb, args.launches))


def run_profile_families(names, launches):
    """One representative launch sequence per kernel family, for ncu captures
    (python bench.py --profile-family NAME[,NAME...] --launches L).

    Families (seeded synthetic inputs; a few hundred MB on the device at most):
      tc        k_bcsr_tc: A 16384^2, 64x16 blocks, random 2 %, N 512, fp16, a
                512-column tile with one accumulator, static item stride
      plan_c3   k_bcsr_tc on a per-matrix plan: the same product in bf16 with the
                default tcgen05 configuration (256-column tile, five-group ring,
                two accumulators), items heaviest first from the plan's queue
      plan_c3_512  the same product in fp16 on a plan with a 512-column tile and
                one accumulator (one item per CTA), each launch started with
                SPMM_RUN_INPUTS_READY after the first
      tc_split  k_bcsr_tc in split fp16 (three MMAs per block), same product
      mma_e4m3  k_bcsr_mma: the same product in e4m3 with per-block scales
      mma16     k_bcsr_mma: A 8192^2, 16x16 blocks, random 5 %, N 1024, fp16
      batch     k_bcsr_tc_batch: the 64-product uneven workload, one launch
      convert   k_dense_to_bcsr (count and fill) + k_scan_counts: dense fp16
                8192 x 8192 (134 MB) with 16x16 blocks at 5 %
      quantize  k_to_f16 / k_to_bf16 / k_absmax / k_to_e4m3: 64 M fp32 values
      mlp       the cost model's forward / backward / AdamW kernels, batch 2000
      hybrid    k_bcsr_tc with the CSR pass in its epilogue (spmm_hcsr_mm): A 4096^2
                (10 % dense 16x16 blocks + 2 % scattered entries), threshold 0.5,
                N 1024
      hybrid_plan  the same product planned: CSR entries as gather blocks
      csr       k_csr_mm on the same matrix's entries, all as CSR
      tc64      k_bcsr_tc64 (64-row blocks, M=64 UMMAs, one CTA per SM): the tc
                product in fp16 and in split fp16, 256-column tile
      plan      k_bcsr_tc on a per-matrix plan: A 8192^2, 64x16 blocks, log-normal
                rows (5 %, CV 1.5), N 512, bf16, 256-column tile (rows far above
                the average load split into parts)
      plan_stack  k_bcsr_tc on a stacked per-matrix plan: A 8192^2, 16x16 blocks,
                band (20 %, the union of each 64 rows' columns ~29 % of the
                blocks), N 4096, fp16; four 16-row blocks assembled per 64-row
                block in the stage
      dense     k_dense_tc: the native dense comparator, A 8192 x 8192, B 8192 x 1024, fp16
      plan_rot  the headline run: fp16 plan, 512-column tile, one accumulator,
                launches chained inputs-ready over six rotating copies (five
                launches before the family's warm-up, so a captured launch sees
                the steady state of the timed loop)
      e4m3_plan_rot  the same with e4m3 operands on the plan the learned model
                picks for them (256-column tile, four-group ring)
      gen       the GPU generators: k_gen_structure + k_gen_values for the tc
                product's structure (A 16384^2, 64x16, 2 %), k_gen_dense for B
                (16384 x 512), k_gen_matrix (reference blockrandom, 8192^2 fp16)
    Each family runs `--launches` times after one warm-up, then synchronises and
    checks the device error word.
    """
    only = set(names.split(","))
    L = launches
    import torch
    import matrixmultiplicationcuda_gb300 as m
    from matrixmultiplicationcuda_gb300 import costmodel
    dev = torch.device("cuda", 0)

    def c3(dtype):
        M = K = 16384
        N = 512
        rp, ci = m.gen_structure(M, K, 64, m.PATTERN_RANDOM, 0.02, 0, seed=20240)
        vals = m.gen_values(len(ci), 64, 16, m.DIST_SCALED_NORMAL, seed=20241)
        Bf = m.gen_dense(K, N, m.DIST_NORMAL, seed=20242)
        A = m.BCSR.from_host(M, K, 64, rp, ci, vals, dtype, device=dev)
        Bq, Blo, Bs = m.quantize(torch.from_numpy(Bf).to(dev).reshape(-1), dtype)
        C = torch.empty((M, N), dtype=torch.float32, device=dev)
        return A, Bq.view(K, N), (Blo.view(K, N) if Blo is not None else None), \
            (float(Bs[0]) if Bs is not None else 1.0), C

    def run(fn):
        fn()
        torch.cuda.synchronize()
        for _ in range(L):
            fn()
        torch.cuda.synchronize()
        m.device_error_check()

    if "tc" in only:
        A, B, Blo, bs, C = c3(m.DType.F16)
        cfg = m.Config(kernel=2, n_tile=512, acc_buffers=1)
        run(lambda: m.spmm(A, B, N=512, C=C, cfg=cfg))
        print("tc: nnzb=%d" % A.nnzb)
    if "tc_split" in only:
        A, B, Blo, bs, C = c3(m.DType.F16_SPLIT)
        cfg = m.Config(kernel=2, n_tile=256, acc_buffers=2, stages=2)
        run(lambda: m.spmm(A, B, N=512, C=C, cfg=cfg, B_lo=Blo))
        print("tc_split: nnzb=%d" % A.nnzb)
    if "mma_e4m3" in only:
        A, B, Blo, bs, C = c3(m.DType.E4M3)
        cfg = m.Config(kernel=1, n_tile=128, stages=4)
        run(lambda: m.spmm(A, B, N=512, C=C, cfg=cfg, b_scale=bs))
        print("mma_e4m3: nnzb=%d" % A.nnzb)
    if "mma16" in only:
        M = K = 8192
        N = 1024
        rp, ci = m.gen_structure(M, K, 16, m.PATTERN_RANDOM, 0.05, 0, seed=7)
        vals = m.gen_values(len(ci), 16, 16, m.DIST_UNIFORM, seed=8)
        A = m.BCSR.from_host(M, K, 16, rp, ci, vals, m.DType.F16, device=dev)
        B = torch.from_numpy(m.gen_dense(K, N, m.DIST_UNIFORM, seed=9)).to(dev).half()
        C = torch.empty((M, N), dtype=torch.float32, device=dev)
        cfg = m.Config(kernel=1, n_tile=256, stages=4)
        run(lambda: m.spmm(A, B, N=N, C=C, cfg=cfg))
        print("mma16: nnzb=%d" % A.nnzb)
    if "batch" in only:
        probs = []
        for sp in m.uneven_batch_specs(64, seed=2024):
            rp, ci, vals, Bf = m.make_problem(sp)
            A = m.BCSR.from_host(sp["M"], sp["K"], sp["bR"], rp, ci, vals, m.DType.F16, device=dev)
            probs.append((A, torch.from_numpy(Bf).to(dev).half(),
                          torch.empty((sp["M"], sp["N"]), dtype=torch.float32, device=dev)))
        plan = m.BatchPlan(probs)
        run(plan.run)
        plan.close()
        print("batch: %d problems" % len(probs))
    if "convert" in only:
        M = K = 8192
        rp, ci = m.gen_structure(M, K, 16, m.PATTERN_RANDOM, 0.05, 0, seed=11)
        vals = m.gen_values(len(ci), 16, 16, m.DIST_UNIFORM, seed=12)
        dense = torch.zeros((M, K), dtype=torch.float16, device=dev)
        blocks = torch.from_numpy(vals.reshape(-1, 16, 16)).to(dev).half()
        rows = np.repeat(np.arange(M // 16), np.diff(rp))
        view = dense.view(M // 16, 16, K // 16, 16).permute(0, 2, 1, 3)
        view[torch.from_numpy(rows).to(dev), torch.from_numpy(ci.astype(np.int64)).to(dev)] = blocks
        run(lambda: m.dense_to_bcsr(dense, 16, 16))
        print("convert: %d x %d, nnzb=%d" % (M, K, len(ci)))
    if "quantize" in only:
        src = torch.randn(64 << 20, device=dev) * 10
        for dt in (m.DType.F16, m.DType.BF16, m.DType.E4M3):
            run(lambda: m.quantize(src, dt, block_elems=1024))
        print("quantize: %d values" % src.numel())
    if only & {"hybrid", "hybrid_plan", "csr"}:
        M = K = 4096
        N = 1024
        blocks = m.generate_matrix(M, K, 0.9, "blockrandom", 16, seed=7)
        scatter = m.generate_matrix(M, K, 0.98, "random", 16, seed=8)
        A = np.where(blocks != 0, blocks, scatter).astype(np.float16).view(np.uint16)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        B = t(m.gen_dense(K, N, m.DIST_UNIFORM, seed=9)).half()
        C = torch.empty((M, N), dtype=torch.float32, device=dev)
        (bh, bi, bd), (ch, cx, cd) = m.host_dense_to_hcsr(A, 0.5)
        Ab = m.BCSR(M, K, 16, 16, t(bh), t(bi), t(bd.view(np.float16)))
        if "hybrid" in only:
            run(lambda: m.hcsr_mm(Ab, t(ch), t(cx), t(cd.view(np.float16)), B, N=N, C=C))
            print("hybrid: %d blocks, %d CSR entries" % (len(bi), len(cx)))
        if "hybrid_plan" in only:
            plan = m.HcsrPlan(Ab, t(ch), t(cx), t(cd.view(np.float16)))
            run(lambda: plan.run(B, N=N, C=C))
            print("hybrid_plan: (blocks, gather blocks) =", plan.info())
            plan.close()
        if "csr" in only:
            _, (rh, rx, rd) = m.host_dense_to_hcsr(A, 1.1)
            rh, rx, rd = t(rh), t(rx), t(rd.view(np.float16))
            run(lambda: m.csr_mm(rh, rx, rd, K, B, N=N, C=C))
            print("csr: %d entries" % rx.numel())
    if "plan_c3" in only:
        A, B, Blo, bs, C = c3(m.DType.BF16)
        plan = m.BcsrPlan(A, 512)
        run(lambda: plan.run(A, B, C=C))
        print("plan_c3: nnzb=%d, (items, split rows) = %s" % (A.nnzb, plan.info()[:2]))
        plan.close()
    if "plan_c3_512" in only:
        A, B, Blo, bs, C = c3(m.DType.F16)
        plan = m.BcsrPlan(A, 512, m.Config(kernel=2, n_tile=512, acc_buffers=1))
        torch.cuda.synchronize()   # no kernel after this writes A or B
        run(lambda: plan.run(A, B, C=C, inputs_ready=True))
        print("plan_c3_512: nnzb=%d, (items, split rows) = %s" % (A.nnzb, plan.info()[:2]))
        plan.close()
    for fam, dt, cfg in (("plan_rot", m.DType.F16, m.Config(kernel=2, n_tile=512, acc_buffers=1)),
                         ("e4m3_plan_rot", m.DType.E4M3, m.Config(kernel=2, n_tile=256, stages=4, acc_buffers=1))):
        if fam not in only:
            continue
        # the benchmark's steady state: six rotating copies (365 MB) of the
        # product, launches chained with the inputs-ready flag, so a captured
        # launch finds the previous one's C dirty in L2 as in the timed loop
        cps = [c3(dt) for _ in range(6)]
        plan = m.BcsrPlan(cps[0][0], 512, cfg)
        torch.cuda.synchronize()   # no kernel after this writes A or B
        k = [0]

        def step(plan=plan, cps=cps, k=k):
            A, B, Blo, bs, C = cps[k[0] % len(cps)]
            k[0] += 1
            plan.run(A, B, C=C, b_scale=bs, inputs_ready=True)

        for _ in range(5):
            step()
        run(step)
        print("%s: nnzb=%d, (items, split rows) = %s" % (fam, cps[0][0].nnzb, plan.info()[:2]))
        plan.close()
    if "tc64" in only:
        A, B, Blo, bs, C = c3(m.DType.F16)
        run(lambda: m.spmm(A, B, N=512, C=C, cfg=m.Config(kernel=3, n_tile=256)))
        A, B, Blo, bs, C = c3(m.DType.F16_SPLIT)
        run(lambda: m.spmm(A, B, N=512, C=C, cfg=m.Config(kernel=3, n_tile=256), B_lo=Blo))
        print("tc64: nnzb=%d" % A.nnzb)
    if "plan" in only:
        M = K = 8192
        rp, ci = m.gen_structure(M, K, 64, m.PATTERN_LOGNORMAL, 0.05, 1.5, seed=77)
        vals = m.gen_values(len(ci), 64, 16, m.DIST_UNIFORM, seed=1)
        A = m.BCSR.from_host(M, K, 64, rp, ci, vals, m.DType.BF16, device=dev)
        B = torch.from_numpy(m.gen_dense(K, 512, m.DIST_UNIFORM, seed=2)).to(dev).bfloat16()
        C = torch.empty((M, 512), dtype=torch.float32, device=dev)
        plan = m.BcsrPlan(A, 512, m.Config(kernel=2, n_tile=256, acc_buffers=2))
        run(lambda: plan.run(A, B, C=C))
        print("plan: (items, split rows) =", plan.info()[:2])
        plan.close()
    if "plan_stack" in only:
        M = K = 8192
        N = 4096
        rp, ci = m.gen_structure(M, K, 16, m.PATTERN_BAND, 0.2, 8, seed=3)
        vals = m.gen_values(len(ci), 16, 16, m.DIST_UNIFORM, seed=4)
        A = m.BCSR.from_host(M, K, 16, rp, ci, vals, m.DType.F16, device=dev)
        B = torch.from_numpy(m.gen_dense(K, N, m.DIST_UNIFORM, seed=5)).to(dev).half()
        C = torch.empty((M, N), dtype=torch.float32, device=dev)
        plan = m.BcsrPlan(A, N)
        run(lambda: plan.run(A, B, C=C))
        print("plan_stack: nnzb=%d, (rows per stack, stacked blocks) =" % len(ci), plan.stacking())
        plan.close()
    if "dense" in only:
        g = torch.Generator().manual_seed(0)
        Ad = (torch.rand((8192, 8192), generator=g) * 2 - 1).half().to(dev)
        Bd = (torch.rand((8192, 1024), generator=g) * 2 - 1).half().to(dev)
        Cd = torch.empty((8192, 1024), dtype=torch.float32, device=dev)
        run(lambda: m.dense_mm(Ad, Bd, C=Cd))
        print("dense: 8192 x 8192 x 1024")
    if "gen" in only:
        def gen():
            rp, ci = m.gpu_gen_structure(16384, 16384, 64, m.PATTERN_RANDOM, 0.02, 0, seed=20240, device=dev)
            m.gpu_gen_values(ci.numel(), 64, 16, m.DIST_SCALED_NORMAL, seed=20241, device=dev)
            m.gpu_gen_dense(16384, 512, m.DIST_NORMAL, seed=20242, device=dev)
            m.gpu_generate_matrix(8192, 8192, 0.9, "blockrandom", 16, seed=7, device=dev)
        run(gen)
        print("gen: done")
    if "mlp" in only:
        s = costmodel.shape()
        rng = np.random.default_rng(0)
        p = costmodel.init_params(s, np.zeros(s.in_, np.float32), np.ones(s.in_, np.float32))
        net = costmodel.MLP(s, p, device=dev)
        X = torch.from_numpy(rng.standard_normal((2000, s.in_)).astype(np.float32)).to(dev)
        T = torch.from_numpy(rng.standard_normal((2000, s.out)).astype(np.float32)).to(dev)
        Mk = torch.ones_like(T)
        run(lambda: net.forward(X))
        run(lambda: net.loss_grad(X, T, Mk))
        print("mlp: batch 2000")



def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--profile", default=None, choices=["f16", "bf16", "e4m3", "f16_split"])
    ap.add_argument("--launches", type=int, default=3)
    ap.add_argument("--profile-family", default=None,
                    help="comma-separated kernel families to launch for a profiler (see run_profile_families)")
    ap.add_argument("--kernel", type=int, default=0)
    ap.add_argument("--n-tile", type=int, default=0)
    ap.add_argument("--stages", type=int, default=0)
    ap.add_argument("--acc", type=int, default=0)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="auto", choices=["auto", "f16", "bf16", "e4m3", "f16_split"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--pick-from", default=None,
                    help="run the precision and configuration named by an earlier run's JSON line (for profiling)")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-wmma", action="store_true", help="reference arm: skip the reference WMMA kernel timing")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world, rank, local = dist_setup()
    if args.profile_family:
        run_profile_families(args.profile_family, args.launches)
    elif args.profile:
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
