"""Benchmark: bit-ops/s of the bcc Gram pass (bcc_lf_YnWt) on one GB300.

Workload (the case/control configuration): cases 4096 x 16384 SNPs and
controls 4096 x 16384, MAF U[0.05,0.5], 256 x 512 planted bicluster with 5%
flips, rows split uniformly over 2 covariate bins.  One step = the full Gram
pass over all bin pairs (AnZt for every pair, AnAt for nb1 <= nb2): seven
products of the +/-1 centred D-weighted Gram with FP64 scores.

  value  bit-ops/s with every operand already in HBM, the seven products run
         as one grouped persistent launch of the tensor-core kernel
         (lakgb_gram_group_run, after one table launch), timed with CUDA
         events on the launching stream; L2 (129 MB) is flushed before each
         step because the packed inputs (~18 MB) would fit in it.  The same
         pass with one launch per product (lakgb_gram_device, default kernel
         choice) is reported as per_launch_pass, and replayed from a CUDA
         graph as cuda_graph; the grouped outputs are checked bit for bit
         against the per-launch ones before timing.
  e2e    the same pass through the reference-facing C entry points
         (wrap_AnZt_vv__run / wrap_AnAt_vv__run) on host buffers, with the
         bit-matrix upload and the FP64 result download inside the timed region.

Whole solves ("solves" in the JSON line): config 1 (case-only 1024 x 1024,
the reference's CPU-runnable case) timed over repeated lakgb_bcc_solve calls
and checked against the reference's golden trace, and one solve of the
case/control workload; the config-1 solve is also timed on the host cores.

`--impl reference` times the reference's CPU implementation of the pass on
this host's cores instead: the reference compiled from its sources when it is
available here (x86-64 with the reference tree), otherwise the plain-C port of
the same kernels (oracle/liblakoracle.so), OpenMP over all host threads.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "bit-ops/s of Gram pass (bcc_lf_YnWt, case/control 2x(2048+2048) x 16384, B_MLT=32)"
UNIT = "bitop/s"
WORKLOAD = "case_control_4096x4096x16384_2bins_gram_pass"


def _rank_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.dir = tempfile.mkdtemp(prefix="lakgb_clocks_")
        self.path = os.path.join(self.dir, "clocks.csv")

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU: the reference's own kernels (x86 with sources) or the C port


def _cpu_backend():
    ref = os.path.join(ROOT, "oracle", "_ref", "liblakref.so")
    if os.path.exists(ref) and os.uname().machine == "x86_64":
        return "ref", "reference"
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True)
    return "oracle", "port"


def cpu_gram_pass(inst, backend: str, threads: int):
    """Time the Gram pass on the host; returns (seconds, bit-ops)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from lakcluster_c_gb300 import abi
    from lakcluster_c_gb300.abi import MHandle
    from lakcluster_c_gb300.gram_pass import block_allele_freq, products
    import kernel_cases as kc

    lib = kc.load_backend(backend)
    if backend == "oracle":
        lib.lako_set_threads(threads)
    else:
        C.c_int.in_dll(lib, "GLOBAL_omp_type").value = 1
        C.c_int.in_dll(lib, "GLOBAL_thread_count").value = threads
    MA = [MHandle(a) for a in inst.A_bins]
    MZ = [MHandle(z) if z.shape[0] else None for z in inst.Z_bins]
    A_ajdk = abi.calc_A_ajdk(block_allele_freq(inst))
    lf = {}
    for b in range(inst.nbins):
        lf[("A", b)] = kc.lhandle_from(kc.call_an_ajdk(backend, abi.TYPE_pm, abi.SPACING_b, MA[b], A_ajdk),
                                       MA[b].rpop_b, abi.AJDK_TOT, abi.SPACING_b)
        if MZ[b] is not None:
            lf[("Z", b)] = kc.lhandle_from(kc.call_an_ajdk(backend, abi.TYPE_pm, abi.SPACING_b, MZ[b], A_ajdk),
                                           MZ[b].rpop_b, abi.AJDK_TOT, abi.SPACING_b)
    work = 0.0
    t0 = time.perf_counter()
    for kind, nb1, nb2, sym in products(inst.nbins):
        if kind == "AnZt":
            Mz, lz = MZ[nb2], lf.get(("Z", nb2))
        else:
            Mz, lz = MA[nb2], lf[("A", nb2)]
        if Mz is None:
            continue
        kc.call_gram(backend, sym, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_b, MA[nb1], Mz, A_ajdk,
                     lf[("A", nb1)], lz)
        work += float(MA[nb1].rpop_j) * float(Mz.rpop_j) * float(inst.ncols)
    return time.perf_counter() - t0, work


CPU_SAMPLE = "full Gram pass of the workload (cases 4096 + controls 4096 x 16384 SNPs, 2 bins)"


def cpu_sample_instance():
    """The CPU sample is the whole workload: one full pass takes a few seconds
    on the host cores, so no subsampling is needed."""
    from lakcluster_c_gb300 import synth
    return synth.case_control(seed=2)


def run_reference(args):
    rank, world, _ = _rank_env()
    if rank != 0:
        return 0
    backend, kind = _cpu_backend()
    threads = os.cpu_count() or 1
    inst = cpu_sample_instance()
    for _ in range(args.warmup):
        cpu_gram_pass(inst, backend, threads)
    secs, work = 0.0, 0.0
    for _ in range(args.steps):
        s, w = cpu_gram_pass(inst, backend, threads)
        secs += s
        work += w
    value = work / secs
    solves = {"case_only_1024x1024": {"cpu": cpu_solve_c1()}} if not args.no_solves else None
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64-popcount+f64",
        "data": "synthetic", "config": {"workload": WORKLOAD, "sample": CPU_SAMPLE},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": CPU_SAMPLE},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if solves is not None:
        line["solves"] = solves
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU


GRAM_POPCOUNT, GRAM_TENSOR = 0, 1  # lakgb_set_gram_impl


def _ncu_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` recorded by the committed ncu summary
    (a line 'traffic_bytes_per_launch: N' in profiles/<kernel>_*.md), or None."""
    prof = os.path.join(ROOT, "profiles")
    if not os.path.isdir(prof):
        return None
    for name in sorted(os.listdir(prof)):
        if name.startswith(kernel) and name.endswith(".md"):
            with open(os.path.join(prof, name)) as f:
                for line in f:
                    if line.strip().startswith("traffic_bytes_per_launch:"):
                        try:
                            return float(line.split(":", 1)[1].split()[0])
                        except ValueError:
                            return None
    return None


def run_gpu(args):
    import torch
    import torch.distributed as dist

    rank, world, local = _rank_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from lakcluster_c_gb300 import build, synth
    if rank == 0 or world == 1:
        build.build_lib()
    if world > 1:
        dist.barrier()
    from lakcluster_c_gb300._lib import load
    from lakcluster_c_gb300.gram_pass import GramPassDevice, GramPassHost, gram_pass_host

    lib = load()
    # Replicas: each rank runs its own independent instance (weak scaling).
    inst = synth.case_control(seed=2 + rank)
    gp = GramPassHost(inst)
    dev = GramPassDevice(gp)
    work = gp.work_bitops()
    # A dedicated stream: its handle is non-zero, so the library launches on it
    # (a zero handle would select the library's own stream) and the CUDA
    # events below bracket exactly the launched kernels.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    for _ in range(args.warmup):
        flush.zero_()
        dev.run(sh)
    torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    kstart = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    kend = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = lib.lakgb_kernel_launches()
    with ClockSampler(local) as clk:
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            dev.run(sh)
            ends[i].record(stream)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
    launches = lib.lakgb_kernel_launches() - launches0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = sum(step_ms) / len(step_ms)

    # The same pass captured once into a CUDA graph and replayed (every shape
    # class was tuned by the warm-up steps, so nothing in it synchronises).
    graph = None
    try:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            dev.run(sh)
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        gms = []
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            g.replay()
            ends[i].record(stream)
        torch.cuda.synchronize()
        gms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
        gm = sum(gms) / len(gms)
        graph = {"ms_per_step": gm, "value": world * work / (gm / 1000.0),
                 "note": "the seven launches of the pass captured once and replayed as one CUDA graph"}
    except Exception as e:  # capture unsupported here: report why, keep the eager numbers
        graph = {"unavailable": str(e)[:200]}

    # The same pass as ONE grouped persistent launch of the tensor-core kernel
    # over all seven products' tiles (lakgb_gram_group_run); outputs compared
    # bit for bit with the per-launch pass above.
    ref = {k: v.view(torch.int64).clone() for k, v in dev.out.items()}
    for v in dev.out.values():
        v.fill_(float("nan"))
    for _ in range(max(3, args.warmup)):
        flush.zero_()
        dev.run_grouped(sh)
    torch.cuda.synchronize()
    grouped_same = all(torch.equal(dev.out[k].view(torch.int64), ref[k]) for k in ref)
    del ref
    if not grouped_same:
        raise RuntimeError("grouped pass differs from the per-launch pass")
    glaunches0 = lib.lakgb_kernel_launches()
    with ClockSampler(local) as gclk:
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            dev.run_grouped(sh)
            ends[i].record(stream)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
    glaunches = lib.lakgb_kernel_launches() - glaunches0
    gpm = sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / args.steps
    if world > 1:
        t = torch.tensor([ms, gpm], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, gpm = float(t[0].item()), float(t[1].item())
    # The headline: the pass as one grouped launch.  The same pass with one
    # launch per product (the form the reference's call sites make) beside it.
    per_launch = {"ms_per_step": ms, "value": world * work / (ms / 1000.0), "gpu_launches": int(launches),
                  "clocks": clk.summary(),
                  "note": "one lakgb_gram_device launch per product (seven per step), default kernel choice"}
    ms, launches, clk = gpm, glaunches, gclk
    value = world * work / (ms / 1000.0)

    # dominant kernel alone: the largest AnZt launch, timed on its stream,
    # with each of the two Gram kernels (the pass above ran the default one)
    big = dev.args[0]
    big.stream = sh
    lib.lakgb_set_gram_impl.argtypes = [C.c_int]
    lib.lakgb_gram_impl.restype = C.c_int
    lib.lakgb_device_status.restype = C.c_int
    default_impl = lib.lakgb_gram_impl()

    def time_big(impl):
        lib.lakgb_set_gram_impl(impl)
        for _ in range(3):
            lib.lakgb_gram_device(C.byref(big))
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()
            kstart[i].record(stream)
            lib.lakgb_gram_device(C.byref(big))
            kend[i].record(stream)
        torch.cuda.synchronize()
        kt = [s.elapsed_time(e) for s, e in zip(kstart, kend)]
        return sum(kt) / len(kt)

    k_ms_popc = time_big(GRAM_POPCOUNT)
    k_ms = time_big(default_impl)
    lib.lakgb_set_gram_impl(default_impl)
    device_status = lib.lakgb_device_status()
    k_work = float(big.nA) * float(big.nZ) * float(inst.ncols)

    # e2e through the reference-facing C entry points, host buffers, no residency
    lib.lakgb_set_residency(0)
    outputs = {}
    gram_pass_host(gp, outputs)
    e2e_t = []
    d2h = 0
    for _ in range(max(1, min(args.steps, 10))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d2h = gram_pass_host(gp, outputs)
        e2e_t.append(time.perf_counter() - t0)
    lib.lakgb_set_residency(1)
    h2d = 0
    for kind, nb1, nb2, sym in _products(inst.nbins):
        MA = gp.MA[nb1]
        MZ = gp.MZ[nb2] if kind == "AnZt" else gp.MA[nb2]
        if MZ is None:
            continue
        h2d += MA.wX.nbytes + (0 if sym else MZ.wX.nbytes) + MA.mc_length
    e2e_s = statistics.median(e2e_t)

    # CPU baseline on a bounded sample (rank 0, N=1)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        backend, kind = _cpu_backend()
        threads = os.cpu_count() or 1
        sample = cpu_sample_instance()
        cpu_gram_pass(sample, backend, threads)  # warm
        secs, w = 0.0, 0.0
        for _ in range(3):
            s1, w1 = cpu_gram_pass(sample, backend, threads)
            secs += s1
            w += w1
        cpu = {"value": w / secs, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": CPU_SAMPLE + ", 3 passes, %.1f s" % secs}

    large = None
    if rank == 0 and not args.no_large:
        large = large_pass_measurement(args, stream, sh, flush)
    grouped = None
    if rank == 0 and not args.no_grouped:
        grouped = grouped_gram_measurement(stream, sh, flush)
    transpose = None
    if rank == 0 and not args.no_transpose:
        transpose = transpose_measurement(stream, sh, with_cpu=not args.no_cpu_baseline)

    ztswn_ww = None
    if rank == 0 and not args.no_ww:
        ztswn_ww = ztswn_ww_measurement(with_cpu=not args.no_cpu_baseline)

    solves = None
    if rank == 0 and not args.no_solves:
        solves = solve_measurements(args, with_cpu=(world == 1 and not args.no_cpu_baseline))
        if not args.no_many:
            solves.update(many_solves_measurements(args))

    peaks, src = _peaks()
    tflops = 2.0 * k_work / (k_ms / 1000.0) / 1e12
    peak_tf = float(peaks.get("bf16_tflops", 1900.0))
    # The fold of the tensor-core kernel: per output element, one FP64 add per
    # 1920-column block after the first, then the score combine (a0d1 - 2S,
    # and three more operations with the row/column terms).
    P = (inst.ncols + 1919) // 1920
    fp64_per_elem = (P - 1) + 1 + (3 if (big.lfA and big.lfZ) else 0)
    fp64_ops = float(big.nA) * float(big.nZ) * fp64_per_elem
    fp64_rate = lib.lakgb_measure_fp64_add_rate()
    traffic = _ncu_traffic("gram_tc_kernel_case_control")
    g_traffic = _ncu_traffic("gram_tc_kernel_grouped")
    g_tflops = 2.0 * work / (ms / 1000.0) / 1e12
    # computed elements of the pass (symmetric products: the upper triangle)
    pass_fp64 = sum((float(a.nA) * (a.nA + 1) / 2 if a.symmetric else float(a.nA) * a.nZ) for a in dev.args)
    pass_fp64 *= fp64_per_elem
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    clocks = clk.summary()
    mhz = clocks.get("sm_mhz") or 1920.0
    popc_peak = 16 * 32 * sm_count * mhz * 1e6  # POPC issue rate: 16 lanes/clk/SM x 32 bits
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "e4m3-bit-mma+f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "bins": inst.nbins, "cases": 4096, "controls": 4096,
                       "snps": inst.ncols, "products_per_step": len(dev.args),
                       "pass_form": "one grouped persistent tcgen05 launch over all products' tiles "
                                    "(lakgb_gram_group_run) after one table launch; per_launch_pass has the "
                                    "same pass as one launch per product",
                       "l2": "flushed before each step (256 MB write)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "gpu_launches": int(launches),
            "roofline": {
                "bound": "tensor", "achieved": g_tflops, "peak": peak_tf, "unit": "TFLOP/s",
                "frac": g_tflops / peak_tf, "traffic": g_traffic,
                "kernel": "gram_tc_kernel<1, grouped> (tcgen05 e4m3): the pass's one persistent launch over "
                          "the seven products' tiles",
                "note": ("bit-pair products counted as 2 ops (one MAC) against the %s dense bf16 tensor peak "
                         "(the e4m3 MMA the kernel issues is nominally 2x the bf16 rate); launch time = the "
                         "step's CUDA-event time, which also holds the table launch (about 4 us). traffic: DRAM "
                         "bytes of one launch from the committed ncu capture (profiles/), null when absent" % src),
                "fp64_pipe": {"achieved_ops_per_s": pass_fp64 / (ms / 1000.0), "peak_adds_per_s": fp64_rate,
                              "frac": pass_fp64 / (ms / 1000.0) / fp64_rate, "ops_per_launch": pass_fp64,
                              "note": "FP64 operations of the fold and score combine (%d per computed element) "
                                      "against the add rate measured live on this GPU "
                                      "(lakgb_measure_fp64_add_rate)" % fp64_per_elem},
                "vs_int_pipe_roofline": {
                    "achieved_bitops": work / (ms / 1000.0), "int_pipe_peak_bitops": popc_peak,
                    "ratio": (work / (ms / 1000.0)) / popc_peak,
                    "note": "the pass against the integer-pipe roofline of a popcount Gram (POPC at 16 lanes/clk/SM "
                            "x 32 bits, sampled SM clock): above 1 means faster than any popcount kernel can run"},
                "largest_single_launch": {
                    "kernel": "gram_tc_kernel<1> alone on the largest AnZt product, %dx%d rows, %d blocks"
                              % (big.nA, big.nZ, P),
                    "kernel_ms": k_ms, "achieved": tflops, "frac": tflops / peak_tf, "traffic": traffic,
                    "fp64_pipe_frac": fp64_ops / (k_ms / 1000.0) / fp64_rate,
                    "vs_int_pipe_roofline": (k_work / (k_ms / 1000.0)) / popc_peak,
                    "note": "not the sole bound: copies of the kernel without the FP64 adds, or without the "
                            "table loads, run at most 6 % faster"},
                "popcount_kernel": {"kernel_ms": k_ms_popc, "achieved_bitops": k_work / (k_ms_popc / 1000.0),
                                    "int_pipe_peak_bitops": popc_peak,
                                    "int_pipe_frac": (k_work / (k_ms_popc / 1000.0)) / popc_peak,
                                    "note": "the CUDA-core kernel on the largest product; POPC issue-rate bound, "
                                            "16 lanes/clk/SM x 32 bits at the sampled SM clock"},
            },
            "device_status": device_status,
            "per_launch_pass": per_launch,
            "cuda_graph": graph,
            "e2e": {"value": work / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "seconds_per_step": e2e_s},
            "clocks": clocks,
        }
        if cpu is not None:
            line["cpu_baseline"] = cpu
        if large is not None:
            line["large_gram_pass"] = large
        if grouped is not None:
            line["grouped_null_gram_passes"] = grouped
        if transpose is not None:
            line["b16_transpose"] = transpose
        if ztswn_ww is not None:
            line["an_ztswn_yt_ww"] = ztswn_ww
        line["gram_autotune"] = autotune_summary(lib)
        if solves is not None:
            line["solves"] = solves
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def autotune_summary(lib):
    """The Gram autotuner's decisions: how many shape classes took each
    kernel, and the first few classes with the times seen."""
    n = lib.lakgb_gram_autotune_table(None, 0)
    buf = C.create_string_buffer(n + 1)
    lib.lakgb_gram_autotune_table(buf, len(buf))
    table = json.loads(buf.value.decode() or "[]")
    chosen = {}
    for e in table:
        chosen[e["choice"]] = chosen.get(e["choice"], 0) + 1
    return {"classes": len(table), "chosen": chosen, "first_classes": table[:6]}


def large_pass_measurement(args, stream, sh, flush):
    """The Gram pass of the large configuration (cases 32768 + controls 32768 x
    131072 SNPs, 3 bins; 15 launches), inputs drawn on the device: every
    product run with both Gram kernels and compared bit for bit, sampled
    entries recomputed on the host, then the pass timed with each kernel."""
    import torch
    from lakcluster_c_gb300.large_pass import POPCOUNT, TENSOR, LargeGramPass

    t0 = time.perf_counter()
    lp = LargeGramPass()
    setup_s = time.perf_counter() - t0
    checks = lp.run_checks()
    work = lp.work_bitops()
    lib = lp.lib
    default_impl = lib.lakgb_gram_impl()
    timings = {}
    for impl, name, reps in ((TENSOR, "tensor", 3), (POPCOUNT, "popcount", 1)):
        lib.lakgb_set_gram_impl(impl)
        lp.run(sh)  # warm
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lp.run(sh)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        timings[name] = {"ms_per_pass": statistics.median(ms), "bitops_per_s": work / (statistics.median(ms) / 1e3),
                         "reps": reps}
    lib.lakgb_set_gram_impl(default_impl)
    return {"workload": "case_control_32768x32768x131072_3bins_gram_pass", "launches": len(lp.args),
            "bitops_per_pass": work, "setup_seconds": setup_s, "checks": checks, **timings,
            "note": "operands drawn on the device (MAF U[0.01,0.5], 2048x4096 planted, 5% flips); row terms from "
                    "wrap_An_ajdk_v; host recomputation of sampled entries in block order"}


def grouped_gram_measurement(stream, sh, flush):
    """The Gram passes of the batched-null instances (24 label-shuffled
    case/control problems, rows logU[1024,8192], SNPs logU[4096,32768], one
    bin; 48 launches): one launch per product (the plain path, default kernel
    choice) against one grouped persistent launch of the tensor-core kernel
    (lakgb_gram_group_run), direct and replayed from a CUDA graph.  Outputs of
    the grouped launch are compared bit for bit with the plain path's."""
    import torch
    from lakcluster_c_gb300 import synth
    from lakcluster_c_gb300.large_pass import GroupedGramPasses, LargeGramPass

    passes = []
    for i in range(24):
        rng = np.random.default_rng(1000 + i)
        r = synth.log_uniform_int(rng, 1024, 8192)
        c = synth.log_uniform_int(rng, 4096, 32768)
        na = r // 2
        passes.append(LargeGramPass(n_cases=na, n_controls=r - na, ncols=c, nbins=1,
                                    planted=(min(na, max(2, r // 16)), max(2, c // 32)), maf=(0.05, 0.5),
                                    seed=1000 + i))
    g = GroupedGramPasses(passes)
    work = g.work_bitops()
    nan = float("nan")

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return statistics.median(ms)

    plain_ms = timed(lambda: g.run_plain(sh))
    want = [o.view(torch.int64).clone() for o in g.outputs()]

    def reset():
        for o in g.outputs():
            o.fill_(nan)
        torch.cuda.synchronize()

    reset()
    grouped_ms = timed(lambda: g.run_grouped(sh))
    same = all(torch.equal(o.view(torch.int64), w) for o, w in zip(g.outputs(), want))
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        g.run_grouped(stream.cuda_stream)
    reset()
    graph_ms = timed(lambda: graph.replay())
    graph_same = all(torch.equal(o.view(torch.int64), w) for o, w in zip(g.outputs(), want))
    launches = g.n
    g.close()
    del want, graph
    return {"workload": "24 null instances' Gram passes (rows logU[1024,8192], SNPs logU[4096,32768], 1 bin)",
            "launches_plain": launches, "bitops": work,
            "plain": {"ms": plain_ms, "bitops_per_s": work / (plain_ms / 1e3)},
            "grouped": {"ms": grouped_ms, "bitops_per_s": work / (grouped_ms / 1e3), "identical_to_plain": same},
            "grouped_cuda_graph": {"ms": graph_ms, "bitops_per_s": work / (graph_ms / 1e3),
                                   "identical_to_plain": graph_same},
            "speedup_grouped_graph": plain_ms / graph_ms,
            "note": "operands drawn on the device with the instances' shapes; one grouped launch = the table "
                    "kernel for every instance's blocks + one persistent tcgen05 launch over all instances' tiles"}


def transpose_measurement(stream, sh, with_cpu: bool):
    """The .b16 transposer (wrap_transpose, dir_c/binary_read.c:174): the
    kernel on a matrix of the large configuration's size (131072 records of
    32768 bits, 512 MB each way) against the measured HBM copy bandwidth; the
    file-to-file call on a 64 MB file; the C oracle on the host cores on an
    8192 x 8192-bit sample."""
    import tempfile
    import torch
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from lakcluster_c_gb300 import infiles
    from lakcluster_c_gb300._lib import load

    lib = load()
    peaks, src = _peaks()
    n_rec, n_bits = 131072, 32768
    nbytes = n_rec * n_bits // 8
    d_in = torch.randint(0, 256, (nbytes,), dtype=torch.uint8, device="cuda")
    d_out = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    for _ in range(3):
        lib.lakgb_bits_transpose_device(d_in.data_ptr(), n_rec, n_bits, d_out.data_ptr(), C.c_void_p(sh))
    torch.cuda.synchronize()
    ms = []
    for _ in range(10):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        lib.lakgb_bits_transpose_device(d_in.data_ptr(), n_rec, n_bits, d_out.data_ptr(), C.c_void_p(sh))
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    k_ms = statistics.median(ms)
    gbs = 2.0 * nbytes / (k_ms / 1e3) / 1e9
    del d_in, d_out
    out = {"kernel": {"records": n_rec, "bits_per_record": n_bits, "bytes_each_way": nbytes, "ms": k_ms,
                      "achieved_gbs": gbs, "peak_gbs": float(peaks.get("hbm_gbs", 6800.0)),
                      "frac": gbs / float(peaks.get("hbm_gbs", 6800.0)),
                      "note": "bytes read + bytes written per launch over its CUDA-event time, against the %s "
                              "HBM copy bandwidth (inputs 512 MB, larger than L2)" % src}}
    rng = np.random.default_rng(11)
    x = (rng.random((8192, 65536)) < 0.5).astype(np.uint8)
    with tempfile.TemporaryDirectory() as td:
        p_in, p_out = os.path.join(td, "x.b16"), os.path.join(td, "x_t.b16")
        infiles.write_b16(p_in, x)
        lib.wrap_transpose(p_in.encode(), p_out.encode(), 1 << 20)  # warm
        t = []
        for _ in range(3):
            t0 = time.perf_counter()
            lib.wrap_transpose(p_in.encode(), p_out.encode(), 1 << 20)
            t.append(time.perf_counter() - t0)
        fb = os.path.getsize(p_in)
        out["file_to_file"] = {"file_bytes": fb, "seconds": min(t), "gbs": 2.0 * fb / min(t) / 1e9,
                               "note": "wrap_transpose on a 64 MB .b16 file (8192 records of 65536 bits): "
                                       "read, upload, kernel, download, write"}
    if with_cpu:
        import kernel_cases as kc
        n, m = 8192, 8192
        a = np.random.default_rng(12).integers(0, 256, n * m // 8, dtype=np.uint8)
        b = np.zeros_like(a)
        lib_o = kc.load_backend("oracle")
        t0 = time.perf_counter()
        lib_o.lako_bits_transpose(a.ctypes.data_as(C.c_void_p), C.c_longlong(m // 8), n,
                                  b.ctypes.data_as(C.c_void_p), C.c_longlong(n // 8), m)
        cs = time.perf_counter() - t0
        out["cpu_baseline"] = {"gbs": 2.0 * a.size / cs / 1e9, "seconds": cs, "cores": os.cpu_count(),
                               "kind": "port", "sample": "8192 records of 8192 bits (8 MB) on the C oracle"}
    return out


def solve_measurements(args, with_cpu: bool):
    """Whole-solve timings: config 1 (case-only 1024 x 1024, the reference's
    CPU-runnable case) and the case/control workload above, through
    lakgb_bcc_solve from host arrays (uploads and downloads included), and the
    same config-1 solve on the host cores."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import bcc_cases as bc
    from lakcluster_c_gb300 import solve as sv, synth

    golden = bc.load_golden()
    out = {}
    d1 = bc.build("case_only_1024x1024")
    p1 = sv.Problem(d1["A"], None, gamma=d1["gamma"])
    r = p1.solve()
    same1 = all(r[k] == golden["case_only_1024x1024"][k] for k in ("trace", "xdrop_a", "xdrop_b"))
    t = []
    for _ in range(max(3, min(args.steps, 5))):
        t0 = time.perf_counter()
        p1.solve()
        t.append(time.perf_counter() - t0)
    s1 = statistics.median(t)
    out["case_only_1024x1024"] = {"seconds": s1, "solves_per_s": 1.0 / s1, "iterations": len(r["trace"]),
                                  "matches_reference": same1, "reps": len(t)}
    inst = synth.case_control(seed=2)
    p2 = sv.Problem(inst.A_bins, inst.Z_bins, gamma=0.05)
    t0 = time.perf_counter()
    r2 = p2.solve()  # first solve of the process: includes the Gram autotuner's one-time measurements
    first = time.perf_counter() - t0
    t = []
    for _ in range(2):
        t0 = time.perf_counter()
        r2b = p2.solve()
        t.append(time.perf_counter() - t0)
    s2 = statistics.median(t)
    c2 = {"seconds": s2, "solves_per_s": 1.0 / s2, "iterations": len(r2["trace"]), "reps": len(t),
          "first_solve_seconds": first, "repeat_identical": r2b == r2}
    if "case_control_4096x4096x16384" in golden:  # from the oracle port (reference too slow)
        g = golden["case_control_4096x4096x16384"]
        c2["matches_oracle_port"] = all(r2[k] == g[k] for k in ("trace", "xdrop_a", "xdrop_b"))
    out["case_control_4096x4096x16384"] = c2
    if with_cpu:
        out["case_only_1024x1024"]["cpu"] = cpu_solve_c1()
    return out


def many_solves_measurements(args):
    """Batched label-shuffled nulls and a served Poisson stream, each against
    the plain one-solve-at-a-time path on the same problems (results must be
    identical)."""
    from lakcluster_c_gb300 import serve, solve as sv, synth
    workers = max(2, min(16, os.cpu_count() or 2))
    out = {}
    # Batched nulls: label-shuffled case/control instances of uneven sizes.
    n_null = 24
    probs = []
    for i in range(n_null):
        inst = synth.null_instance(1000 + i, rows=(1024, 8192), cols=(4096, 32768))
        probs.append(sv.Problem(inst.A_bins, inst.Z_bins, gamma=0.05))
    plain, t_plain = serve.solve_plain(probs)
    batched, t_batch, peak = serve.solve_batched(probs, workers=workers)
    out["batched_nulls"] = {
        "instances": n_null, "rows": "logU[1024,8192]", "cols": "logU[4096,32768]", "workers": workers,
        "plain_solves_per_s": n_null / t_plain, "batched_solves_per_s": n_null / t_batch,
        "speedup": t_plain / t_batch, "peak_concurrency": peak, "identical_to_plain": batched == plain}
    # Served stream: Poisson arrivals at twice the plain path's throughput.
    n_req = 16
    reqs = []
    for i in range(n_req):
        inst = synth.served_request(5000 + i, rows=(512, 4096), cols=(2048, 16384))
        reqs.append(sv.Problem(inst.A_bins, inst.Z_bins, gamma=0.05))
    solo, t_solo = serve.solve_plain(reqs)
    rate = 2.0 * n_req / t_solo
    r1, lat1, wall1, _ = serve.serve_stream(reqs, rate, workers=1, seed=7)
    rw, latw, wallw, peakw = serve.serve_stream(reqs, rate, workers=workers, seed=7)
    out["served"] = {
        "requests": n_req, "rows": "logU[512,4096]", "cols": "logU[2048,16384]", "categories": "U{0..3}",
        "arrival_rate_per_s": rate, "workers": workers,
        "plain": dict(serve.latency_stats(lat1), solves_per_s=n_req / wall1),
        "continuous_batching": dict(serve.latency_stats(latw), solves_per_s=n_req / wallw, peak_concurrency=peakw),
        "identical_to_solo": (r1 == solo) and (rw == solo)}
    return out


def cpu_solve_c1():
    """Config-1 solve on the host cores: the reference program where it
    builds (x86-64 with its sources), else the solve driver on the C oracle."""
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import bcc_cases as bc
    threads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as td:
        p = bc.write_case("case_only_1024x1024", os.path.join(td, "in"), os.path.join(td, "out"))
        txt = open(p).read().replace("GLOBAL_thread_count= 1;", "GLOBAL_thread_count= %d;" % threads)
        txt = txt.replace("GLOBAL_omp_type= 0;", "GLOBAL_omp_type= 1;")
        open(p, "w").write(txt)
        if os.path.exists(bc.REF_PROGRAM) and os.uname().machine == "x86_64":
            cmd, kind = None, "reference"
        else:
            subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
            cmd, kind = [os.path.join(ROOT, "oracle", "lakbcc_port"), p, str(threads)], "port"
        t = []
        for _ in range(2):
            t0 = time.perf_counter()
            if cmd is None:
                bc.run_reference(p)
            else:
                subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
            t.append(time.perf_counter() - t0)
    s = min(t)
    return {"seconds": s, "solves_per_s": 1.0 / s, "cores": threads, "kind": kind, "reps": len(t)}


def _products(nbins):
    from lakcluster_c_gb300.gram_pass import products
    return products(nbins)


def ztswn_ww_measurement(with_cpu: bool):
    """The bit-plane loop product An_ZtSWn_Yt_ww (dir_c/An_ZtSWn_Yt_ww.c:5-111):
    2048 patient rows x 16384 SNPs against the 32-bit planes of 1024 Wt rows
    (one covariate column), operands resident; median of 5 calls, each with its
    small uploads and its 16 KB download.  Work counted as the reference counts
    it (:108): rows x covariates x Wt rows x ncols_per_z x padded SNP bits,
    against the integer-pipe roofline (POPC, 16 lanes/clk/SM x 32 bits at the
    maximum SM clock).  The first 64 rows are checked against the C oracle,
    which is also timed on them."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from lakcluster_c_gb300 import abi
    from lakcluster_c_gb300._lib import load

    lib = load()
    rng = np.random.default_rng(21)
    n, m, nw, B = 2048, 16384, 1024, 32
    mcl, ycl = abi.bsize(m), abi.bsize(nw)
    a_bytes = rng.integers(0, 256, (n, mcl), dtype=np.uint8)
    y_bytes = rng.integers(0, 256, (n, ycl), dtype=np.uint8)

    def handles(rows):
        An = abi.MHandle(None, nrows=rows, ncols=m, wX=a_bytes[:rows])
        Yn = abi.MHandle(None, nrows=rows, ncols=nw, wX=y_bytes[:rows])
        return An, Yn

    Wt = abi.MHandle(None, nrows=nw, ncols=16, wX=np.zeros((nw, abi.bsize(16)), np.uint8))
    St = abi.MHandle(None, nrows=1, ncols=16, wX=np.zeros((1, abi.bsize(16)), np.uint8))
    pl = abi.MHandle(None, nrows=(B + 1) * nw, ncols=m,
                     wX=rng.integers(0, 256, ((B + 1) * nw, mcl), dtype=np.uint8))
    pl.s.ncols_per_z, pl.s.min_d, pl.s.mlt_d = B + 1, -2.5, float(2 ** 32) / 7.0
    arr = (C.POINTER(abi.M_handle) * 1)(C.pointer(pl.s))
    A_ajdk = abi.calc_A_ajdk(0.05 + 0.9 * rng.random(abi.psize(m)))
    Y_ajdk = abi.calc_A_ajdk(0.05 + 0.9 * rng.random(abi.psize(nw)))
    dp = C.POINTER(C.c_double)

    def call(fn, An, Yn, gpu):
        out = C.POINTER(abi.L_handle)()
        args = (abi.SPACING_a, abi.SPACING_a, An.ptr, St.ptr, arr, Wt.ptr, Yn.ptr, A_ajdk.ctypes.data_as(dp),
                Y_ajdk.ctypes.data_as(dp), C.byref(out))
        k = fn(C.byref(C.c_int(0)), (C.c_void_p * 128)(), None, *args) if gpu else fn(*args)
        return np.ctypeslib.as_array(C.cast(out.contents.lf, dp), (k,)).copy()

    An, Yn = handles(n)
    lib.lakgb_set_residency(1)
    try:
        got = call(lib.wrap_An_ZtSWn_Yt_ww__run, An, Yn, True)
        t = []
        for _ in range(5):
            t0 = time.perf_counter()
            call(lib.wrap_An_ZtSWn_Yt_ww__run, An, Yn, True)
            t.append(time.perf_counter() - t0)
    finally:
        lib.lakgb_set_residency(0)
    secs = statistics.median(t)
    work = float(n) * 1 * nw * (B + 1) * mcl * 8
    peak = 16.0 * 32 * 152 * 2070e6
    out = {"workload": "2048 rows x 16384 SNPs, 1024 Wt rows x 33 planes, 1 covariate column",
           "seconds": secs, "bitops": work, "bitops_per_s": work / secs, "int_pipe_peak_bitops": peak,
           "int_pipe_frac": work / secs / peak, "device_status": int(lib.lakgb_device_status())}
    import kernel_cases as kc
    lib_o = kc.load_backend("oracle")
    As, Ys = handles(64)
    t0 = time.perf_counter()
    want = call(lib_o.lako_An_ZtSWn_Yt_ww, As, Ys, False)
    cs = time.perf_counter() - t0
    out["first_64_rows_equal_oracle"] = bool(np.array_equal(got[:64].view(np.uint64), want[:64].view(np.uint64)))
    if with_cpu:
        out["cpu_baseline"] = {"bitops_per_s": work * 64 / n / cs, "seconds": cs, "cores": os.cpu_count(),
                               "kind": "port", "sample": "the first 64 rows on the C oracle"}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-solves", action="store_true", help="skip the whole-solve timings")
    ap.add_argument("--no-many", action="store_true", help="skip the batched / served timings")
    ap.add_argument("--no-transpose", action="store_true", help="skip the .b16 transposer measurement")
    ap.add_argument("--no-ww", action="store_true", help="skip the An_ZtSWn_Yt_ww bit-plane product measurement")
    ap.add_argument("--no-grouped", action="store_true",
                    help="skip the grouped Gram passes of the batched-null instances")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the large-configuration Gram pass (32768 + 32768 x 131072)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
