"""Benchmark: bit-ops/s of the bcc Gram pass (bcc_lf_YnWt) on one GB300.

Workload (the large single-solve configuration, the largest that the metric
is quoted on and that fits one GPU): cases 32768 and controls 32768 x 131072
SNPs, MAF U[0.01,0.5], a 2048 x 4096 planted bicluster with 5% flips, rows
assigned uniformly to 3 covariate bins.  One step = the full Gram pass over
all bin pairs (AnZt for every pair, AnAt for nb1 <= nb2): 15 products of the
+/-1 centred D-weighted Gram with FP64 scores, 2.35e14 bit pairs.  The packed
inputs (1.08 GB) are larger than L2, so no flush is needed between steps.

  value  bit-ops/s with every operand already in HBM, the 15 products run as
         one persistent launch of the tensor-core kernel each
         (lakgb_gram_device), timed with CUDA events on the launching
         stream; the same pass as one grouped launch (lakgb_gram_group_run)
         is checked bit for bit against it and reported beside it, and every
         product is also run with the CUDA-core popcount kernel and compared.
  e2e    the same pass through the reference-facing C entry points
         (wrap_AnZt_vv__run / wrap_AnAt_vv__run) on host buffers: the packed
         bins uploaded once per pass from pinned memory, the 14.3 GB of FP64
         scores copied back, inside the timed region; checked bit for bit
         against the device-resident pass.

The host-core baseline times one product of this shape on a row subset
(6144 case x 6144 control rows x 131072 SNPs) with the reference's kernels
where they build (x86-64 with the reference tree) or the plain-C port of the
same kernels (oracle/liblakoracle.so), OpenMP over all host threads.
`--impl reference` runs that CPU path as the reference arm.

Extras in the same JSON line: the case/control configuration's pass (cases
4096 + controls 4096 x 16384, 2 bins), the batched-null Gram passes, the .b16
transposer, the bit-plane An_ZtSWn_Yt_ww product, whole solves, batched nulls
and a served stream.
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

METRIC = ("bit-ops/s of Gram pass (bcc_lf_YnWt; large case/control: cases 32768 + controls 32768 x 131072 SNPs, "
          "3 bins, B_MLT=32)")
UNIT = "bitop/s"
WORKLOAD = "case_control_32768x32768x131072_3bins_gram_pass"
CONFIG = {"workload": WORKLOAD, "cases": 32768, "controls": 32768, "snps": 131072, "bins": 3,
          "products_per_step": 15, "maf": "U[0.01,0.5]", "planted": "2048x4096, 5% flips",
          "l2": "no flush: the packed inputs (1.08 GB) are larger than L2 (129 MB)"}
LARGE_CPU_ROWS = 6144
CPU_SAMPLE = ("one AnZt product of the workload's shape on a row subset: %d case x %d control rows x 131072 SNPs "
              "(MAF U[0.01,0.5], planted rows with 5%% flips), D-weighted with row terms, rows drawn on the host"
              % (LARGE_CPU_ROWS, LARGE_CPU_ROWS))


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


# ---------------------------------------------------------------------------
# CPU: the reference's own kernels (x86 with sources) or the C port, on a
# bounded sample of the large workload


class CpuLargeSample:
    """One AnZt product of the large workload's shape on a row subset, on the
    host cores: LARGE_CPU_ROWS case rows x LARGE_CPU_ROWS control rows x all
    131072 SNPs, D-weighted with the AJDK_1_1 row terms (the arithmetic of
    every product of the pass).  Rows are drawn on the host with the
    workload's distributions; timing does not depend on the bit values."""

    def __init__(self, backend: str, threads: int, n_rows: int, ncols: int = 131072):
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from lakcluster_c_gb300 import abi
        from lakcluster_c_gb300.large_pass import host_rows
        import kernel_cases as kc

        self.backend, self.kc, self.abi = backend, kc, abi
        self.lib = kc.load_backend(backend)
        if backend == "oracle":
            self.lib.lako_set_threads(threads)
        else:
            C.c_int.in_dll(self.lib, "GLOBAL_omp_type").value = 1
            C.c_int.in_dll(self.lib, "GLOBAL_thread_count").value = threads
        A = host_rows(n_rows, ncols, seed=3)
        Z = host_rows(n_rows, ncols, planted=(0, 0), seed=4)
        self.MA = abi.MHandle(None, wX=A, nrows=n_rows, ncols=ncols)
        self.MZ = abi.MHandle(None, wX=Z, nrows=n_rows, ncols=ncols)
        P = abi.psize(ncols)
        pc = np.unpackbits(np.arange(256, dtype=np.uint8)[:, None], axis=1).sum(1)
        cnt = pc[A.reshape(n_rows, P, abi.POPLENGTH // 8)].sum(axis=(0, 2)).astype(np.float64)
        bits = np.minimum(abi.POPLENGTH, ncols - abi.POPLENGTH * np.arange(P)).astype(np.float64)
        self.A_ajdk = abi.calc_A_ajdk(cnt / (bits * n_rows))
        self.lfA = kc.lhandle_from(kc.call_an_ajdk(backend, abi.TYPE_pm, abi.SPACING_b, self.MA, self.A_ajdk),
                                   self.MA.rpop_b, abi.AJDK_TOT, abi.SPACING_b)
        self.lfZ = kc.lhandle_from(kc.call_an_ajdk(backend, abi.TYPE_pm, abi.SPACING_b, self.MZ, self.A_ajdk),
                                   self.MZ.rpop_b, abi.AJDK_TOT, abi.SPACING_b)
        self.work = float(n_rows) * float(n_rows) * float(ncols)
        self.out = C.POINTER(abi.L_handle)()

    def step(self) -> float:
        """One product; returns its wall time (s)."""
        abi, kc = self.abi, self.kc
        aj = self.A_ajdk.ctypes.data_as(C.POINTER(C.c_double))
        t0 = time.perf_counter()
        if self.backend == "oracle":
            self.lib.lako_AnZt_vv(abi.TYPE_pm, abi.SPACING_b, abi.SPACING_b, self.MA.ptr, self.MZ.ptr, aj,
                                  self.lfA.ptr, self.lfZ.ptr, C.byref(self.out))
        else:
            self.lib.wrap_AnZt_vv__run(*kc._thread_args(), abi.TYPE_pm, abi.SPACING_b, abi.SPACING_b,
                                       self.MA.ptr, self.MZ.ptr, aj, self.lfA.ptr, self.lfZ.ptr, C.byref(self.out))
        return time.perf_counter() - t0


def run_reference(args):
    rank, world, _ = _rank_env()
    if rank != 0:
        return 0
    backend, kind = _cpu_backend()
    threads = os.cpu_count() or 1
    smp = CpuLargeSample(backend, threads, LARGE_CPU_ROWS)
    for _ in range(args.warmup):
        smp.step()
    secs = sum(smp.step() for _ in range(args.steps))
    value = smp.work * args.steps / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64-popcount+f64",
        "data": "synthetic", "config": dict(CONFIG, parallelism="replicas" if world > 1 else "single"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": CPU_SAMPLE},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU


GRAM_POPCOUNT, GRAM_TENSOR = 0, 1  # lakgb_set_gram_impl


def _ncu_figures(prefix: str):
    """Figures recorded by a committed ncu summary profiles/<prefix>*.md as
    lines 'name: value' (traffic_bytes_per_launch, bitops_per_launch), or {}."""
    prof = os.path.join(ROOT, "profiles")
    out = {}
    if not os.path.isdir(prof):
        return out
    for name in sorted(os.listdir(prof)):
        if name.startswith(prefix) and name.endswith(".md"):
            with open(os.path.join(prof, name)) as f:
                for line in f:
                    k, _, v = line.strip().partition(":")
                    if k in ("traffic_bytes_per_launch", "bitops_per_launch") and v.strip():
                        try:
                            out[k] = float(v.split()[0])
                        except ValueError:
                            pass
            out["file"] = name
            break
    return out


def _timed_steps(stream, fn, steps):
    import torch
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for i in range(steps):
        starts[i].record(stream)
        fn()
        ends[i].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in zip(starts, ends)]


def large_pass_headline(args, lib, stream, sh, rank, world, local):
    """The headline: the Gram pass of the large configuration, one grouped
    persistent launch over its 15 products' tiles (after one table launch),
    operands and outputs in HBM; its per-launch form, both Gram kernels on
    every product, the pass from host buffers through the reference-facing
    entry points, and the roofline figures."""
    import torch
    import torch.distributed as dist
    from lakcluster_c_gb300.large_pass import POPCOUNT, GroupedGramPasses, LargeGramPass, LargeGramPassHost

    t0 = time.perf_counter()
    lp = LargeGramPass(seed=3 + rank)
    setup_s = time.perf_counter() - t0
    work = lp.work_bitops()
    g = GroupedGramPasses([lp])
    # The grouped launch must give the per-launch pass's outputs bit for bit.
    g.run_plain(sh)
    torch.cuda.synchronize()
    want = [o.view(torch.int64).clone() for o in g.outputs()]
    for o in g.outputs():
        o.fill_(float("nan"))
    g.run_grouped(sh)
    torch.cuda.synchronize()
    grouped_same = all(torch.equal(o.view(torch.int64), w) for o, w in zip(g.outputs(), want))
    del want
    if not grouped_same:
        raise RuntimeError("grouped pass differs from the per-launch pass")
    for _ in range(args.warmup):
        g.run_plain(sh)
    torch.cuda.synchronize()
    launches0 = lib.lakgb_kernel_launches()
    with ClockSampler(local) as clk:
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        step_ms = _timed_steps(stream, lambda: g.run_plain(sh), args.steps)
        if world > 1:
            dist.barrier()
    launches = lib.lakgb_kernel_launches() - launches0
    ms = sum(step_ms) / len(step_ms)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t[0].item())
    value = world * work / (ms / 1000.0)
    device_status = lib.lakgb_device_status()

    # e2e: the reference-facing entry points on host buffers
    host = LargeGramPassHost(lp, pinned_outputs=True)
    lib.lakgb_set_residency(1)
    try:
        host.forget_inputs()
        d2h = host.run()
        same_host = True
        for (key, a, n), out in zip(lp.args, g.outputs()):
            hv = host.output(key)[:n].view(np.uint64)
            same_host = same_host and np.array_equal(hv, out[:n].view(torch.int64).cpu().numpy().view(np.uint64))
        e2e_t = []
        with ClockSampler(local) as e2e_clk:
            for _ in range(max(1, min(args.steps, 4))):
                host.forget_inputs()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                d2h = host.run()
                e2e_t.append(time.perf_counter() - t0)
        host.forget_inputs()
        call_s = host.run_timed()
    finally:
        host.forget_inputs()
        lib.lakgb_set_residency(0)
    e2e_s = statistics.median(e2e_t)
    h2d = host.h2d_bytes()
    e2e = {"value": world * work / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "seconds_per_step": e2e_s, "identical_to_device_pass": same_host,
           "pass_seconds": e2e_t, "call_seconds_one_pass": call_s, "clocks": e2e_clk.summary(),
           "note": "15 calls of wrap_AnZt_vv__run / wrap_AnAt_vv__run on host M_handles (pinned packed bins, "
                   "uploaded once per pass: residency on, the bins forgotten before every pass) into caller-owned "
                   "host L_handles over page-locked memory (14.3 GB of FP64 scores copied back per pass)"}

    # the same pass as one grouped persistent launch over all products' tiles
    pl = _timed_steps(stream, lambda: g.run_grouped(sh), max(3, min(args.steps, 10)))
    # both Gram kernels on every product, bit for bit; sampled entries on the host
    checks = lp.run_checks() if rank == 0 else None
    popc = None
    if rank == 0:
        default_impl = lib.lakgb_gram_impl()
        lib.lakgb_set_gram_impl(POPCOUNT)
        try:
            pms = _timed_steps(stream, lambda: lp.run(sh), 1)[0]
        finally:
            lib.lakgb_set_gram_impl(default_impl)
        popc = {"ms_per_pass": pms, "bitops_per_s": work / (pms / 1e3),
                "note": "the CUDA-core popcount Gram on every product of the pass, one launch each"}

    # roofline figures of the dominant kernel (one launch per product)
    peaks, src = _peaks()
    peak_tf = float(peaks.get("bf16_tflops", 1900.0))
    peak_tf_sus = float(peaks.get("bf16_tflops_sustained", peak_tf))
    tflops = 2.0 * work / (ms / 1000.0) / 1e12
    P = lp.P
    fp64_per_elem = (P - 1) + 4  # block adds after the first, then the score combine with row terms
    elems = 0.0
    for (kind, nb1, nb2, sym), a, n in lp.args:
        elems += float(a.nA) * (a.nA + 1) / 2 if sym else float(a.nA) * a.nZ
    fp64_rate = lib.lakgb_measure_fp64_add_rate()
    prof = _ncu_figures("gram_tc_kernel_large")
    traffic = None
    if "traffic_bytes_per_launch" in prof and prof.get("bitops_per_launch"):
        traffic = prof["traffic_bytes_per_launch"] * work / prof["bitops_per_launch"]
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    clocks = clk.summary()
    mhz = clocks.get("sm_mhz") or 1920.0
    popc_peak = 16 * 32 * sm_count * mhz * 1e6
    roof = {
        "bound": "tensor", "achieved": tflops, "peak": peak_tf, "unit": "TFLOP/s", "frac": tflops / peak_tf,
        "traffic": traffic,
        "kernel": "gram_tc_kernel<1> (tcgen05 e4m3 counts + FP64 fold), one persistent launch per product",
        "note": ("bit pairs of the pass (full square for AnAt) counted as 2 ops (one MAC) per step time, which "
                 "also holds the 15 table launches (a few us each), against the %s dense bf16 burst peak; frac against "
                 "the sustained peak %.3f. traffic: DRAM bytes per launch scaled by work from the committed ncu "
                 "capture of the same kernel on a smaller case of this shape (%s)"
                 % (src, tflops / peak_tf_sus, prof.get("file", "absent"))),
        "fp64_pipe": {"ops_per_launch": elems * fp64_per_elem,
                      "achieved_ops_per_s": elems * fp64_per_elem / (ms / 1000.0),
                      "peak_adds_per_s": fp64_rate,
                      "frac": elems * fp64_per_elem / (ms / 1000.0) / fp64_rate,
                      "note": "the fold's FP64 operations (%d per computed element) against the add rate measured "
                              "live on this GPU" % fp64_per_elem},
        "vs_int_pipe_roofline": {"achieved_bitops": work / (ms / 1000.0), "int_pipe_peak_bitops": popc_peak,
                                 "ratio": (work / (ms / 1000.0)) / popc_peak,
                                 "note": "against the integer-pipe roofline of any popcount Gram (POPC 16 lanes/clk"
                                         "/SM x 32 bits at the sampled SM clock)"},
    }
    out = {"value": value, "ms": ms, "launches": int(launches), "clocks": clocks, "roofline": roof, "e2e": e2e,
           "device_status": device_status, "setup_seconds": setup_s,
           "step_ms": {"min": min(step_ms), "median": statistics.median(step_ms), "max": max(step_ms)},
           "grouped_pass": {"ms_per_step": statistics.mean(pl), "value": world * work / (statistics.mean(pl) / 1e3),
                            "step_ms": {"min": min(pl), "median": statistics.median(pl), "max": max(pl)},
                            "note": "the same 15 products as one grouped persistent launch (lakgb_gram_group_run) "
                                    "after one table launch; identical outputs"},
           "popcount_pass": popc, "checks": checks}
    g.close()
    del g, lp, host
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return out


def case_control_pass_measurement(args, lib, stream, sh, world, with_cpu: bool):
    """The Gram pass of the case/control configuration (cases 4096 +
    controls 4096 x 16384 SNPs, 2 bins, seven products): one grouped launch
    (L2 flushed before each step: its inputs fit in L2), one launch per
    product, a CUDA-graph replay, the pass from host buffers, and the C
    port / reference on the host cores on the same pass."""
    import torch
    from lakcluster_c_gb300 import synth
    from lakcluster_c_gb300.gram_pass import GramPassDevice, GramPassHost, gram_pass_host

    inst = synth.case_control(seed=2)
    gp = GramPassHost(inst)
    dev = GramPassDevice(gp)
    work = gp.work_bitops()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step(fn):
        def f():
            flush.zero_()
            fn()
        return f

    for _ in range(3):
        dev.run(sh)
    torch.cuda.synchronize()
    per_ms = statistics.mean(_timed_steps(stream, step(lambda: dev.run(sh)), args.steps))
    graph = None
    try:
        gr = torch.cuda.CUDAGraph()
        with torch.cuda.graph(gr, stream=stream):
            dev.run(sh)
        torch.cuda.synchronize()
        gms = statistics.mean(_timed_steps(stream, step(gr.replay), args.steps))
        graph = {"ms_per_step": gms, "value": work / (gms / 1e3)}
        del gr
    except Exception as e:  # capture unsupported here: report why
        graph = {"unavailable": str(e)[:200]}
    ref = {k: v.view(torch.int64).clone() for k, v in dev.out.items()}
    for v in dev.out.values():
        v.fill_(float("nan"))
    for _ in range(3):
        dev.run_grouped(sh)
    torch.cuda.synchronize()
    same = all(torch.equal(dev.out[k].view(torch.int64), ref[k]) for k in ref)
    del ref
    gms = statistics.mean(_timed_steps(stream, step(lambda: dev.run_grouped(sh)), args.steps))
    dev.close()
    lib.lakgb_set_residency(0)
    outputs = {}
    gram_pass_host(gp, outputs)
    e2e_t = []
    d2h = 0
    for _ in range(5):
        t0 = time.perf_counter()
        d2h = gram_pass_host(gp, outputs)
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e_t)
    h2d = 0
    for kind, nb1, nb2, sym in _products(inst.nbins):
        MA = gp.MA[nb1]
        MZ = gp.MZ[nb2] if kind == "AnZt" else gp.MA[nb2]
        if MZ is not None:
            h2d += MA.wX.nbytes + (0 if sym else MZ.wX.nbytes) + MA.mc_length
    peaks, src = _peaks()
    peak_tf = float(peaks.get("bf16_tflops", 1900.0))
    out = {"workload": "case_control_4096x4096x16384_2bins_gram_pass", "products": len(dev.args),
           "bitops_per_pass": work, "value": work / (gms / 1e3), "ms_per_step": gms,
           "grouped_identical_to_per_launch": same,
           "tflops_frac_of_bf16_peak": 2.0 * work / (gms / 1e3) / 1e12 / peak_tf,
           "per_launch_pass": {"ms_per_step": per_ms, "value": work / (per_ms / 1e3)},
           "cuda_graph": graph,
           "e2e": {"value": work / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                   "d2h_bytes_per_step": int(d2h), "seconds_per_step": e2e_s},
           "l2": "flushed before each step (256 MB write)"}
    if with_cpu:
        backend, kind = _cpu_backend()
        threads = os.cpu_count() or 1
        cpu_gram_pass(inst, backend, threads)
        secs, w = 0.0, 0.0
        for _ in range(3):
            s1, w1 = cpu_gram_pass(inst, backend, threads)
            secs += s1
            w += w1
        out["cpu"] = {"value": w / secs, "unit": UNIT, "cores": threads, "kind": kind,
                      "sample": "the full pass, 3 passes, %.1f s" % secs}
    del flush
    torch.cuda.empty_cache()
    return out


def run_gpu(args):
    import torch
    import torch.distributed as dist

    rank, world, local = _rank_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from lakcluster_c_gb300 import build
    if rank == 0 or world == 1:
        build.build_lib()
    if world > 1:
        dist.barrier()
    from lakcluster_c_gb300._lib import load

    lib = load()
    # A dedicated stream: its handle is non-zero, so the library launches on it
    # (a zero handle would select the library's own stream) and the CUDA
    # events bracket exactly the launched kernels.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    head = large_pass_headline(args, lib, stream, sh, rank, world, local)

    # CPU baseline on a bounded sample (rank 0, N=1)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        backend, kind = _cpu_backend()
        threads = os.cpu_count() or 1
        smp = CpuLargeSample(backend, threads, LARGE_CPU_ROWS)
        smp.step()
        secs = sum(smp.step() for _ in range(3))
        cpu = {"value": 3 * smp.work / secs, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": CPU_SAMPLE + "; 3 products, %.1f s" % secs}
        del smp

    extras = {}
    if rank == 0:
        if not args.no_c2:
            extras["case_control_gram_pass"] = case_control_pass_measurement(
                args, lib, stream, sh, world, with_cpu=(world == 1 and not args.no_cpu_baseline))
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        if not args.no_grouped:
            extras["grouped_null_gram_passes"] = grouped_gram_measurement(stream, sh, flush)
        if not args.no_transpose:
            extras["b16_transpose"] = transpose_measurement(stream, sh, with_cpu=not args.no_cpu_baseline)
            extras["bed_to_b16"] = bed_measurement(with_cpu=not args.no_cpu_baseline)
        if not args.no_ww:
            extras["an_ztswn_yt_ww"] = ztswn_ww_measurement(with_cpu=not args.no_cpu_baseline)
        del flush
        if not args.no_solves:
            solves = solve_measurements(args, with_cpu=(world == 1 and not args.no_cpu_baseline))
            if not args.no_many:
                solves.update(many_solves_measurements(args))
            extras["solves"] = solves
        extras["gram_autotune"] = autotune_summary(lib)

    if rank == 0:
        line = {
            "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "e4m3-bit-mma+f64", "data": "synthetic",
            "config": dict(CONFIG, parallelism="replicas" if world > 1 else "single"),
            "pass_form": "one persistent tcgen05 launch per product (lakgb_gram_device, 15 per step, each after "
                         "its table launch); grouped_pass has the pass as one grouped launch",
            "gpu_launches": head["launches"],
            "roofline": head["roofline"],
            "e2e": head["e2e"],
            "clocks": head["clocks"],
            "device_status": head["device_status"],
            "step_ms": head["step_ms"],
            "grouped_pass": head["grouped_pass"],
            "popcount_pass": head["popcount_pass"],
            "parity_checks": head["checks"],
            "setup_seconds": head["setup_seconds"],
        }
        if cpu is not None:
            line["cpu_baseline"] = cpu
        line.update(extras)
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


def bed_measurement(with_cpu: bool):
    """PLINK .bed to .b16 (bed_to_b16, dir_c/bed_to_b16.c:711-1355) through
    lakgb_bed_to_b16_mem: 200000 SNPs x 16384 patients (819 MB of .bed
    records in page-locked host memory; MAF U[0.05,0.5], Hardy-Weinberg
    genotypes, 0.4 % missing calls, drawn on the GPU), both passes over the
    records (upload, code counts, allele expansion), the host statistics and
    sort, and the allele matrix's download inside the call.  The numpy
    restatement of the conversion (tests/bed_cases.py) is timed on the first
    2000 SNPs."""
    import torch
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from lakcluster_c_gb300._lib import load

    class Prm(C.Structure):
        _fields_ = [("a", C.c_double), ("b", C.c_double), ("c", C.c_double), ("d", C.c_double)]

    class Res(C.Structure):
        _fields_ = [("n_snp", C.c_int), ("n_fam", C.c_int), ("n_snp_retain", C.c_int), ("n_pat_retain", C.c_int),
                    ("n_allele", C.c_int), ("row_bytes", C.c_longlong)] + [(n, C.c_void_p) for n in (
                        "snp", "pat", "order", "freq", "maf", "mss", "I", "A_n")]

    lib = load()
    lib.lakgb_bed_to_b16_mem.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(Prm), C.POINTER(Res)]
    lib.lakgb_bed_result_free.argtypes = [C.POINTER(Res)]
    n_snp, n_fam = 200000, 16384
    n_bam = n_fam // 4
    thr = (0.01, 0.05, 0.01, 0.04)
    host = torch.empty((n_snp, n_bam), dtype=torch.uint8, pin_memory=True)
    g = torch.Generator(device="cuda")
    g.manual_seed(31)
    w = torch.tensor([1, 4, 16, 64], dtype=torch.int32, device="cuda")
    for r0 in range(0, n_snp, 20000):
        n = min(20000, n_snp - r0)
        q = 0.05 + 0.45 * torch.rand((n, 1), generator=g, device="cuda")
        u = torch.rand((n, n_fam), generator=g, device="cuda")
        c = torch.where(u < q * q, 0, torch.where(u < q * q + 2 * q * (1 - q), 2, 3))
        c = torch.where(torch.rand((n, n_fam), generator=g, device="cuda") < 0.004, 1, c)
        host[r0:r0 + n] = (c.view(n, n_bam, 4).to(torch.int32) * w).sum(2).to(torch.uint8).cpu()
        del q, u, c
    torch.cuda.synchronize()
    prm = Prm(*thr)
    t = []
    res = Res()
    for rep in range(4):
        t0 = time.perf_counter()
        rc = lib.lakgb_bed_to_b16_mem(host.data_ptr(), n_snp, n_fam, C.byref(prm), C.byref(res))
        dt = time.perf_counter() - t0
        assert rc == 0
        if rep:
            t.append(dt)
        kept = (res.n_snp_retain, res.n_pat_retain, res.n_allele, res.row_bytes)
        lib.lakgb_bed_result_free(C.byref(res))
    s = statistics.median(t)
    out = {"snps": n_snp, "patients": n_fam, "bed_bytes": n_snp * n_bam, "seconds": s, "seconds_all": t,
           "bed_gbs": n_snp * n_bam / s / 1e9, "genotypes_per_s": n_snp * n_fam / s,
           "kept_snps": kept[0], "kept_patients": kept[1], "alleles": kept[2],
           "allele_matrix_bytes": kept[2] * kept[3],
           "note": "whole conversion from page-locked host records: two uploads of the records, both GPU passes, "
                   "host statistics and allele sort, the allele matrix's download"}
    if with_cpu:
        import bed_cases as bd
        rec = host[:2000].numpy()
        t0 = time.perf_counter()
        bd.oracle(rec, n_fam, thr)
        cs = time.perf_counter() - t0
        out["cpu_baseline"] = {"genotypes_per_s": 2000 * n_fam / cs, "seconds": cs, "cores": 1, "kind": "port",
                               "sample": "the numpy restatement on the first 2000 SNPs"}
    del host
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
    if "case_control_4096x4096x16384" in golden:  # the reference program's outputs
        g = golden["case_control_4096x4096x16384"]
        c2["matches_reference"] = all(r2[k] == g[k] for k in ("trace", "xdrop_a", "xdrop_b"))
    out["case_control_4096x4096x16384"] = c2
    if with_cpu:
        out["case_only_1024x1024"]["cpu"] = cpu_solve_c1()
    return out


def many_solves_measurements(args):
    """Batched label-shuffled nulls and a served Poisson stream, each against
    the plain one-solve-at-a-time path on the same problems (results must be
    identical).

    Batched nulls: 256 instances with rows logU[1024, 8192] (split case /
    control by a label permutation) and SNPs logU[4096, 32768], drawn on the
    GPU; all submitted at once.  The plain path is timed on every 8th instance
    (32 solves, the same size distribution) and its throughput compared with
    the batched one; those 32 results must equal their batched results.

    Served stream: 24 requests with rows logU[512, 16384] and SNPs
    logU[2048, 65536], 0-3 covariate categories, MAF U[0.05, 0.5]; the plain
    path solves them one at a time; the server takes Poisson arrivals at 2x
    and 4x the plain throughput and all 24 at once (saturation), reporting
    solves/s and p50 / p99 latency at each rate."""
    from lakcluster_c_gb300 import serve, solve as sv, synth
    workers = max(2, min(16, os.cpu_count() or 2))
    out = {}
    n_null, stride = 256, 8
    probs = []
    for i in range(n_null):
        inst = synth.null_instance_packed(1000 + i)
        probs.append(sv.Problem(inst.A_bins, inst.Z_bins, gamma=0.05, packed_ncols=inst.ncols))
    sample = probs[::stride]
    plain, t_plain = serve.solve_plain(sample)
    batched, t_batch, peak = serve.solve_batched(probs, workers=workers)
    plain_rate, batch_rate = len(sample) / t_plain, n_null / t_batch
    out["batched_nulls"] = {
        "instances": n_null, "rows": "logU[1024,8192]", "cols": "logU[4096,32768]", "workers": workers,
        "plain_sample": "every %dth instance (%d solves)" % (stride, len(sample)),
        "plain_solves_per_s": plain_rate, "batched_solves_per_s": batch_rate,
        "speedup": batch_rate / plain_rate, "peak_concurrency": peak,
        "identical_to_plain": batched[::stride] == plain}
    n_req = 24
    reqs = []
    for i in range(n_req):
        inst = synth.served_request_packed(5000 + i)
        reqs.append(sv.Problem(inst.A_bins, inst.Z_bins, gamma=0.05, packed_ncols=inst.ncols))
    solo, t_solo = serve.solve_plain(reqs)
    plain_rate = n_req / t_solo
    served = {"requests": n_req, "rows": "logU[512,16384]", "cols": "logU[2048,65536]", "categories": "U{0..3}",
              "workers": workers, "plain_solves_per_s": plain_rate, "rates": []}
    same = True
    for mult in (2.0, 4.0, float("inf")):
        rate = mult * plain_rate
        r, lat, wall, peak = serve.serve_stream(reqs, rate, workers=workers, seed=7)
        same = same and r == solo
        served["rates"].append(dict(serve.latency_stats(lat), arrival_rate_per_s=(rate if mult != float("inf") else
                                                                                  "all at once"),
                                    solves_per_s=n_req / wall, speedup=(n_req / wall) / plain_rate,
                                    peak_concurrency=peak))
    served["identical_to_solo"] = same
    out["served"] = served
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
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-solves", action="store_true", help="skip the whole-solve timings")
    ap.add_argument("--no-many", action="store_true", help="skip the batched / served timings")
    ap.add_argument("--no-transpose", action="store_true", help="skip the .b16 transposer measurement")
    ap.add_argument("--no-ww", action="store_true", help="skip the An_ZtSWn_Yt_ww bit-plane product measurement")
    ap.add_argument("--no-grouped", action="store_true",
                    help="skip the grouped Gram passes of the batched-null instances")
    ap.add_argument("--no-c2", action="store_true",
                    help="skip the case/control configuration's Gram pass (4096 + 4096 x 16384)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
