#!/usr/bin/env python3
"""Benchmark: Mie instance-evaluations per second of a whole optics table.

One step = one full sulfate-like table on the GPU: 36 RH x 60 wavelengths x
5 lognormal bins on one shared grid of 2000 wet radii (4.32e6 Mie instances),
181 scattering angles, size/RH integration and 64 GSF moments -- the
(bin x wavelength x RH) sweep of dointegration.fun followed by the pygeos
pass of rungsf.  Inputs are synthetic and seeded (geosmie_gb300/workloads.py).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  --impl reference times the CPU restatement of the
reference's own per-size algorithm (oracle/, scipy Bessel functions, per-angle
sums) on the host cores over a fixed stratified sample of the same table.
Multi-GPU: replicas (each rank builds the whole table; the path needs no
exchange), value = all ranks' instances / max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "Mie instance-evals/s + table gen time, mixed vs FP64 plain on 1 GB300 at ≤1e-6 rel"
UNIT = "instance-evals/s"
# CPU sample: wavelength and RH indices of the stratified sample of units
SAMPLE_LAMBDA = [0, 12, 24, 36, 48, 59]
# DRAM bytes (read + write) per (wavelength, RH, component) unit from one ncu
# capture of the 12-wavelength sulfate table (432 units; profiles/
# k_tab_s12_tc_k_tab_coeffs_mixed_sulfate12.md: dram__bytes.sum.per_second x
# duration), scaled to a run by its units
NCU_BYTES_PER_UNIT = {"k_tab_coeffs_mixed": 904.567513e9 * 527.776e-6 / 432,
                      "k_tab_s12_tc": 789.561399e9 * 693.696e-6 / 432}
SAMPLE_RH = [0, 35]


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, ws, device=None):
    """The largest of the ranks' x (all_reduce with MAX over the default
    process group, on `device`: a CUDA device under NCCL, the CPU under gloo);
    x itself on one rank."""
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank, ws, steps, seconds):
    """Whole-job throughput of ws replicas: every rank processed
    units_per_rank x steps units; seconds is the max-over-ranks time."""
    return ws * units_per_rank * steps / seconds


def _oracle_unit(args):
    """One (wavelength, RH) unit of the table on the CPU with the oracle:
    per-size coefficients, per-angle S1/S2 sums (pymiecoated's algorithm),
    Mueller elements, integration of all bins, normalisation, GSF."""
    spec, li, ri, n_gsf = args
    from oracle import gsf as ogsf
    from oracle import integration as oi
    lam = float(spec["lambda"][li])
    x = 2 * np.pi * np.asarray(spec["grid"]) / lam
    m = complex(spec["m"][li, ri, 0])
    ang = np.asarray(spec["ang"])
    raw = oi.raw_mie(x, np.cos(np.radians(ang)), lam, m.real, m.imag, batch=False)
    gf = float(spec["gf_psd"][ri])
    out = []
    for b in range(np.asarray(spec["frac"]).shape[0]):
        pp = spec["psd_param"][b][0]
        w = oi.lognorm_psd(pp[0] * gf, pp[3], x, lam, pp[2] * gf, pp[1]) * spec["dgrid"]
        w = w / w.sum()
        w0 = oi.lognorm_psd(pp[0], pp[3], x, lam, pp[2], pp[1]) * spec["dgrid"]
        rr = x * lam / (2 * np.pi)
        reff0 = np.sum(rr ** 4 * w0) / np.sum(rr ** 3 * w0)
        ret = oi.integrate_psd(x, [raw], [w], [1.0], lam, [reff0], float(spec["rhop0"][b]),
                               float(spec["rhop"][b, ri]))
        fin = oi.finalize_unit(ret, ang, gf, float(spec["rhop"][b, ri]), [m.real], [m.imag], 0.0, 0.0)
        out.append(np.stack([fin[k] for k in ["p11", "p22", "p33", "p44", "p12", "p34"]]))
    ogsf.expand(ang, np.array(out), n_gsf)
    return x.size


def cpu_sample(spec, n_gsf, processes=1):
    units = [(spec, li, ri, n_gsf) for li in SAMPLE_LAMBDA for ri in SAMPLE_RH]
    t0 = time.perf_counter()
    if processes > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(processes) as pool:
            n = sum(pool.map(_oracle_unit, units))
    else:
        n = sum(_oracle_unit(u) for u in units)
    return n, time.perf_counter() - t0, len(units)


def run_reference(args):
    """--impl reference: the CPU path timed on the host cores (rank 0 only)."""
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from geosmie_gb300 import workloads
    from oracle import gsf as ogsf
    ogsf.build()
    spec, desc = workloads.sulfate_table()
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(spec, 64, processes=cores)
    times = []
    n = 0
    for _ in range(args.steps):
        n, dt, nu = cpu_sample(spec, 64, processes=cores)
        times.append(dt)
    tot = sum(times)
    value = n * args.steps / tot
    sample = ("%d of 2160 (wavelength, RH) units of the table (wavelength indices %s x RH indices %s), "
              "2000 radii each, all 5 bins, 181 angles, 64 GSF moments" % (len(SAMPLE_LAMBDA) * len(SAMPLE_RH),
                                                                          SAMPLE_LAMBDA, SAMPLE_RH))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                         "note": "CPU restatement of pymiecoated + dointegration (scipy jv/yv, per-angle "
                                 "sums; the reference's numba is not installed) and of spher_expan.f in C, "
                                 "multiprocessing pool over units"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "projected_table_s": 4.32e6 / value,
    }
    print(json.dumps(line))
    return 0


def algorithmic_flop(counts):
    """Algorithmic flop per launch of the table kernels, from the per-instance
    work of the reference's algorithm: coefficients 14 nmx + 50 nmax (FP64
    flop); angular sums 16 nmax N_ang (four complex-by-real multiply-adds per
    order and angle); the Mueller elements, 12 flop per (instance, angle),
    and their size integration, a multiply-add for each of the 6 elements
    per (instance, bin, angle).  Split products, padding and the S+/S- form
    are the implementation's, not the algorithm's, and are not counted."""
    nang, nbin, inst = counts["nang"], counts["nbin"], counts["instances"]
    coef = 14.0 * counts["sum_nmx"] + 50.0 * counts["sum_nmax"]
    sums = 16.0 * counts["sum_nmax"] * nang
    mueller = (12.0 + 12.0 * nbin) * nang * inst
    return {"k_tab_coeffs": coef, "k_tab_coeffs_mixed": coef, "k_tab_s12_plain": sums + mueller,
            "k_tab_s12_tc": sums, "k_tab_s12_tc_epilogue": mueller}


def executed_flop(counts):
    """Flop the kernels execute per launch (pipe utilisation).  FP64 pipe:
    the plain sums in the S+/S- form (8 per order and angle; the S+ and S-
    sums halve the reference's multiply-adds), the Mueller elements (14) and
    the number-weighted accumulation (8 per bin) per (instance, angle); the
    plain coefficients 12 per D_n step and 89 per order.  The mixed
    coefficient kernel's double-float work counted as the FP64 flop of the
    same steps: 15 per warm-up D_n step, 32 per order.  Tensor cores: 6 MMAs
    (M 128 angles x N 64 (32 sizes, Re/Im) x K 16) per 16-order chunk of a
    half tile of 32 sizes, per 128-angle block (3 split products x 2 GEMMs,
    padded)."""
    nang, nbin, inst = counts["nang"], counts["nbin"], counts["instances"]
    return {"k_tab_s12_plain": (8.0 * counts["sum_nmax"] + (14.0 + 8.0 * nbin) * inst) * nang,
            "k_tab_coeffs": 12.0 * counts["sum_nmx"] + 89.0 * counts["sum_nmax"],
            "k_tab_coeffs_mixed": 15.0 * counts["sum_warm"] + 32.0 * counts["sum_nmax"],
            "k_tab_s12_tc": counts["sum_kc16_half"] * 6 * 2 * 128 * 64 * 16 * (-(-nang // 128))}


ON_FP64_PIPE = ("k_tab_s12_plain", "k_tab_coeffs")


def roofline_of(ktimes, counts, peaks, fp64_peak):
    """Per-kernel rates and the roofline of the dominant kernel.

    ktimes: {kernel: (launches, total ms)} from CUDA events on the launching
    stream; peaks: MEASURED_PEAKS-style dict (bf16_tflops); fp64_peak:
    measured DFMA GFLOP/s.  achieved = algorithmic flop per launch / mean
    launch time; the executed flop (what the pipe ran) is reported beside
    it.  Returns (kernels, roof)."""
    alg = algorithmic_flop(counts)
    exe = executed_flop(counts)
    kernels = {}
    tot = max(1e-9, sum(v[1] for v in ktimes.values()))
    for name, (nl_, tms) in ktimes.items():
        sec = tms / max(nl_, 1) * 1e-3
        k = {"launches": nl_, "ms_per_launch": tms / max(nl_, 1), "share": tms / tot}
        if name in ON_FP64_PIPE:
            k["algorithmic_gflops"] = alg[name] / sec / 1e9
            k["fp64_gflops"] = exe[name] / sec / 1e9
            k["fp64_pipe_frac"] = exe[name] / sec / 1e9 / fp64_peak
        elif name == "k_tab_coeffs_mixed":
            k["algorithmic_gflops"] = alg[name] / sec / 1e9
            k["fp64_equivalent_gflops_as_fp32_pairs"] = exe[name] / sec / 1e9
        elif name == "k_tab_s12_tc":
            k["algorithmic_tflops"] = alg[name] / sec / 1e12
            k["executed_mma_tflops"] = exe[name] / sec / 1e12
            k["epilogue_algorithmic_tflops"] = alg["k_tab_s12_tc_epilogue"] / sec / 1e12
            k["tensor_peak_tflops"] = peaks.get("bf16_tflops")
        kernels[name] = k
    roof = None
    top = max(ktimes.items(), key=lambda kv: kv[1][1])[0] if ktimes else None
    if top in ON_FP64_PIPE:
        nl_, tms = ktimes[top]
        sec = tms / max(nl_, 1) * 1e-3
        ach = alg[top] / sec / 1e9
        tb = NCU_BYTES_PER_UNIT.get(top)
        roof = {"bound": "fp64", "kernel": top, "achieved": ach, "peak": fp64_peak, "unit": "GFLOP/s",
                "frac": ach / fp64_peak, "traffic": tb * counts["units"] if tb else None,
                "traffic_unit": "bytes per launch (ncu capture scaled by units)",
                "peak_source": "DFMA throughput measured in this run (gbmie_measure_fp64_peak); "
                               "MEASURED_PEAKS.json has no FP64 figure",
                "algorithmic_flop_per_launch": alg[top], "executed_flop_per_launch": exe[top],
                "executed_frac": exe[top] / sec / 1e9 / fp64_peak}
    elif top == "k_tab_s12_tc":
        nl_, tms = ktimes[top]
        sec = tms / max(nl_, 1) * 1e-3
        peak = peaks.get("bf16_tflops")
        roof = {"bound": "tensor", "kernel": top, "achieved": alg[top] / sec / 1e12,
                "peak": peak, "unit": "TFLOP/s", "frac": alg[top] / sec / 1e12 / peak,
                "traffic": NCU_BYTES_PER_UNIT[top] * counts["units"],
                "traffic_unit": "bytes per launch (ncu capture scaled by units)",
                "peak_source": ("fallback bf16 burst figure (MEASURED_PEAKS.json absent), of fallback"
                                if peaks.get("fallback") else "MEASURED_PEAKS.json bf16_tflops (burst), of measured"),
                "algorithmic_flop_per_launch": alg[top], "executed_mma_flop_per_launch": exe[top],
                "executed_frac": exe[top] / sec / 1e12 / peak,
                "note": "achieved = the angular sums' algorithmic flop (16 per order and angle); the "
                        "tensor cores execute executed_mma_flop (3 split products x 2 GEMMs on padded "
                        "tiles). The tensor pipe is not this kernel's limit: the fused Mueller/PSD "
                        "epilogue is (latency-bound FP32 work of 8 warps)"}
    return kernels, roof


class Clocks(object):
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, index):
        self.index = index
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + ",".join(self.FIELDS),
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [v.strip() for v in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--small", action="store_true", help="reduced table (quick check, not a bench line)")
    ap.add_argument("--lambdas", type=int, default=60, help="wavelengths of the table (profiling subsets)")
    ap.add_argument("--rh", type=int, default=36, help="RH values of the table (profiling subsets)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = local
    from geosmie_gb300 import _native, workloads
    from geosmie_gb300.table import NL_ORDER, SCALAR_ORDER, SCATKEYS, TablePlan, run_tables
    ctx = _native.context(dev)
    if args.small:
        spec, desc = workloads.sulfate_table(n_rh=6, n_lambda=10, n_radii=500)
    else:
        spec, desc = workloads.sulfate_table(n_rh=args.rh, n_lambda=args.lambdas)
    counts = workloads.work_counts(spec)
    n_gsf = 64
    peak = _native._D()
    ctx.call("gbmie_measure_fp64_peak", _native.ctypes.byref(peak))
    fp64_peak = peak.value

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:%d" % dev)
    stream = torch.cuda.current_stream(dev)

    def timed(plan, graph=False, with_clocks=False):
        """Warm-up, then K tables between barriers + syncs, L2 flushed before
        each (256 MB write, inside the timed region).  Returns (ms, launches,
        kernel times, clocks)."""
        clocks = Clocks(dev)
        if with_clocks:
            clocks.start()   # sampling spans the last warm-up tables and the timed region
        for _ in range(args.warmup):
            plan.run(graph=graph)
        plan.sync()
        ctx.set_timing(True)
        launches0 = ctx.launches()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            flush.zero_()
            plan.run(graph=graph)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        clk = clocks.stop() if with_clocks else None
        launches = ctx.launches() - launches0
        kt = ctx.kernel_times()
        ctx.set_timing(False)
        plan.sync()   # device error flags -> status
        if ws > 1:
            ms = max_over_ranks(ms, ws, device="cuda:%d" % dev)
            torch.distributed.barrier()
        return ms, launches, kt, clk

    # launch parameters tuned on the table itself before timing (plan set-up;
    # later plans of the same shape, e.g. the end-to-end ones, reuse them)
    plan_plain = TablePlan(spec, precision=_native.GBMIE_PLAIN_FP64, n_gsf=n_gsf, device=dev)
    tune_plain = plan_plain.autotune()
    ms_plain, _, kt_plain, _ = timed(plan_plain)
    ra = plan_plain.results()
    plan_plain.close()
    del plan_plain
    plan_mixed = TablePlan(spec, precision=_native.GBMIE_MIXED, n_gsf=n_gsf, device=dev)
    tune_mixed = plan_mixed.autotune()
    # eager launches with per-kernel CUDA events: kernel shares and the roofline
    ms_eager, _, ktimes, _ = timed(plan_mixed)
    # the product path: the whole table replayed as one CUDA graph
    ms, launches, _, clk = timed(plan_mixed, graph=True, with_clocks=True)
    ms_step = ms / args.steps
    value = replica_value(counts["instances"], ws, args.steps, ms * 1e-3)
    # accuracy of the mixed table against the FP64 table (same run), every output
    rb = plan_mixed.results()
    p11 = np.abs(ra["p11"])
    acc = {"phase_max_abs_err_over_p11": {k: float(np.max(np.abs(rb[k] - ra[k]) / p11)) for k in SCATKEYS},
           "pback_max_abs_err_over_p11back": float(np.max(np.abs(rb["pback"] - ra["pback"]) /
                                                          np.abs(ra["pback"][..., :1]))),
           "pmom_max_abs_err_over_max_alpha1": {
               nm: float(np.max(np.abs(rb["pmom"][..., j, :] - ra["pmom"][..., j, :]) /
                                np.max(np.abs(ra["pmom"][..., 0, :]), axis=-1)[..., None]))
               for j, nm in enumerate(["alpha1", "beta1", "alpha3", "beta2", "alpha2", "alpha4"])},
           "scalars_max_rel_err": {k: float(np.max(np.abs(rb[k] - ra[k]) / np.maximum(np.abs(ra[k]), 1e-300)))
                                   for k in SCALAR_ORDER},
           "wavelength_independent_max_rel_err": {
               k: float(np.max(np.abs(rb["nl_" + k] - ra["nl_" + k]) / np.maximum(np.abs(ra["nl_" + k]), 1e-300)))
               for k in NL_ORDER}}
    acc["qabs_max_abs_err_over_qext"] = float(np.max(np.abs(rb["qabs"] - ra["qabs"]) / np.abs(ra["qext"])))
    plan_mixed.close()
    del plan_mixed

    # ---- end to end through the public API: host inputs in, host table out ----
    # K tables through run_tables: each table's plan from host arrays (input
    # copy, device layout), its run and its results read back to the host;
    # plan creation and the copy back overlap the neighbouring tables' runs
    probe = TablePlan(spec, precision=_native.GBMIE_MIXED, n_gsf=n_gsf, device=dev)
    h2d = sum(v.numel() * v.element_size() for v in probe.t.values())
    d2h = sum(v.numel() * v.element_size() for v in probe.out_t.values())
    probe.close()
    for _ in run_tables([spec] * 2, precision=_native.GBMIE_MIXED, n_gsf=n_gsf, device=dev):
        pass   # warm-up of the streams and the allocation pool
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    n_done = 0
    for res in run_tables([spec] * args.steps, precision=_native.GBMIE_MIXED, n_gsf=n_gsf, device=dev):
        n_done += 1
    torch.cuda.synchronize(dev)
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws, device="cuda:%d" % dev)
    e2e_value = replica_value(counts["instances"], ws, n_done, e2e_s)

    # ---- roofline of the dominant kernel ----
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        peaks = {"bf16_tflops": 1900.0, "hbm_gbs": 6800.0, "fallback": True}
    kernels, roof = roofline_of(ktimes, counts, peaks, fp64_peak)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline and not args.small:
        n, dt, nu = cpu_sample(spec, n_gsf, processes=1)
        cpu = {"value": n / dt, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "%d (wavelength, RH) units x 2000 radii, all bins, 181 angles, 64 GSF moments; "
                         "CPU restatement of the reference algorithm (numba absent)" % nu,
               "seconds": dt}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-pair (double-float) recurrences + f16x2-split tensor contractions (f32 accumulate)", "data": "synthetic (seeded; no dataset)",
        "config": {"workload": desc, "instances": counts["instances"], "sum_nmax": counts["sum_nmax"],
                   "gsf_moments": n_gsf, "precision": "mixed: double-float (FP32-pair) D_n and N/M recurrences on FP64-built "
                   "psi/chi rows, tcgen05 split-FP16 contractions with FP32 accumulation", "parallelism": "replicas" if ws > 1 else "1 GPU",
                   "l2": "flushed before every table (256 MB write inside the timed region)",
                   "launch": "whole table replayed as one CUDA graph (gbmie_table_run_graph)"},
        "table_gen_ms": {"mixed": ms_step, "mixed_eager_launches": ms_eager / args.steps,
                         "plain_fp64": ms_plain / args.steps},
        "mixed_vs_plain_speedup": ms_plain / ms,
        "plain_fp64": {"value": replica_value(counts["instances"], ws, args.steps, ms_plain * 1e-3), "unit": UNIT,
                       "kernels": roofline_of(kt_plain, counts, peaks, fp64_peak)[0]},
        "accuracy_mixed_vs_fp64": acc,
        "roofline": roof,
        "kernels": kernels,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "note": "K tables through geosmie_gb300.table.run_tables: per table a plan from host arrays "
                        "(one page-locked input copy, device layout), its run and its results copied to "
                        "page-locked host memory; plan creation and the copy back overlap the neighbouring "
                        "tables' runs (setup and copy streams)",
                "ms_per_table": e2e_s * 1e3 / max(n_done, 1)},
        "gpu_launches": launches,
        "autotuned": {"mixed": tune_mixed, "plain_fp64": tune_plain},
        "clocks": clk,
        "fp64_peak_gflops": fp64_peak,
    }
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
