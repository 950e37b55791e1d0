#!/usr/bin/env python3
"""Benchmark: Mie instance-evaluations per second of whole optics tables.

One step = one whole table of the headline workload (default: the
sulfate-like table, 36 RH x 60 wavelengths x 5 lognormal bins on one shared
grid of 2000 wet radii = 4.32e6 Mie instances, 181 scattering angles, size/RH
integration and 64 GSF moments -- the (bin x wavelength x RH) sweep of
dointegration.fun followed by the pygeos pass of rungsf).  Inputs are
synthetic and seeded (geosmie_gb300/workloads.py).  The default run also
measures the other four benchmark workloads (homogeneous single wavelength,
dust-like bins, coated black carbon, sea-salt-like large sizes on 4000 Gauss
nodes with 1000 GSF moments) with fewer steps and reports them under
"configs".

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config 1..5] [--no-others] [--no-cpu-baseline]

Prints one JSON line; the figures a reader checks first (table times, the
mixed-over-FP64 speed-up, the error blocks) are its last keys.  --impl
reference times the CPU restatement of the reference's own per-size
algorithm (oracle/, scipy Bessel functions, per-angle sums, spher_expan in C)
on all host cores over a fixed stratified sample of the same table.
Multi-GPU: replicas (each rank builds the whole table; the path needs no
exchange), value = all ranks' instances / max-over-ranks time.
"""
import argparse
import functools
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
# CPU sample of the sulfate table: wavelength and RH indices of the
# stratified units (accuracy against the oracle and the 1-core baseline)
SAMPLE_LAMBDA = [0, 12, 24, 36, 48, 59]
SAMPLE_RH = [0, 35]
# reference arm: 8 wavelengths x 6 RH = 48 stratified units; each step takes
# one unit per host core, rotating through the list
REF_LAMBDA = [0, 8, 17, 25, 34, 42, 51, 59]
REF_RH = [0, 7, 14, 21, 28, 35]
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per (wavelength,
# RH, component) unit from one ncu capture of each kernel on the 12-wavelength
# sulfate table (432 units; profiles/k_tab_s12_tc_sulfate12.md,
# profiles/k_tab_coeffs_mixed_sulfate12.md), scaled to a run by its units
# (sulfate table only)
NCU_BYTES_PER_UNIT = {"k_tab_coeffs_mixed": (34.952192e6 + 371.037952e6) / 432,
                      "k_tab_s12_tc": (323.177472e6 + 16.813312e6) / 432}
SCAT = ["p11", "p12", "p22", "p33", "p34", "p44"]
SCALARS = ["qext", "qsca", "qb", "g", "csca", "cext", "ssa", "bsca", "bext", "bbck", "refreal", "refimag",
           "lidar_ratio"]
NLKEYS = ["mass", "volume", "area", "rEff", "rMass", "rhop", "growth_factor"]


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


def sig(x, n=4):
    """x rounded to n significant digits (floats inside dicts and lists too)."""
    if isinstance(x, dict):
        return {k: sig(v, n) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [sig(v, n) for v in x]
    if isinstance(x, (float, np.floating)):
        return float("%.*g" % (n, x))
    return x


# ---------------------------------------------------------------------------
# workloads (the five benchmark configurations)
# ---------------------------------------------------------------------------
@functools.lru_cache(maxsize=None)
def build_config(cfg):
    """(specs, description, n_gsf, n_gsf_nodes, oracle sample units
    [(spec index, wavelength index, RH index)]) of benchmark workload cfg."""
    from geosmie_gb300 import workloads
    if cfg == 1:
        spec, d = workloads.homogeneous_single()
        return [spec], d, 0, 0, [(0, 0, 0)]
    if cfg == 2:
        specs, d = workloads.dust_bins()
        return specs, d, 0, 0, [(b, li, 0) for b in range(5) for li in (0, 39)]
    if cfg == 3:
        spec, d = workloads.sulfate_table()
        return [spec], d + " + 64 GSF moments", 64, 0, [(0, li, ri) for li in SAMPLE_LAMBDA for ri in SAMPLE_RH]
    if cfg == 4:
        spec, d = workloads.coated_bc()
        return [spec], d, 0, 0, [(0, 0, 0), (0, 15, 105), (0, 29, 199)]
    if cfg == 5:
        spec, d, nm, nn = workloads.seasalt_large()
        return [spec], d, nm, nn, [(0, 10, 0), (0, 19, 0)]
    raise ValueError("configuration %r (1..5)" % cfg)


def config_counts(cfg):
    """Work counts summed over the workload's tables, and per launch (each
    table launches each kernel once)."""
    from geosmie_gb300 import workloads
    specs = build_config(cfg)[0]
    cs = [workloads.work_counts(s) for s in specs]
    tot = {k: (sum(c[k] for c in cs) if k not in ("nang", "nbin", "coated") else cs[0][k]) for k in cs[0]}
    per = {k: (v / len(specs) if k not in ("nang", "nbin", "coated") else v) for k, v in tot.items()}
    return tot, per


def _unit_task(args):
    """One (wavelength, RH) unit of a workload on one CPU core with the
    oracle: per-size coefficients, per-angle S1/S2 sums (pymiecoated's
    algorithm; homogeneous spheres size by size as MultipleMie does, or
    vectorised over sizes with batch), Mueller elements, integration of every
    bin, normalisation, GSF.  Returns (key, results of the unit, seconds,
    instances)."""
    cfg, si, li, ri, batch = args
    from oracle import integration
    specs, _, n_gsf, nodes, _ = build_config(cfg)
    spec = specs[si]
    t0 = time.perf_counter()
    res = integration.run_spec(spec, n_gsf=n_gsf, n_gsf_nodes=nodes, units=[(li, ri)], batch=batch)
    dt = time.perf_counter() - t0
    sub = {k: v[:, li, ri] for k, v in res.items() if isinstance(v, np.ndarray) and v.ndim >= 3}
    ninst = np.asarray(spec["m"]).shape[2] * len(spec["grid"])
    return (cfg, si, li, ri), sub, dt, ninst


def unit_tasks(cfg):
    """The oracle tasks of workload cfg's sample units: the headline sulfate
    table size by size (the reference's own structure, timed as the 1-core
    baseline); the others vectorised over sizes (accuracy checks that finish
    in seconds)."""
    return [(cfg,) + u + (cfg != 3,) for u in build_config(cfg)[4]]


def _pool(processes):
    """A spawn pool of single-threaded numpy workers (spawn: safe after the
    process has used CUDA)."""
    import multiprocessing as mp
    for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[v] = "1"
    return mp.get_context("spawn").Pool(processes)


# ---------------------------------------------------------------------------
# accuracy summaries
# ---------------------------------------------------------------------------
def accuracy(got, ref, mixed=False, fwd=None):
    """Largest errors of every output family of table results `got` against
    `ref` (same shapes): phase elements relative to P11 at the same angle,
    pback relative to its P11, scalars relative, qabs relative to itself
    (mixed) or to qext (FP64, where qext - qsca cancels), GSF moments
    relative to the entry's largest alpha1, wavelength-independent values
    relative; fwd: a mask of forward angles reported separately."""
    p11 = np.abs(ref["p11"])
    a = {"phase_over_p11": max(float(np.max(np.abs(got[k] - ref[k]) / p11)) for k in SCAT),
         "pback": float(np.max(np.abs(got["pback"] - ref["pback"]) / np.abs(ref["pback"][..., :1]))),
         "scalars_rel": max(float(np.max(np.abs(got[k] - ref[k]) / np.maximum(np.abs(ref[k]), 1e-300)))
                            for k in SCALARS)}
    if mixed:
        a["qabs_rel"] = float(np.max(np.abs(got["qabs"] - ref["qabs"]) /
                                     (np.abs(ref["qabs"]) + 1e-12 * np.abs(ref["qext"]))))
    else:
        a["qabs_over_qext"] = float(np.max(np.abs(got["qabs"] - ref["qabs"]) / np.abs(ref["qext"])))
    if "pmom" in got and "pmom" in ref:
        scale = np.max(np.abs(ref["pmom"][..., 0, :]), axis=-1)[..., None, None]
        a["pmom_over_alpha1"] = float(np.max(np.abs(got["pmom"] - ref["pmom"]) / scale))
    nl = [k for k in NLKEYS if "nl_" + k in got and "nl_" + k in ref]
    if nl:
        a["nl_rel"] = max(float(np.max(np.abs(got["nl_" + k] - ref["nl_" + k]) / np.abs(ref["nl_" + k])))
                          for k in nl)
    if fwd is not None:
        a["fwd_p11_rel"] = float(np.max(np.abs(got["p11"][..., fwd] - ref["p11"][..., fwd]) /
                                        ref["p11"][..., fwd]))
    return a


def worst(blocks):
    """Element-wise maximum of accuracy dicts."""
    out = {}
    for b in blocks:
        for k, v in b.items():
            out[k] = max(out.get(k, 0.0), v)
    return out


def _units_of(results, si, units):
    """Results of table si at the sample units, shaped like the oracle's
    per-unit dicts ([bin, ...] per unit, stacked over units)."""
    li = np.array([u[1] for u in units])
    ri = np.array([u[2] for u in units])
    return {k: v[:, li, ri] for k, v in results[si].items() if isinstance(v, np.ndarray) and v.ndim >= 3}


def oracle_accuracy(units, plain, mixed, oracle):
    """FP64 and mixed tables against the oracle at the sample units."""
    blocks_p, blocks_m = [], []
    for si in sorted(set(u[0] for u in units)):
        us = [u for u in units if u[0] == si]
        ref = {}
        for k in oracle[us[0]]:
            ref[k] = np.stack([oracle[u][k] for u in us], axis=1)
        blocks_p.append(accuracy(_units_of(plain, si, us), ref))
        blocks_m.append(accuracy(_units_of(mixed, si, us), ref, mixed=True))
    return {"fp64": worst(blocks_p), "mixed": worst(blocks_m), "units": len(units)}


# ---------------------------------------------------------------------------
# roofline arithmetic
# ---------------------------------------------------------------------------
def algorithmic_flop(counts):
    """Algorithmic flop per launch of the table kernels, from the per-instance
    work of the reference's algorithm: homogeneous coefficients 14 nmx + 50
    nmax (FP64 flop: one D_n step per order up to nmx, a_n/b_n per order,
    mie_coeffs.py:83-130); coated coefficients 42 nmx + 170 nmax (D_n at the
    three arguments m1 x, m2 x, m2 y and the ratio chain uu..kv2, dns, gns,
    a_n, b_n per order, mie_coeffs.py:216-251); angular sums 16 nmax N_ang
    (four complex-by-real multiply-adds per order and angle); the Mueller
    elements, 12 flop per (instance, angle), and their size integration, a
    multiply-add for each of the 6 elements per (instance, bin, angle).
    Split products, padding and the S+/S- form are the implementation's, not
    the algorithm's, and are not counted."""
    nang, nbin, inst = counts["nang"], counts["nbin"], counts["instances"]
    coef = 14.0 * counts["sum_nmx"] + 50.0 * counts["sum_nmax"]
    coated = 42.0 * counts["sum_nmx"] + 170.0 * counts["sum_nmax"]
    sums = 16.0 * counts["sum_nmax"] * nang
    mueller = (12.0 + 12.0 * nbin) * nang * inst
    return {"k_tab_coeffs": coef, "k_tab_coeffs_mixed": coef, "k_tab_s12_plain": sums + mueller,
            "k_tab_s12_tc": sums, "k_tab_s12_tc_epilogue": mueller, "k_tab_coeffs_coated": coated,
            "k_tab_coeffs_mixed_coated": coated}


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
    padded); a whole-tile item runs both halves as N = 128, the same flop,
    except that a last tile of 32 sizes or fewer taken whole also runs its
    empty half (not counted)."""
    nang, nbin, inst = counts["nang"], counts["nbin"], counts["instances"]
    return {"k_tab_s12_plain": (8.0 * counts["sum_nmax"] + (14.0 + 8.0 * nbin) * inst) * nang,
            "k_tab_coeffs": 12.0 * counts["sum_nmx"] + 89.0 * counts["sum_nmax"],
            "k_tab_coeffs_mixed": 15.0 * counts["sum_warm"] + 32.0 * counts["sum_nmax"],
            "k_tab_s12_tc": counts["sum_kc16_half"] * 6 * 2 * 128 * 64 * 16 * (-(-nang // 128))}


ON_FP64_PIPE = ("k_tab_s12_plain", "k_tab_coeffs", "k_tab_coeffs_coated", "k_tab_coeffs_mixed_coated")


def roofline_of(ktimes, counts, peaks, fp64_peak, traffic_per_unit=None):
    """Per-kernel rates and the roofline of the dominant kernel.

    ktimes: {kernel: (launches, total ms)} from CUDA events on the launching
    stream; counts: work counts per launch; peaks: MEASURED_PEAKS-style dict
    (bf16_tflops); fp64_peak: measured DFMA GFLOP/s; traffic_per_unit: ncu
    DRAM bytes per (wavelength, RH, component) unit of the kernels (default:
    the sulfate table's capture).  achieved = algorithmic flop per launch /
    mean launch time; the executed flop (what the pipe ran) is reported
    beside it.  Returns (kernels, roof)."""
    traffic_per_unit = NCU_BYTES_PER_UNIT if traffic_per_unit is None else traffic_per_unit
    alg = algorithmic_flop(counts)
    exe = executed_flop(counts)
    kernels = {}
    tot = max(1e-9, sum(v[1] for v in ktimes.values()))
    for name, (nl_, tms) in ktimes.items():
        sec = tms / max(nl_, 1) * 1e-3
        k = {"launches": nl_, "ms_per_launch": tms / max(nl_, 1), "share": tms / tot}
        if name in ON_FP64_PIPE:
            k["algorithmic_gflops"] = alg[name] / sec / 1e9
            if name in exe:
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
        tb = traffic_per_unit.get(top)
        roof = {"bound": "fp64", "kernel": top, "achieved": ach, "peak": fp64_peak, "unit": "GFLOP/s",
                "frac": ach / fp64_peak, "traffic": tb * counts["units"] if tb else None,
                "traffic_unit": "bytes per launch (ncu capture scaled by units)",
                "peak_source": "DFMA throughput measured in this run (gbmie_measure_fp64_peak); "
                               "MEASURED_PEAKS.json has no FP64 figure",
                "algorithmic_flop_per_launch": alg[top]}
        if top in exe:
            roof["executed_flop_per_launch"] = exe[top]
            roof["executed_frac"] = exe[top] / sec / 1e9 / fp64_peak
    elif top == "k_tab_s12_tc":
        nl_, tms = ktimes[top]
        sec = tms / max(nl_, 1) * 1e-3
        peak = peaks.get("bf16_tflops")
        tb = traffic_per_unit.get(top)
        roof = {"bound": "tensor", "kernel": top, "achieved": alg[top] / sec / 1e12,
                "peak": peak, "unit": "TFLOP/s", "frac": alg[top] / sec / 1e12 / peak,
                "traffic": tb * counts["units"] if tb else None,
                "traffic_unit": "bytes per launch (ncu capture scaled by units)",
                "peak_source": ("fallback bf16 burst figure (MEASURED_PEAKS.json absent), of fallback"
                                if peaks.get("fallback") else "MEASURED_PEAKS.json bf16_tflops (burst), of measured"),
                "algorithmic_flop_per_launch": alg[top], "executed_mma_flop_per_launch": exe[top],
                "executed_frac": exe[top] / sec / 1e12 / peak,
                "note": "achieved = the angular sums' algorithmic flop (16 per order and angle); the "
                        "tensor cores execute executed_mma_flop (3 split products x 2 GEMMs on padded "
                        "tiles); the fused Mueller/PSD epilogue's FP32 work limits the kernel"}
    elif top is not None:
        nl_, tms = ktimes[top]
        roof = {"bound": "latency", "kernel": top, "achieved": None, "peak": None, "unit": None, "frac": None,
                "traffic": None, "ms_per_launch": tms / max(nl_, 1)}
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


# ---------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------
def reference_speed():
    """The port's speed over the reference's own pure-Python code on the same
    sulfate-table units, measured once on the build host
    (tests/golden/reference_speed.json, tests/golden/time_reference.py): the
    reference cannot travel to the GPU host."""
    try:
        with open(os.path.join(ROOT, "tests", "golden", "reference_speed.json")) as fp:
            return json.load(fp)
    except (OSError, ValueError):
        return None


def run_reference(args):
    """--impl reference: the CPU path timed on the host cores (rank 0 only)."""
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from oracle import gsf as ogsf
    ogsf.build()
    specs, desc, n_gsf, _, _ = build_config(3)
    cores = os.cpu_count() or 1
    allu = [(3, 0, li, ri, False) for li in REF_LAMBDA for ri in REF_RH]

    def step_units(k):   # one unit per core, rotating through the stratified list
        return [allu[(k * cores + j) % len(allu)] for j in range(cores)]
    pool = _pool(cores)   # created once, outside the timed steps
    try:
        for k in range(args.warmup):
            pool.map(_unit_task, step_units(k), chunksize=1)
        times, unit_s = [], []
        n = 0
        for k in range(args.warmup, args.warmup + args.steps):
            t0 = time.perf_counter()
            out = pool.map(_unit_task, step_units(k), chunksize=1)
            times.append(time.perf_counter() - t0)
            n += sum(o[3] for o in out)
            unit_s.extend(o[2] for o in out)
    finally:
        pool.close()
        pool.join()
    tot = sum(times)
    value = n / tot
    ninst = 4.32e6
    sample = ("%d (wavelength, RH) units of the table per step, one per core, rotating through %d stratified "
              "units (wavelength indices %s x RH indices %s); 2000 radii each, size by size, all 5 bins, 181 "
              "angles, 64 GSF moments; the full-table time is extrapolated from the sample's rate"
              % (cores, len(allu), REF_LAMBDA, REF_RH))
    rs = reference_speed()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                         "note": "CPU restatement of pymiecoated + dointegration (scipy jv/yv, size by size, "
                                 "per-angle sums; the reference's numba is not installed) and of "
                                 "spher_expan.f in C; a process pool over units created once before the "
                                 "warm-up"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "extrapolated_table_s": ninst / value,
        "per_unit_core_s_median": statistics.median(unit_s),
    }
    if rs:
        f = rs["port_over_reference"]
        line["reference_code"] = {"port_over_reference": f, "reference_equivalent_value": value / f,
                                  "extrapolated_table_s": ninst * f / value, "measured": rs["measured"]}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=3, help="headline workload 1..5 (default 3, sulfate)")
    ap.add_argument("--no-others", action="store_true", help="measure the headline workload only")
    ap.add_argument("--other-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--small", action="store_true", help="reduced sulfate table (quick check, not a bench line)")
    ap.add_argument("--lambdas", type=int, default=60, help="wavelengths of the sulfate table (profiling subsets)")
    ap.add_argument("--rh", type=int, default=36, help="RH values of the sulfate table (profiling subsets)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.lambdas != 60 or args.rh != 36:
        args.small = True   # a profiling subset, not a bench line
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
    from geosmie_gb300.table import TablePlan, run_tables
    ctx = _native.context(dev)
    peak = _native._D()
    ctx.call("gbmie_measure_fp64_peak", _native.ctypes.byref(peak))
    fp64_peak = peak.value
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        peaks = {"bf16_tflops": 1900.0, "hbm_gbs": 6800.0, "fallback": True}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:%d" % dev)
    stream = torch.cuda.current_stream(dev)

    def timed(plans, steps, warmup, graph=False, with_clocks=False):
        """Warm-up, then `steps` steps (every plan once) between barriers +
        syncs, L2 flushed before each step (256 MB write, inside the timed
        region).  Returns (ms, launches, kernel times, clocks)."""
        clocks = Clocks(dev)
        if with_clocks:
            clocks.start()   # sampling spans the last warm-up steps and the timed region
        for _ in range(warmup):
            for p in plans:
                p.run(graph=graph)
        for p in plans:
            p.sync()
        ctx.set_timing(True)
        launches0 = ctx.launches()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            flush.zero_()
            for p in plans:
                p.run(graph=graph)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        clk = clocks.stop() if with_clocks else None
        launches = ctx.launches() - launches0
        kt = ctx.kernel_times()
        ctx.set_timing(False)
        for p in plans:
            p.sync()   # device error flags -> status
        if ws > 1:
            ms = max_over_ranks(ms, ws, device="cuda:%d" % dev)
            torch.distributed.barrier()
        return ms, launches, kt, clk

    def measure(cfg, steps, warmup, headline):
        """Both precisions of workload cfg: FP64 table time, mixed table time
        (eager with per-kernel events, then replayed as CUDA graphs), the
        mixed-vs-FP64 errors, the end-to-end rate through run_tables, the
        roofline of the dominant mixed kernel; keeps both tables' results."""
        if args.small and cfg == 3:
            if args.lambdas != 60 or args.rh != 36:
                specs = [workloads.sulfate_table(n_rh=args.rh, n_lambda=args.lambdas)[0]]
                desc = "sulfate table subset: %d RH x %d wavelengths (profiling)" % (args.rh, args.lambdas)
            else:
                specs = [workloads.sulfate_table(n_rh=6, n_lambda=10, n_radii=500)[0]]
                desc = "reduced sulfate table (quick check)"
            n_gsf, nodes = 64, 0
        else:
            specs, desc, n_gsf, nodes, _ = build_config(cfg)
        tot, per = config_counts(cfg) if not args.small else (workloads.work_counts(specs[0]),) * 2
        r = {"cfg": cfg, "workload": desc, "instances": tot["instances"]}
        plans = [TablePlan(s, precision=_native.GBMIE_PLAIN_FP64, n_gsf=n_gsf, n_gsf_nodes=nodes, device=dev)
                 for s in specs]
        if headline:
            r["autotuned_plain"] = [p.autotune() for p in plans]
        ms_plain, _, kt_plain, _ = timed(plans, steps, warmup)
        r["plain"] = [p.results() for p in plans]
        for p in plans:
            p.close()
        del plans
        plans = [TablePlan(s, precision=_native.GBMIE_MIXED, n_gsf=n_gsf, n_gsf_nodes=nodes, device=dev)
                 for s in specs]
        r["autotuned_mixed"] = [p.autotune() for p in plans]
        ms_eager, _, ktimes, _ = timed(plans, steps, warmup)
        ms, launches, _, clk = timed(plans, steps, warmup, graph=True, with_clocks=headline)
        r["mixed"] = [p.results() for p in plans]
        if headline and specs[0].get("m_core") is None:
            # the same table with the D_n recurrence in FP64 from the
            # reference's start (the cost of that precision plan on this GPU)
            for p in plans:
                p.set_dn_fp64(True)
            ms_dn, _, kt_dn, _ = timed(plans, steps, warmup)
            dn = [p.results() for p in plans]
            for p in plans:
                p.set_dn_fp64(False)
            r["dn64"] = {"ms": ms_dn / steps, "coeff_kernel_ms": kt_dn.get("k_tab_coeffs_mixed_dn64", (1, None))[1],
                         "acc_vs_fp64": worst([accuracy(b, a, mixed=True) for a, b in zip(r["plain"], dn)])}
            if r["dn64"]["coeff_kernel_ms"] is not None:
                r["dn64"]["coeff_kernel_ms"] /= steps
        for p in plans:
            p.close()
        del plans
        r.update(ms_plain=ms_plain / steps, ms_eager=ms_eager / steps, ms=ms / steps, launches=launches,
                 clocks=clk, steps=steps, warmup=warmup)
        r["value"] = replica_value(tot["instances"], ws, steps, ms * 1e-3)
        r["plain_value"] = replica_value(tot["instances"], ws, steps, ms_plain * 1e-3)
        fwd = None
        if nodes:   # Gauss-node angles: the forward peak below 1 degree
            fwd = np.asarray(specs[0]["ang"]) < 1.0
        r["acc_mixed_vs_fp64"] = worst([accuracy(b, a, mixed=True, fwd=fwd) for a, b in zip(r["plain"], r["mixed"])])
        r["kernels"], r["roofline"] = roofline_of(ktimes, per, peaks, fp64_peak,
                                                  None if cfg == 3 and not args.small else {})
        r["kernels_plain"] = roofline_of(kt_plain, per, peaks, fp64_peak, {})[0]
        # end to end through the public API: host inputs in, host tables out
        probe = [TablePlan(s, precision=_native.GBMIE_MIXED, n_gsf=n_gsf, n_gsf_nodes=nodes, device=dev)
                 for s in specs]
        h2d = sum(v.numel() * v.element_size() for p in probe for v in p.t.values())
        d2h = sum(v.numel() * v.element_size() for p in probe for v in p.out_t.values())
        for p in probe:
            p.close()
        for _ in run_tables(specs * 2, precision=_native.GBMIE_MIXED, n_gsf=n_gsf, device=dev,
                            n_gsf_nodes=nodes):
            pass   # warm-up of the streams and the allocation pool
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        n_done = 0
        for _ in run_tables(specs * steps, precision=_native.GBMIE_MIXED, n_gsf=n_gsf, device=dev,
                            n_gsf_nodes=nodes):
            n_done += 1
        torch.cuda.synchronize(dev)
        e2e_s = max_over_ranks(time.perf_counter() - t0, ws, device="cuda:%d" % dev)
        r["e2e"] = {"value": replica_value(tot["instances"], ws, n_done / len(specs), e2e_s), "unit": UNIT,
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": e2e_s * 1e3 * len(specs) / max(n_done, 1)}
        return r

    head = measure(args.config, args.steps, args.warmup, headline=True)
    others = []
    if not args.no_others and not args.small:
        for cfg in [c for c in (1, 2, 3, 4, 5) if c != args.config]:
            others.append(measure(cfg, args.other_steps, 3, headline=False))

    # ---- oracle on the CPU: accuracy at stratified units, 1-core baseline ----
    oracle_of = {}
    if rank == 0 and not args.no_cpu_baseline and not args.small:
        tasks = [t for r in [head] + others for t in unit_tasks(r["cfg"])]
        pool = _pool(min(len(tasks), os.cpu_count() or 1))
        try:
            for key, sub, dt, ninst in pool.map(_unit_task, tasks, chunksize=1):
                oracle_of[key] = (sub, dt, ninst)
        finally:
            pool.close()
            pool.join()
    for r in [head] + others:
        units = build_config(r["cfg"])[4] if not args.small else []
        got = {u: oracle_of[(r["cfg"],) + u] for u in units if (r["cfg"],) + u in oracle_of}
        if got:
            r["acc_vs_oracle"] = oracle_accuracy(list(got), r["plain"], r["mixed"], {u: g[0] for u, g in got.items()})
            secs = sum(g[1] for g in got.values())
            inst = sum(g[2] for g in got.values())
            r["cpu_baseline"] = {"value": inst / secs, "unit": UNIT, "cores": 1, "kind": "port",
                                 "sample": "%d (wavelength, RH) units of the workload, every bin, all angles%s, "
                                           "%s; each unit on one core (units run side by side in a process pool)"
                                           % (len(got), ", GSF moments" if build_config(r["cfg"])[2] else "",
                                              "size by size" if r["cfg"] == 3 else "vectorised over sizes"),
                                 "seconds": secs}
        else:
            r["acc_vs_oracle"] = None
            r["cpu_baseline"] = None

    def compact(r):
        roof = r["roofline"] or {}
        return sig({"workload": r["workload"], "instances": r["instances"], "value": r["value"],
                    "table_ms": {"mixed": r["ms"], "plain_fp64": r["ms_plain"]},
                    "mixed_vs_plain_speedup": r["ms_plain"] / r["ms"],
                    "e2e": r["e2e"]["value"],
                    "roofline": {k: roof.get(k) for k in ("kernel", "bound", "achieved", "unit", "frac")},
                    "top_kernels_ms": {k: v["ms_per_launch"] for k, v in
                                       sorted(r["kernels"].items(), key=lambda kv: -kv[1]["share"])[:3]},
                    "cpu_baseline": r["cpu_baseline"]["value"] if r["cpu_baseline"] else None,
                    "mixed_vs_fp64": r["acc_mixed_vs_fp64"],
                    "vs_oracle": {k: (r["acc_vs_oracle"][k] if r["acc_vs_oracle"] else None)
                                  for k in ("fp64", "mixed")}}, 3)

    rs = reference_speed()
    h = head
    line = {
        "metric": METRIC, "value": h["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": h["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32-pair (double-float) recurrences + f16x2-split tensor contractions (f32 accumulate)",
        "data": "synthetic (seeded; no dataset)",
        "kernels": sig({k: {kk: v[kk] for kk in ("launches", "ms_per_launch", "share")}
                        for k, v in h["kernels"].items()}, 3),
        "kernels_plain_fp64": sig({k: {kk: v[kk] for kk in ("ms_per_launch", "share")}
                                   for k, v in h["kernels_plain"].items()}, 3),
        "autotuned": {"mixed": h["autotuned_mixed"], "plain_fp64": h.get("autotuned_plain")},
        "fp64_peak_gflops": fp64_peak,
        "config": {"workload": h["workload"], "instances": h["instances"],
                   "precision": "mixed: double-float (FP32-pair) D_n and N/M recurrences on FP64-built psi/chi "
                                "rows, tcgen05 split-FP16 contractions with FP32 accumulation",
                   "parallelism": "replicas" if ws > 1 else "1 GPU",
                   "l2": "flushed before every table (256 MB write inside the timed region)",
                   "launch": "whole table replayed as one CUDA graph (gbmie_table_run_graph)"},
        "configs": {str(r["cfg"]): compact(r) for r in others},
        "roofline": h["roofline"],
        "cpu_baseline": h["cpu_baseline"],
        "reference_code": ({"port_over_reference": rs["port_over_reference"], "measured": rs["measured"]}
                           if rs else None),
        "e2e": dict(h["e2e"], note="K tables through geosmie_gb300.table.run_tables: per table a plan from "
                                   "host arrays, its run and its results copied to page-locked host memory; "
                                   "plan creation and the copy back overlap the neighbouring tables' runs"),
        "gpu_launches": h["launches"],
        "clocks": h["clocks"],
        "dn_fp64_variant": sig(dict(h["dn64"], coeff_kernel_ms_default=h["kernels"].get("k_tab_coeffs_mixed", {}).get(
            "ms_per_launch")), 3) if h.get("dn64") else None,
        "table_gen_ms": sig({"mixed": h["ms"], "mixed_eager_launches": h["ms_eager"], "plain_fp64": h["ms_plain"]}),
        "mixed_vs_plain_speedup": sig(h["ms_plain"] / h["ms"]),
        "plain_fp64_value": sig(h["plain_value"]),
        "accuracy_mixed_vs_fp64": sig(h["acc_mixed_vs_fp64"], 3),
        "accuracy_vs_oracle": sig(h["acc_vs_oracle"], 3),
    }
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
