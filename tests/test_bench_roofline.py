"""Roofline arithmetic of bench.py on the CPU: achieved = algorithmic flop
per launch (the reference algorithm's per-instance work) over the mean launch
time; the tensor cores' executed flop (split products, padding) is reported
beside it, not as the achieved figure."""
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402
from geosmie_gb300 import workloads  # noqa: E402

PEAKS = {"bf16_tflops": 1933.6, "hbm_gbs": 6694.5}


@pytest.fixture(scope="module")
def counts():
    spec, _ = workloads.sulfate_table(n_rh=6, n_lambda=10, n_radii=500)
    return workloads.work_counts(spec)


def test_mixed_roofline_is_algorithmic_tensor_work(counts):
    kt = {"k_tab_s12_tc": (4, 4.0), "k_tab_coeffs_mixed": (4, 3.0), "k_tab_scalars": (4, 0.6),
          "k_tab_finalize": (4, 0.4)}
    kernels, roof = bench.roofline_of(kt, counts, PEAKS, 3000.0)
    assert abs(sum(k["share"] for k in kernels.values()) - 1.0) < 1e-12
    alg = 16.0 * counts["sum_nmax"] * counts["nang"]
    assert roof["bound"] == "tensor" and roof["kernel"] == "k_tab_s12_tc" and roof["unit"] == "TFLOP/s"
    assert roof["achieved"] == pytest.approx(alg / 1e-3 / 1e12, rel=1e-12)
    assert roof["frac"] == pytest.approx(roof["achieved"] / PEAKS["bf16_tflops"], rel=1e-12)
    assert roof["algorithmic_flop_per_launch"] == alg
    # the executed MMA work (3 split products x 2 GEMMs, padded tiles) exceeds the algorithmic work
    assert roof["executed_mma_flop_per_launch"] > 3 * alg
    assert roof["executed_frac"] > roof["frac"]
    assert roof["traffic"] == pytest.approx(bench.NCU_BYTES_PER_UNIT["k_tab_s12_tc"] * counts["units"])
    w = 14.0 * counts["sum_nmx"] + 50.0 * counts["sum_nmax"]
    assert kernels["k_tab_coeffs_mixed"]["algorithmic_gflops"] == pytest.approx(w / 0.75e-3 / 1e9)
    assert kernels["k_tab_coeffs_mixed"]["fp64_equivalent_gflops_as_fp32_pairs"] > 0
    assert kernels["k_tab_s12_tc"]["algorithmic_tflops"] == pytest.approx(roof["achieved"])
    assert "k_tab_scalars" in kernels and "algorithmic_gflops" not in kernels["k_tab_scalars"]


def test_plain_roofline_is_fp64_pipe(counts):
    kt = {"k_tab_s12_plain": (2, 30.0), "k_tab_coeffs": (2, 10.0), "k_tab_scalars": (2, 1.0)}
    kernels, roof = bench.roofline_of(kt, counts, PEAKS, 3000.0)
    nang, inst, nbin = counts["nang"], counts["instances"], counts["nbin"]
    alg = 16.0 * counts["sum_nmax"] * nang + (12.0 + 12.0 * nbin) * nang * inst
    assert roof["bound"] == "fp64" and roof["kernel"] == "k_tab_s12_plain" and roof["unit"] == "GFLOP/s"
    assert roof["achieved"] == pytest.approx(alg / 15e-3 / 1e9, rel=1e-12)
    assert roof["frac"] == pytest.approx(roof["achieved"] / 3000.0, rel=1e-12)
    assert roof["traffic"] is None
    # the S+/S- form executes half the reference's multiply-adds of the sums
    exe = 8.0 * counts["sum_nmax"] * nang + (14.0 + 8.0 * nbin) * inst * nang
    assert roof["executed_flop_per_launch"] == exe and exe < alg
    assert kernels["k_tab_s12_plain"]["fp64_pipe_frac"] == pytest.approx(exe / 15e-3 / 1e9 / 3000.0)
    w = 14.0 * counts["sum_nmx"] + 50.0 * counts["sum_nmax"]
    assert kernels["k_tab_coeffs"]["algorithmic_gflops"] == pytest.approx(w / 5e-3 / 1e9)


def test_fallback_peak_is_named(counts):
    kt = {"k_tab_s12_tc": (1, 1.0)}
    _, roof = bench.roofline_of(kt, counts, {"bf16_tflops": 1900.0, "fallback": True}, 3000.0)
    assert "of fallback" in roof["peak_source"] and roof["peak"] == 1900.0
    _, roof = bench.roofline_of(kt, counts, PEAKS, 3000.0)
    assert "of measured" in roof["peak_source"]


def test_no_kernels_no_roofline(counts):
    assert bench.roofline_of({}, counts, PEAKS, 3000.0) == ({}, None)


def test_accuracy_summaries():
    """bench.accuracy: phase errors relative to P11 at the same angle, qabs
    relative to itself for the mixed path and to qext for FP64, moments
    relative to the entry's largest alpha1; oracle_accuracy compares a
    table's sample units with per-unit oracle results."""
    import numpy as np
    rng = np.random.default_rng(1)
    shp = (2, 3, 4)
    ref = {k: rng.uniform(1.0, 2.0, shp + (7,)) for k in bench.SCAT}
    ref.update({k: rng.uniform(1.0, 2.0, shp) for k in bench.SCALARS + ["qabs"]})
    ref["pback"] = rng.uniform(1.0, 2.0, shp + (6,))
    ref["pmom"] = rng.uniform(1.0, 2.0, shp + (6, 5))
    ref.update({"nl_" + k: rng.uniform(1.0, 2.0, shp) for k in bench.NLKEYS})
    got = {k: v.copy() for k, v in ref.items()}
    got["p34"][1, 2, 3, 4] += 1e-7 * ref["p11"][1, 2, 3, 4]
    got["qabs"][0, 0, 0] *= 1 + 3e-7
    got["pmom"][1, 1, 1, 2, 3] += 2e-7 * np.max(ref["pmom"][1, 1, 1, 0, :])
    a = bench.accuracy(got, ref, mixed=True)
    assert abs(a["phase_over_p11"] - 1e-7) < 1e-12
    assert abs(a["qabs_rel"] - 3e-7) < 1e-10 and "qabs_over_qext" not in a
    assert abs(a["pmom_over_alpha1"] - 2e-7) < 1e-12
    assert a["scalars_rel"] == 0.0 and a["nl_rel"] == 0.0
    b = bench.accuracy(got, ref)
    assert "qabs_over_qext" in b and b["qabs_over_qext"] <= 3e-7 * 2.0
    units = [(0, 1, 2), (0, 2, 3)]
    orc = {u: {k: v[:, u[1], u[2]] for k, v in ref.items()} for u in units}
    acc = bench.oracle_accuracy(units, [got], [ref], orc)
    assert acc["units"] == 2 and acc["mixed"]["phase_over_p11"] == 0.0
    assert abs(acc["fp64"]["phase_over_p11"] - 1e-7) < 1e-12
    assert bench.sig({"a": [1.23456789, 2]}, 3) == {"a": [1.23, 2]}


def test_config_sample_units_in_range():
    """Every oracle sample unit of the five workloads indexes an existing
    (table, wavelength, RH) unit; the headline sulfate units are timed size by
    size, the others vectorised."""
    for cfg in (1, 2, 3, 4):
        specs = bench.build_config(cfg)[0]
        for t in bench.unit_tasks(cfg):
            c, si, li, ri, batch = t
            m = specs[si]["m"]
            assert c == cfg and 0 <= li < m.shape[0] and 0 <= ri < m.shape[1]
            assert batch == (cfg != 3)
    tot, per = bench.config_counts(2)
    assert tot["instances"] == 5 * 40 * 1000 and per["instances"] == 40 * 1000
