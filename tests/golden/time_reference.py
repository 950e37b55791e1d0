"""Measure how much faster the oracle's CPU port is than the reference's own
code on units of the sulfate-like benchmark table, and record the factor in
tests/golden/reference_speed.json (read by bench.py's reference arm, which
runs the port on the GPU host: the reference cannot travel there).

Run where the GEOSmie sources are present:

    python tests/golden/time_reference.py --ref /root/reference

(or with GEOSMIE_REF set).  For each unit (one wavelength, one RH of the
table, 2000 radii, 181 angles) it times, on one core:
  * reference: pymiecoated MultipleMie(x, None, cos).preCalculate() (its
    Bessel and pi/tau caches; charged at 1/36, since a radius grid shares it
    across the table's 36 RH values) + dointegration.rawMie (the per-size
    calculateS12SizeRange loop, Mueller elements), with the no-op numba shim
    of make_golden.py: pure Python, as numba is not installed;
  * port: oracle.integration.raw_mie(..., batch=False), the same work size by
    size.
The PSD integration and the GSF expansion are not part of the factor (the
same C restatement of spher_expan serves both; the integration is a few
dot products).
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
UNITS = [(0, 18), (30, 18), (59, 18)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("GEOSMIE_REF"),
                    help="root of the GEOSmie reference tree (default: $GEOSMIE_REF)")
    a = ap.parse_args()
    if not a.ref:
        ap.error("give --ref (or set GEOSMIE_REF) to the root of the GEOSmie reference tree")
    sys.path.insert(0, HERE)
    import make_golden
    make_golden._install_shims()
    src = os.path.join(a.ref, "src")
    sys.path.insert(0, os.path.join(src, "pymiecoated"))
    sys.path.insert(0, os.path.join(src, "geosmie"))
    sys.path.insert(0, ROOT)
    from pymiecoated.mie_coated import MultipleMie
    cwd = os.getcwd()
    os.chdir(src + "/geosmie")   # particleparams reads data/ relative to the working directory
    try:
        import dointegration as di
    finally:
        os.chdir(cwd)
    from geosmie_gb300 import workloads
    from oracle import integration as oi
    spec, _ = workloads.sulfate_table()
    cost = np.cos(np.radians(spec["ang"]))
    rows = []
    for li, ri in UNITS:
        lam = float(spec["lambda"][li])
        x = 2 * np.pi * np.asarray(spec["grid"]) / lam
        m = complex(spec["m"][li, ri, 0])
        t0 = time.perf_counter()
        mm = MultipleMie(x, None, cost)
        mm.preCalculate()
        t1 = time.perf_counter()
        ref = di.rawMie(mm, list(oi.SCATKEYS), ["qext", "qsca", "qabs", "qb", "g", "csca", "cext"], lam,
                        m.real, m.imag, None, cost)
        t2 = time.perf_counter()
        port = oi.raw_mie(x, cost, lam, m.real, m.imag, batch=False)
        t3 = time.perf_counter()
        err = max(float(np.max(np.abs(port[k] - ref[k]) / np.abs(ref["p11"]))) for k in oi.SCATKEYS)
        t_ref = (t1 - t0) / 36.0 + (t2 - t1)
        rows.append({"wavelength_index": li, "rh_index": ri, "reference_s": t_ref,
                     "reference_precalculate_s": t1 - t0, "port_s": t3 - t2, "max_phase_diff_over_p11": err})
        print(rows[-1])
    f = sum(r["reference_s"] for r in rows) / sum(r["port_s"] for r in rows)
    out = {"port_over_reference": f, "units": rows,
           "measured": "build host, one core each, pure-Python reference (numba not installed) against the "
                       "oracle port on %d sulfate-table units (2000 radii x 181 angles): Mie part "
                       "(coefficients, S1/S2, Mueller elements)" % len(rows)}
    with open(os.path.join(HERE, "reference_speed.json"), "w") as fp:
        json.dump(out, fp, indent=1)
    print("port / reference speed: %.1f" % f)


if __name__ == "__main__":
    main()
