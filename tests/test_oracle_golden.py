"""Pin the CPU oracle to the reference (CPU only).

Known answers: pymiecoated/test/test_mie.py:45-109 (tolerance 1e3*DBL_EPS
there; the complex S12 comparison is made on |delta|/|ref| here).
Fixtures: tests/golden/*.npz, produced by tests/golden/make_golden.py from
the reference's own code.
"""
import json
import sys

import numpy as np
import pytest

from conftest import load_golden, relerr
from oracle import integration, pymie

EPS = 1e3 * sys.float_info.epsilon

# pymiecoated/test/test_mie.py:48-53,60-61 / :70-75,82-83 / :92-97,105-106
KAT = [
    (dict(eps=(1.5 + 0.5j) ** 2, x=2.5),
     (2.562873497454734, 1.0970718190883924, 1.4658016783663417, 0.12358646817981821,
      0.74890597894850719, 0.112651210275834),
     (complex(-0.49958438416709694, -0.24032581667666403),
      complex(0.11666852712178288, 0.051661382367147853))),
    (dict(eps=(1.5 + 0.5j) ** 2, eps2=(1.2 + 0.2j) ** 2, x=1.5, y=5.0),
     (2.0765452928100769, 0.90777572021757091, 1.168769572592506, 0.022692436240597712,
      0.90560220988567752, 0.024997844440209204),
     (complex(0.28677219451960079, -0.063605895700765691),
      complex(-0.32635924647084191, 0.12670342074119806))),
    (dict(eps=2.2 + 0.8j, mu=1.6 + 1.4j, x=4.0),
     (2.6665582594291073, 1.1255460946883893, 1.541012164740718, 0.0072453174040961301,
      0.89955981937838192, 0.0064371574281033928),
     (complex(0.14683196954000932, -0.017479181764394575),
      complex(-0.12475414168001844, 0.28120475717321358))),
]


@pytest.mark.parametrize("kw,eff_ref,s12_ref", KAT)
def test_known_answers(kw, eff_ref, s12_ref):
    an, bn, nmax = pymie.mie_coeffs(**kw)
    y = kw.get("y", kw["x"])
    eff = pymie.props(an, bn, nmax, y)
    for v, r in zip(eff, eff_ref):
        assert abs(v - r) / abs(r) < EPS
    s1, s2 = pymie.s12(an, bn, nmax, -0.6)
    assert abs(s1 - s12_ref[0]) / abs(s12_ref[0]) < EPS
    assert abs(s2 - s12_ref[1]) / abs(s12_ref[1]) < EPS


def test_errors_like_reference():
    # pymiecoated/test/test_mie.py:128-156 and mie_coeffs.py:45-60
    with pytest.raises(ValueError):
        pymie.mie_coeffs(eps=None, x=1.0)
    with pytest.raises(ValueError):
        pymie.mie_coeffs(eps=2.0, x=1.0, y=1.5)
    with pytest.raises(ValueError):
        pymie.mie_coeffs(eps=2.0, x=1.0, y=1.5, eps2=1.4, mu=1.5 + 0.6j)
    an, bn, nmax = pymie.mie_coeffs(eps=2.0, x=1.0)
    with pytest.raises(ValueError):
        pymie.s12(an, bn, nmax, -1.5)


def test_single_fixture_scalar_and_batch():
    g = load_golden("mie_single.npz")
    off = g["offsets"]
    ans, bns, nmax = pymie.batch_coeffs_homog(g["x"], g["eps"], g["mu"])
    for i in range(len(g["x"])):
        a, b, n = pymie.coeffs_homog(g["eps"][i], g["mu"][i], g["x"][i])
        ra, rb = g["an"][off[i]:off[i + 1]], g["bn"][off[i]:off[i + 1]]
        assert n == off[i + 1] - off[i]
        # same arithmetic as the reference: agreement to a few ulps
        assert np.max(np.abs(a - ra)) <= 1e-13 * max(1.0, np.max(np.abs(ra)))
        assert np.max(np.abs(ans[i] - ra)) <= 1e-13 * max(1.0, np.max(np.abs(ra)))
        eff = pymie.props(a, b, n, g["x"][i])
        assert np.all(relerr(eff[:2], g["eff"][i][:2]) < 1e-12)
        for k, u in enumerate(g["u"]):
            s1, s2 = pymie.s12(a, b, n, u)
            scale = max(abs(g["s1"][i, k]), abs(g["s2"][i, k]), 1e-300)
            assert abs(s1 - g["s1"][i, k]) / scale < 1e-11
            assert abs(s2 - g["s2"][i, k]) / scale < 1e-11


def test_coated_fixture():
    g = load_golden("mie_coated.npz")
    for i in range(len(g["x"])):
        a, b, n = pymie.mie_coeffs(eps=g["m1"][i] ** 2, eps2=g["m2"][i] ** 2, x=g["x"][i], y=g["y"][i])
        eff = pymie.props(a, b, n, g["y"][i])
        assert np.all(relerr(eff, g["eff"][i]) < 1e-12)


def test_size_range_fixture():
    g = load_golden("size_range.npz")
    v = pymie.size_range(g["x"], g["cost"], float(g["mr"]), float(g["mi"]))
    s1 = np.array([[a for a, _ in row] for row in v["s12"]])
    for k in ["qext", "qsca", "asy", "qb"]:
        assert np.all(relerr(np.array(v[k]), g[k]) < 1e-12)
    assert np.max(np.abs(s1 - g["s1"]) / np.max(np.abs(g["s1"]), axis=1, keepdims=True)) < 1e-12


@pytest.mark.parametrize("name", ["lognorm", "trivial", "seasalt", "su"])
def test_table_fixture(name):
    g = load_golden("table_%s.npz" % name)
    params = json.loads(str(g["params_json"]))
    out = integration.run_table(params, list(g["mlist"]), g["waterm"])
    for key in integration.SCATKEYS + integration.SCALARKEYS + integration.EXTRAKEYS + \
            integration.NLSCALARKEYS + ["pback"]:
        ref = g["out_" + key]
        got = out[key]
        assert got.shape == ref.shape, key
        scale = np.maximum(np.abs(ref), 1e-300)
        if key in ("p12", "p34", "p33", "p44", "p22"):
            scale = np.maximum(scale, np.abs(g["out_p11"]))
        if key == "pback":   # P12, P34 at 180 degrees are zero up to rounding
            scale = np.maximum(scale, np.abs(ref[..., :1]))
        assert np.max(np.abs(got - ref) / scale) < 1e-10, key
