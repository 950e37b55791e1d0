"""pymiecoated-compatible API: CPU-side validation and GPU parity.

CPU tests mirror pymiecoated/test/test_mie.py:112-156 (keywords, errors);
these raise before any device call.  GPU tests compare the CUDA path with the
reference's known answers (test_mie.py:45-109) and the golden fixtures.
Tolerances: 1e-10 relative for qext/qsca/asy (and the other efficiencies),
1e-9 for S1/S2 relative to the largest |S| of the instance.
"""
import sys

import numpy as np
import pytest

from conftest import eff_tolerance, load_golden, relerr
from geosmie_gb300 import Mie, MultipleMie

KAT_EPS = 1e3 * sys.float_info.epsilon


def test_errors_cpu():
    mie = Mie()
    with pytest.raises(ValueError):
        mie.x = -1.0
    mie.x = 1.0
    with pytest.raises(ValueError):
        mie.qext()                     # missing m
    mie.m = complex(1.5, 0.5)
    with pytest.raises(ValueError):
        mie.y = 0.5                    # y < x
    mie.y = 1.5
    with pytest.raises(ValueError):
        mie.qext()                     # y without m2
    mie.m2 = complex(1.2, 0.5)
    with pytest.raises(ValueError):
        mie.S12(-1.5)
    mie.mu = complex(1.5, 0.6)
    with pytest.raises(ValueError):
        mie.qext()                     # coated with mu != 1


def test_cache_first_in_first_out_cpu():
    """A Mie object's cache keeps its ten newest parameter sets
    (mie_aux.py:22-33); re-storing a key keeps its place."""
    from geosmie_gb300.mie import Cache
    c = Cache()
    for k in range(10):
        c[k] = str(k)
    c[3] = "again"
    assert len(c) == 10 and c[3] == "again" and c.log == list(range(10))
    c[10] = "10"
    assert 0 not in c and len(c) == 10 and c.log == list(range(1, 11))
    for k in range(11, 25):
        c[k] = str(k)
    assert sorted(c) == list(range(15, 25)) and c.log == list(range(15, 25))
    del c[20]
    c[25] = "25"
    assert sorted(c) == [15, 16, 17, 18, 19, 21, 22, 23, 24, 25]
    assert Mie()._cache.size == 10


def test_m2_getter_is_fixed():
    mie = Mie(m=1.5 + 0.5j, m2=1.2 + 0.2j, x=1.5, y=5.0)
    assert abs(mie.m2 - (1.2 + 0.2j)) < 1e-15


KAT = [
    (dict(m=complex(1.5, 0.5), x=2.5),
     (2.562873497454734, 1.0970718190883924, 1.4658016783663417, 0.12358646817981821,
      0.74890597894850719, 0.112651210275834),
     (complex(-0.49958438416709694, -0.24032581667666403), complex(0.11666852712178288, 0.051661382367147853))),
    (dict(m=complex(1.5, 0.5), m2=complex(1.2, 0.2), x=1.5, y=5.0),
     (2.0765452928100769, 0.90777572021757091, 1.168769572592506, 0.022692436240597712,
      0.90560220988567752, 0.024997844440209204),
     (complex(0.28677219451960079, -0.063605895700765691), complex(-0.32635924647084191, 0.12670342074119806))),
    (dict(eps=complex(2.2, 0.8), mu=complex(1.6, 1.4), x=4.0),
     (2.6665582594291073, 1.1255460946883893, 1.541012164740718, 0.0072453174040961301,
      0.89955981937838192, 0.0064371574281033928),
     (complex(0.14683196954000932, -0.017479181764394575), complex(-0.12475414168001844, 0.28120475717321358))),
]


@pytest.mark.gpu
@pytest.mark.parametrize("kw,eff_ref,s12_ref", KAT)
def test_known_answers_gpu(kw, eff_ref, s12_ref):
    mie = Mie(**kw)
    got = [mie.qext(), mie.qsca(), mie.qabs(), mie.qb(), mie.asy(), mie.qratio()]
    for g, r in zip(got, eff_ref):
        assert abs(g - r) / abs(r) < KAT_EPS
    s1, s2 = mie.S12(-0.6)
    assert abs(s1 - s12_ref[0]) / abs(s12_ref[0]) < KAT_EPS
    assert abs(s2 - s12_ref[1]) / abs(s12_ref[1]) < KAT_EPS


@pytest.mark.gpu
def test_keywords_gpu():
    mie = Mie(m=complex(1.5, 0.5), m2=complex(1.2, 0.2), x=1.5, y=5.0)
    mie2 = Mie()
    mie2.m = complex(1.5, 0.5)
    mie2.m2 = complex(1.2, 0.2)
    mie2.x = 1.5
    mie2.y = 5.0
    for f1, f2 in zip((mie.qext, mie.qsca, mie.qabs, mie.qb, mie.asy, mie.qratio),
                      (mie2.qext, mie2.qsca, mie2.qabs, mie2.qb, mie2.asy, mie2.qratio)):
        assert f1() == f2()


@pytest.mark.gpu
def test_single_fixture_gpu():
    from geosmie_gb300.mie import coefficients, s12
    g = load_golden("mie_single.npz")
    off, an, bn, eff = coefficients(g["x"], g["eps"], g["mu"])
    off = off.cpu().numpy()
    assert np.array_equal(off, g["offsets"])
    an = an.cpu().numpy()
    bn = bn.cpu().numpy()
    eff = eff.cpu().numpy()
    for i in range(len(g["x"])):
        sl = slice(off[i], off[i + 1])
        tol = eff_tolerance(g["eff"][i], g["x"][i], g["an"][sl], g["bn"][sl])
        assert np.all(np.abs(eff[i] - g["eff"][i]) <= tol), (i, g["x"][i], eff[i], g["eff"][i])
        # coefficients relative to the instance's largest |a_n|, with the same
        # small-x allowance (b_n's numerator cancels to O(x^2))
        sc = max(np.max(np.abs(g["an"][sl])), np.max(np.abs(g["bn"][sl])), 1e-300)
        ctol = 1e-10 + 1e3 * np.finfo(float).eps / g["x"][i] ** 2
        assert np.max(np.abs(an[sl] - g["an"][sl])) / sc < 1e-10
        assert np.max(np.abs(bn[sl] - g["bn"][sl])) / sc < ctol
    s1, s2 = s12(*coefficients(g["x"], g["eps"], g["mu"])[:3], g["u"])
    s1 = s1.cpu().numpy()
    s2 = s2.cpu().numpy()
    sc = np.maximum(np.max(np.abs(g["s1"]), axis=1, keepdims=True), np.max(np.abs(g["s2"]), axis=1, keepdims=True))
    assert np.max(np.abs(s1 - g["s1"]) / sc) < 1e-9
    assert np.max(np.abs(s2 - g["s2"]) / sc) < 1e-9


@pytest.mark.gpu
def test_coated_fixture_gpu():
    g = load_golden("mie_coated.npz")
    for i in range(len(g["x"])):
        mie = Mie(m=complex(g["m1"][i]), m2=complex(g["m2"][i]), x=float(g["x"][i]), y=float(g["y"][i]))
        got = np.array([mie.qext(), mie.qsca(), mie.qabs(), mie.qb(), mie.asy(), mie.qratio()])
        assert np.all(np.abs(got - g["eff"][i]) <= eff_tolerance(g["eff"][i], g["x"][i])), i
        sc = max(np.max(np.abs(g["s1"][i])), np.max(np.abs(g["s2"][i])))
        for k, u in enumerate(g["u"]):
            s1, s2 = mie.S12(float(u))
            assert abs(s1 - g["s1"][i, k]) / sc < 1e-9
            assert abs(s2 - g["s2"][i, k]) / sc < 1e-9


@pytest.mark.gpu
def test_size_range_fixture_gpu():
    g = load_golden("size_range.npz")
    mm = MultipleMie(g["x"], None, g["cost"])
    mm.preCalculate()
    v = mm.calculateS12SizeRange(float(g["mr"]), float(g["mi"]))
    for i, x in enumerate(g["x"]):
        ref = [g[k][i] for k in ["qext", "qsca", "qabs", "qb", "asy", "qratio"]]
        got = [v[k][i] for k in ["qext", "qsca", "qabs", "qb", "asy", "qratio"]]
        assert np.all(np.abs(np.array(got) - ref) <= eff_tolerance(ref, x)), (i, x)
    sc = np.max(np.abs(g["s1"]), axis=1, keepdims=True)
    assert np.max(np.abs(v["s12"].s1 - g["s1"]) / sc) < 1e-9
    assert np.max(np.abs(v["s12"].s2 - g["s2"]) / sc) < 1e-9
    # the reference's row access pattern (dointegration.py:1230-1231)
    row = v["s12"][3]
    assert complex(row[5][0]) == complex(v["s12"].s1[3, 5])


@pytest.mark.gpu
def test_calculate_s12_methods_gpu():
    """MultipleMie.calculateS12 and calculateS12WithParams (mie_coated.py:51-59)
    against the reference's own sweep and coefficients: calculateS12 per size
    against the size_range fixture, calculateS12WithParams with the
    reference's a_n/b_n (mie_single fixture) against the reference's S1/S2,
    1e-9 of the instance's largest |S|."""
    g = load_golden("size_range.npz")
    mm = MultipleMie(g["x"], None, g["cost"])
    mm.preCalculate()
    eps = complex(float(g["mr"]), float(g["mi"])) ** 2
    sc = np.max(np.abs(g["s1"]), axis=1)
    for i in [0, 17, 40, 79]:
        row = mm.calculateS12(float(g["x"][i]), eps, 1.0, (), ())
        assert row.shape == (g["cost"].size, 2)
        assert np.max(np.abs(row[:, 0] - g["s1"][i])) / sc[i] < 1e-9
        assert np.max(np.abs(row[:, 1] - g["s2"][i])) / sc[i] < 1e-9
    s = load_golden("mie_single.npz")
    mm = MultipleMie(s["x"], None, s["u"])
    off = s["offsets"]
    for i in range(0, len(s["x"]), 7):
        sl = slice(off[i], off[i + 1])
        row = mm.calculateS12WithParams(float(s["x"][i]), (), (), (s["an"][sl], s["bn"][sl], off[i + 1] - off[i]))
        scale = max(np.max(np.abs(s["s1"][i])), np.max(np.abs(s["s2"][i])))
        assert np.max(np.abs(row[:, 0] - s["s1"][i])) / scale < 1e-9, i
        assert np.max(np.abs(row[:, 1] - s["s2"][i])) / scale < 1e-9, i


@pytest.mark.gpu
def test_s12_pt_gpu():
    """Mie.S12_pt with the scaled pi/tau rows of gbmie_pitau equals Mie.S12
    at the same cosine (the reference's known answer, test_mie.py:45-53);
    rows longer than nmax are accepted, shorter ones raise ValueError."""
    from geosmie_gb300.mie import pitau
    mie = Mie(m=complex(1.5, 0.5), x=2.5)
    ref = KAT[0][2]
    for extra in (0, 9):
        nmax = mie._get().nmax
        pin, tin = pitau([-0.6], nmax + extra)
        s1, s2 = mie.S12_pt(pin[0].cpu().numpy(), tin[0].cpu().numpy())
        assert abs(s1 - ref[0]) / abs(ref[0]) < KAT_EPS
        assert abs(s2 - ref[1]) / abs(ref[1]) < KAT_EPS
    pin, tin = pitau([-0.6], mie._get().nmax - 1)
    with pytest.raises(ValueError):
        mie.S12_pt(pin[0].cpu().numpy(), tin[0].cpu().numpy())


@pytest.mark.gpu
def test_large_and_edge_sizes_gpu():
    from geosmie_gb300.mie import coefficients
    from oracle import pymie
    # x = k pi (psi_0 = 0), a root of tan x = x (psi_1 = 0), and large sizes
    xs = np.array([1e-4, 8e-4, 0.5, np.pi, 5 * np.pi, 50 * np.pi, 4.493409457909064, 300.0, 630.0, 2500.0])
    eps = (1.5 + 1e-8j) ** 2
    off, an, bn, eff = coefficients(xs, eps)
    eff = eff.cpu().numpy()
    for i, x in enumerate(xs):
        a, b, n = pymie.coeffs_homog(eps, 1.0, x)
        ref = np.array(pymie.props(a, b, n, x))
        assert np.all(np.abs(eff[i] - ref) <= eff_tolerance(ref, x, a, b)), (x, eff[i], ref)
    # x = 0: zero efficiencies (the reference's stated intent)
    off, an, bn, eff = coefficients([0.0, 1.0], 2.25)
    assert np.all(eff.cpu().numpy()[0] == 0.0)
    # NaN / negative sizes are rejected by the device checks
    with pytest.raises(ValueError):
        coefficients([1.0, float("nan")], 2.25)
    with pytest.raises(ValueError):
        coefficients([1.0, -2.0], 2.25)


@pytest.mark.gpu
def test_small_x_against_exact_values_gpu():
    """Where the reference's g is ill-conditioned (x << 1) the GPU value is at
    least as close to the 50-digit value as the reference's own."""
    from geosmie_gb300.mie import coefficients
    from oracle import pymie
    g = load_golden("mie_exact_small_x.npz")
    off, an, bn, eff = coefficients(g["x"], g["m"] ** 2)
    eff = eff.cpu().numpy()
    for i, (x, m) in enumerate(zip(g["x"], g["m"])):
        a, b, n = pymie.coeffs_homog(m * m, 1.0, x)
        ref = pymie.props(a, b, n, x)
        err_gpu = abs(eff[i, 4] - g["g"][i])
        err_ref = abs(ref[4] - g["g"][i])
        assert err_gpu <= err_ref + 1e-11 * abs(g["g"][i]), (x, m, err_gpu, err_ref)
        assert abs(eff[i, 1] - g["qsca"][i]) <= 1e-12 * g["qsca"][i]


@pytest.mark.gpu
def test_coated_shell_at_psi_zero_gpu():
    """A nearly real shell index with Re(m2 x) = k pi: psi_0(v) ~ 0."""
    from oracle import pymie
    m1, m2 = 1.95 + 0.79j, 1.333 + 1e-9j
    for x, y in [(4 * np.pi / 1.333, 20.0), (2 * np.pi / 1.333, 9.0)]:
        mie = Mie(m=m1, m2=m2, x=x, y=y)
        got = np.array([mie.qext(), mie.qsca(), mie.qabs(), mie.qb(), mie.asy(), mie.qratio()])
        a, b, n = pymie.coeffs_coated(m1 * m1, m2 * m2, x, y)
        ref = np.array(pymie.props(a, b, n, y))
        assert np.all(np.abs(got - ref) <= eff_tolerance(ref, y, a, b)), (x, y, got, ref)
