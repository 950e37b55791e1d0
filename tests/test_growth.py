"""CARMA sulfate growth (rhDep type 'su') on the CPU: geosmie_gb300.growth
against the reference's own carma_utils (wtpct :136-188, dens :190-243,
grow_v75 :245-314) over 126 (RH, dry radius, temperature) cases recorded in
tests/golden/growth_su.npz (tests/golden/make_golden.py).  The table driver
grows every lognormal mode radius of an 'su' table with grow_v75, so the
growth factors must be the reference's to the bit."""
import numpy as np

from conftest import load_golden
from geosmie_gb300 import growth


def test_grow_v75_bit_exact_cpu():
    g = load_golden("growth_su.npz")
    for i, h in enumerate(g["rh"]):
        for k, t in enumerate(g["temp"]):
            assert growth.wtpct(float(h), temp=float(t)) == g["wtpct"][i, k]
            assert growth.density(float(h), temp=float(t)) == g["dens"][i, k]
            for j, r in enumerate(g["rd"]):
                assert growth.grow_v75(float(h), float(r), temp=float(t)) == g["ratio"][i, j, k], (h, r, t)


def test_grow_v75_monotone_in_rh_cpu():
    """Wetter air grows a droplet more (property check over the fixture grid)."""
    g = load_golden("growth_su.npz")
    assert np.all(g["ratio"] > 1.0)
    assert np.all(np.diff(g["ratio"], axis=0) > 0)
