"""Humidity growth of sulfate particles after CARMA (the 'su' growth law).

Restates geosmie/carma_utils.py:
  wtpct     :127-184  weight percent of H2SO4 in a sulfuric-acid droplet
                      (Tabazadeh et al. parameterisation, valid for 185-260 K)
                      at water activity = relative humidity
  density   :188-242  droplet density: the weight-percent table dnwtp with
                      density coefficients dnc0 + dnc1 T, linear in weight
                      percent between table entries
  grow_v75  :246-310  wet/dry radius ratio: the RH is corrected for the
                      Kelvin effect of a droplet of the dry size at 80 wt %,
                      then r_wet = r_dry (100 rho_dry / (wt% rho_wet))^(1/3)
used by particleparams.humidityGrowth (:103-108) for 'su' particles.  The
coefficient tables are the reference's, kept as they are (a table has to
be alike to give the same growth).  Scalar host arithmetic; it runs once
per (bin mode radius, RH) while a table is set up.
"""
import numpy as np

RHOP_DRY = 1.923   # g cm-3, dry sulfate density

# water activity ranges and (a, b, c, d) of the low and high temperature fits
_TAB = [
    (0.05, (12.37208932, -0.16125516114, -30.490657554, -2.1133114241),
     (13.455394705, -0.1921312255, -34.285174607, -1.7620073078)),
    (0.85, (11.820654354, -0.20786404244, -4.807306373, -5.1727540348),
     (12.891938068, -0.23233847708, -6.4261237757, -4.9005471319)),
    (None, (-180.06541028, -0.38601102592, -93.317846778, 273.88132245),
     (-176.95814097, -0.36257048154, -90.469744201, 267.45509988)),
]

DNWTP = [0., 1., 5., 10., 20., 25., 30., 35., 40., 41., 45., 50., 53., 55., 56., 60., 65., 66., 70., 72., 73., 74.,
         75., 76., 78., 79., 80., 81., 82., 83., 84., 85., 86., 87., 88., 89., 90., 91., 92., 93., 94., 95., 96., 97.,
         98., 100.]
DNC0 = [1., 1.13185, 1.17171, 1.22164, 1.3219, 1.37209, 1.42185, 1.4705, 1.51767, 1.52731, 1.56584, 1.61834,
        1.65191, 1.6752, 1.68708, 1.7356, 1.7997, 1.81271, 1.86696, 1.89491, 1.9092, 1.92395, 1.93904, 1.95438,
        1.98574, 2.00151, 2.01703, 2.03234, 2.04716, 2.06082, 2.07363, 2.08461, 2.09386, 2.10143, 2.10764, 2.11283,
        2.11671, 2.11938, 2.12125, 2.1219, 2.12723, 2.12654, 2.12621, 2.12561, 2.12494, 2.12093]
DNC1 = [0., -0.000435022, -0.000479481, -0.000531558, -0.000622448, -0.000660866, -0.000693492, -0.000718251,
        -0.000732869, -0.000735755, -0.000744294, -0.000761493, -0.000774238, -0.00078392, -0.000788939,
        -0.00080946, -0.000839848, -0.000845825, -0.000874337, -0.000890074, -0.00089873, -0.000908778,
        -0.000920012, -0.000932184, -0.000959514, -0.000974043, -0.000988264, -0.00100258, -0.00101634,
        -0.00102762, -0.00103757, -0.00104337, -0.00104563, -0.00104458, -0.00104144, -0.00103719, -0.00103089,
        -0.00102262, -0.00101355, -0.00100249, -0.00100934, -0.000998299, -0.000990961, -0.000985845,
        -0.000984529, -0.000989315]


def wtpct(relhum, temp=220.0):
    """Weight percent of H2SO4 at water activity relhum and temperature temp
    [K], restricted to [1, 100]."""
    activ = relhum
    if activ < 0.05:
        activ = max(activ, 1.e-6)
        lo, hi = _TAB[0][1], _TAB[0][2]
    elif activ <= 0.85:
        lo, hi = _TAB[1][1], _TAB[1][2]
    else:
        activ = min(activ, 1.)
        lo, hi = _TAB[2][1], _TAB[2][2]
    contl = lo[0] * (activ ** lo[1]) + lo[2] * activ + lo[3]
    conth = hi[0] * (activ ** hi[1]) + hi[2] * activ + hi[3]
    contt = contl + (conth - contl) * ((temp - 190.) / 70.)
    conwtp = (contt * 98.) + 1000.
    w = (100. * contt * 98.) / conwtp
    return min(max(w, 1.), 100.)


def density(relhum, temp=220.0):
    """Droplet density [g cm-3] at relative humidity relhum."""
    wtp = wtpct(relhum, temp=temp)
    i = 0
    while wtp > DNWTP[i]:
        i += 1
    den2 = DNC0[i] + DNC1[i] * temp
    if i == 0 or wtp == DNWTP[i]:
        return den2
    den1 = DNC0[i - 1] + DNC1[i - 1] * temp
    frac = (DNWTP[i] - wtp) / (DNWTP[i] - DNWTP[i - 1])
    return den1 * frac + den2 * (1.0 - frac)


def grow_v75(relhum, rd, temp=220.0):
    """Wet/dry radius ratio of a sulfate droplet of dry radius rd [m]."""
    rdry = rd * 100.                 # cm
    mw_h2so4 = 98.                   # g mol-1
    rgas = 8.31447e7                 # erg mol-1 K-1
    # water vapour mass concentration at relhum (saturation after the
    # Clausius-Clapeyron form with L, R_v at 0 C) [g cm-3]
    llv, rv, ttr, estr = 2.501e6, 461., 273.16, 611.
    es = estr * np.exp(llv / rv * (1. / ttr - 1 / temp))
    kb = 1.38e-23
    n_v = relhum * es / (kb * temp)
    navogad = 6.022e23
    mw_h2o = 0.018
    h2o_mass = n_v / navogad * mw_h2o * 1000. / 1.e6
    # Kelvin effect of a droplet of 80 wt % with the dry size's wet radius
    wtpkelv = 80.
    den1 = 2.00151 - 0.000974043 * temp
    den2 = 2.01703 - 0.000988264 * temp
    drho_dwt = den2 - den1
    sig1 = 79.3556 - 0.0267212 * temp
    sig2 = 75.608 - 0.0269204 * temp
    dsigma_dwt = (sig2 - sig1) / (85.9195 - 79.432)
    sigkelv = sig1 + dsigma_dwt * (80.0 - 79.432)
    rwet = rdry * (100. * RHOP_DRY / wtpkelv / den2) ** (1. / 3.)
    kb_ = 1. + wtpkelv * drho_dwt / den2 - 3. * wtpkelv * dsigma_dwt / (2. * sigkelv)
    ka_ = 2. * mw_h2so4 * sigkelv / (den1 * rgas * temp * rwet)
    h2o_kelv = h2o_mass / np.exp(ka_ * kb_)
    # the RH this corresponds to, then the wet radius at it
    k_cgs = 1.3807e-16
    mw_h2o_cgs = 18.
    rh_k = h2o_kelv * navogad / mw_h2o_cgs * k_cgs * temp / (es * 10.)
    rhopwet = density(rh_k, temp=temp)
    # (the reference evaluates this weight percent at its default 220 K)
    rwet = rdry * (100. * RHOP_DRY / wtpct(rh_k) / rhopwet) ** (1. / 3.)
    return rwet / rdry
