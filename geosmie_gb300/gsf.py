"""GSF expansion: the rungsf / convertncdf (pygeos mode) drop-in.

``expand`` replaces one run of gsf/spher_expan.f per scattering matrix
(convertncdf.py:173-189) with one batched GPU call; ``pmom_from_table``
replaces the (wavelength, RH, bin) loop of convertncdf.processFileRaw
(:319-401) including its output-order remap [0, 4, 2, 5, 1, 3] and the
zero padding to numExpand (129 in the reference).
"""
import ctypes

import numpy as np
import torch

from . import _native

ELEMENTS_IN = ["p11", "p22", "p33", "p44", "p12", "p34"]   # spher_expan.f input order
PYGEOS_REMAP = [0, 4, 2, 5, 1, 3]                           # convertncdf.py:381


def expand(ang_deg, F, nnodes=129, precision=_native.GBMIE_PLAIN_FP64, device=0):
    """Expansion coefficients of ntab matrices on one angle grid.

    ang_deg [nang] ascending degrees; F [ntab, 6, nang] as F11 F22 F33 F44 F12
    F34.  Returns (coef [ntab, 6, nnodes] as alpha1 alpha2 alpha3 alpha4 beta1
    beta2 normalised to alpha1(0) = 1, cnorm [ntab] = 1/alpha1(0)).  The
    reference's text output rounds to 10 decimals (spher_expan.f:104); these
    values are not rounded.
    """
    ctx = _native.context(device)
    dv = ctx.device
    ang = torch.as_tensor(np.ascontiguousarray(ang_deg, np.float64)).to(dv)
    Ft = torch.as_tensor(np.ascontiguousarray(F, np.float64)).to(dv)
    ntab = Ft.shape[0]
    coef = torch.empty((ntab, 6, nnodes), dtype=torch.float64, device=dv)
    cnorm = torch.empty(ntab, dtype=torch.float64, device=dv)
    ctx.call("gbmie_gsf", ctypes.c_int32(ntab), ctypes.c_int32(ang.numel()), _native.ptr(ang), _native.ptr(Ft),
             ctypes.c_int32(nnodes), _native.ptr(coef), _native.ptr(cnorm), ctypes.c_int32(precision))
    ctx.sync()
    return coef.cpu().numpy(), cnorm.cpu().numpy()


def pygeos_pmom(coef, num_expand=129):
    """pmom[..., p, m] from expansion coefficients [..., 6, L] in
    spher_expan's order (alpha1 alpha2 alpha3 alpha4 beta1 beta2): the output
    remap [0, 4, 2, 5, 1, 3] of convertncdf.py:381-394 (p order P11 P12 P33
    P34 P22 P44) and the zero padding (or truncation) to num_expand moments."""
    coef = np.asarray(coef, np.float64)
    pmom = np.zeros(coef.shape[:-2] + (6, num_expand))
    n = min(num_expand, coef.shape[-1])
    for ii, npol in enumerate(PYGEOS_REMAP):
        pmom[..., npol, :n] = coef[..., ii, :n]
    return pmom


def pmom_from_table(table, ang_deg, num_expand=129, nnodes=129, device=0):
    """pmom[bin, wavelength, rh, p, m] of a table (rungsf, pygeos mode)."""
    F = np.stack([table[k] for k in ELEMENTS_IN], axis=3)   # [bin, wl, rh, 6, nang]
    shp = F.shape
    coef, _ = expand(ang_deg, F.reshape(-1, 6, shp[-1]), nnodes, device=device)
    return pygeos_pmom(coef.reshape(shp[0], shp[1], shp[2], 6, nnodes), num_expand)
