"""Drop-in replacements of pymiecoated's ``Mie`` and ``MultipleMie``.

Same constructor keywords, properties, methods, cache and ValueError
conventions as pymiecoated/mie_coated.py:41-397 (see the method docstrings
for line references); every number is computed by libgbmie.so on the GPU.

Deliberate differences from the reference, each a fix of a reference bug:
  * ``Mie.m2`` returns sqrt(eps2); the reference getter recurses forever
    (mie_coated.py:366-367).
  * ``Mie(x=0)`` returns zero efficiencies, the stated intent of
    mie_coated.py:186-189, which raises NameError in the reference.
  * ``MultipleMie`` accepts a ``yArr`` of shell sizes (coated batch); the
    reference's coated batch branch cannot run (mie_coated.py:76-80).
  * ``ajv``/``ayv`` (caller-supplied Bessel arrays) are accepted and ignored:
    the Riccati-Bessel functions are always computed on the device.
"""
import collections

import numpy as np
import torch

from . import _native

__all__ = ["Mie", "MultipleMie", "Cache"]


class Cache(dict):
    """Bounded first-in-first-out cache of a Mie object's results: once more
    than `size` (10) parameter sets are stored, the oldest one is dropped
    (pymiecoated/mie_aux.py:22-33).  Storing a key that is already present
    replaces its value and keeps its place in the order."""

    def __init__(self, size=10):
        super().__init__()
        self.size = size
        self._order = collections.deque()

    @property
    def log(self):
        """The stored keys, oldest first."""
        return list(self._order)

    def __setitem__(self, key, value):
        if key not in self:
            self._order.append(key)
        super().__setitem__(key, value)
        while len(self._order) > self.size:
            super().pop(self._order.popleft(), None)

    def __delitem__(self, key):
        super().__delitem__(key)
        self._order.remove(key)


def _dev(a, dtype, device):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).to(device)


def coefficients(x, eps, mu=None, y=None, eps2=None, device=0, with_eff=True):
    """a_n, b_n (ragged, CSR by offsets) and efficiencies of many instances.

    Device counterpart of pymiecoated/mie_coeffs.py:36-73 batched: returns
    (offsets int64 [n+1], an complex128 [total], bn, eff float64 [n, 6]) as
    CUDA tensors.  Raises ValueError for the reference's invalid inputs.
    """
    ctx = _native.context(device)
    dv = ctx.device
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    n = x.size
    eps = np.broadcast_to(np.asarray(eps, dtype=np.complex128), (n,))
    dx = _dev(x, torch.float64, dv)
    deps = _dev(eps, torch.complex128, dv)
    dmu = None if mu is None else _dev(np.broadcast_to(np.asarray(mu, np.complex128), (n,)), torch.complex128, dv)
    dy = deps2 = None
    size = dx
    if y is not None:
        dy = _dev(np.broadcast_to(np.asarray(y, np.float64), (n,)), torch.float64, dv)
        deps2 = _dev(np.broadcast_to(np.asarray(eps2, np.complex128), (n,)), torch.complex128, dv)
        size = dy
    off = torch.empty(n + 1, dtype=torch.int64, device=dv)
    total = _native._I64()
    ctx.call("gbmie_layout", _native._I64(n), _native.ptr(size), _native.ptr(off), _native.ctypes.byref(total))
    an = torch.empty(max(total.value, 1), dtype=torch.complex128, device=dv)
    bn = torch.empty_like(an)
    eff = torch.empty((n, 6), dtype=torch.float64, device=dv) if with_eff else None
    ctx.call("gbmie_coeffs", _native._I64(n), _native.ptr(dx), _native.ptr(dy), _native.ptr(deps),
             _native.ptr(dmu), _native.ptr(deps2), _native.ptr(off), _native.ptr(an), _native.ptr(bn),
             _native.ptr(eff))
    ctx.sync()
    return off, an, bn, eff


def s12(off, an, bn, cos_theta, device=0):
    """S1, S2 [n, nang] complex128 (CUDA) from CSR coefficients."""
    ctx = _native.context(device)
    dv = ctx.device
    cost = _dev(np.atleast_1d(np.asarray(cos_theta, np.float64)), torch.float64, dv)
    n = off.numel() - 1
    s1 = torch.empty((n, cost.numel()), dtype=torch.complex128, device=dv)
    s2 = torch.empty_like(s1)
    ctx.call("gbmie_s12", _native._I64(n), _native.ptr(off), _native.ptr(an), _native.ptr(bn),
             _native._I32(cost.numel()), _native.ptr(cost), _native.ptr(s1), _native.ptr(s2))
    ctx.sync()
    return s1, s2


def pitau(cos_theta, nmax, device=0):
    """Scaled angular functions pi~_n, tau~_n [nang, nmax] (CUDA float64) at
    the given cosines (pymiecoated/mie_props.py:166-231, the rows of
    MultipleMie.preCalculatePT, mie_coated.py:160-179)."""
    ctx = _native.context(device)
    cost = _dev(np.atleast_1d(np.asarray(cos_theta, np.float64)), torch.float64, ctx.device)
    nmax = max(int(nmax), 2)
    pin = torch.empty((cost.numel(), nmax), dtype=torch.float64, device=ctx.device)
    tin = torch.empty_like(pin)
    ctx.call("gbmie_pitau", _native._I32(cost.numel()), _native.ptr(cost), _native._I32(nmax), _native.ptr(pin),
             _native.ptr(tin))
    ctx.sync()
    return pin, tin


def s12_pt(off, an, bn, pin, tin, device=0):
    """S1, S2 [n, nang] complex128 (CUDA) from CSR coefficients and
    caller-supplied scaled pi~/tau~ rows [nang, ld] with ld >= every
    instance's nmax (mie_props.py:115-149); ValueError if a row is shorter
    than an instance's nmax."""
    ctx = _native.context(device)
    dv = ctx.device
    pin = torch.as_tensor(np.asarray(pin, np.float64) if not torch.is_tensor(pin) else pin,
                          dtype=torch.float64).to(dv)
    tin = torch.as_tensor(np.asarray(tin, np.float64) if not torch.is_tensor(tin) else tin,
                          dtype=torch.float64).to(dv)
    if pin.dim() == 1:
        pin = pin[None, :]
        tin = tin[None, :]
    if pin.shape != tin.shape:
        raise ValueError("pin and tin must have the same shape")
    pin = pin.contiguous()
    tin = tin.contiguous()
    n = off.numel() - 1
    nang, ld = pin.shape
    s1 = torch.empty((n, nang), dtype=torch.complex128, device=dv)
    s2 = torch.empty_like(s1)
    ctx.call("gbmie_s12_pt", _native._I64(n), _native.ptr(off), _native.ptr(an), _native.ptr(bn),
             _native._I32(nang), _native._I32(ld), _native.ptr(pin), _native.ptr(tin), _native.ptr(s1),
             _native.ptr(s2))
    ctx.sync()
    return s1, s2


class MieScatterProps(object):
    """Coefficients of one parameter set and their properties
    (pymiecoated/mie_coated.py:181-211)."""

    def __init__(self, params, device=0):
        eps, mu, x, y, eps2 = params
        if x is None or eps is None:
            raise ValueError("Must specify x and either eps or m.")
        coated = y is not None
        if coated == (eps2 is None):
            raise ValueError("Must specify both y and m2 for coated particles.")
        mu = complex(1.0) if mu is None else complex(mu)
        if coated and mu != complex(1.0):
            raise ValueError("Multilayer calculations for magnetic particles are not currently supported.")
        self.device = device
        self.size = float(x) if y is None else float(y)
        if coated:
            off, an, bn, eff = coefficients([float(x)], complex(eps), None, [float(y)], complex(eps2), device)
        else:
            off, an, bn, eff = coefficients([float(x)], complex(eps), mu, None, None, device)
        self.off, self.an, self.bn = off, an, bn
        e = eff.cpu().numpy()[0]
        self._props = dict(zip(["qext", "qsca", "qabs", "qb", "asy", "qratio"], [float(v) for v in e]))

    @property
    def nmax(self):
        return int(self.off[-1].item())

    def prop(self, name):
        return self._props[name]

    def S12(self, u):
        s1, s2 = s12(self.off, self.an, self.bn, [float(u)], self.device)
        return complex(s1[0, 0].item()), complex(s2[0, 0].item())

    def S12_pt(self, pin, tin):
        """S1, S2 from caller-supplied scaled pi/tau arrays of at least nmax
        entries (mie_props.py:115-117), summed on the device by
        gbmie_s12_pt."""
        s1, s2 = s12_pt(self.off, self.an, self.bn, pin, tin, self.device)
        return complex(s1[0, 0].item()), complex(s2[0, 0].item())


class Mie(object):
    """pymiecoated.Mie (mie_coated.py:214-397) on the GPU.

    Attributes x, eps, mu, eps2, y, m, m2 as in the reference; methods qext,
    qsca, qabs, qb, asy, qratio, S12(u), S12_pt(pin, tin).
    """

    def __init__(self, **kwargs):
        self._cache = Cache()
        self.eps = None
        self.mu = 1.0
        self._x = None
        self._y = None
        self.eps2 = None
        self.ajv = ()
        self.ayv = ()
        self.device = kwargs.pop("device", 0)
        for k in ["eps", "mu", "eps2"]:
            if k in kwargs:
                self.__dict__[k] = kwargs[k]
        if "m" in kwargs:
            self.m = kwargs["m"]
        if "m2" in kwargs:
            self.m2 = kwargs["m2"]
        if "x" in kwargs:
            self.x = kwargs["x"]
        if "y" in kwargs:
            self.y = kwargs["y"]
        if "ajv" in kwargs:
            self.ajv = tuple(kwargs["ajv"])
        if "ayv" in kwargs:
            self.ayv = tuple(kwargs["ayv"])

    def _params_signature(self):
        return (self.eps, self.mu, self.x, self.y, self.eps2)

    def _get(self):
        sig = self._params_signature()
        if sig not in self._cache:
            self._cache[sig] = MieScatterProps(sig, self.device)
        return self._cache[sig]

    def qext(self):
        """Extinction efficiency."""
        return self._get().prop("qext")

    def qsca(self):
        """Scattering efficiency."""
        return self._get().prop("qsca")

    def qabs(self):
        """Absorption efficiency."""
        return self._get().prop("qabs")

    def qb(self):
        """Backscattering efficiency."""
        return self._get().prop("qb")

    def asy(self):
        """Asymmetry parameter <cos(theta)>."""
        return self._get().prop("asy")

    def qratio(self):
        """Backscattering ratio qb/qsca."""
        return self._get().prop("qratio")

    def S12(self, u):
        """Amplitude scattering matrix elements S1, S2 at cos(theta) = u
        (Bohren and Huffman conventions); ValueError unless -1 <= u <= 1."""
        if abs(u) > 1:
            raise ValueError("The cosine u must be between -1 and 1.")
        return self._get().S12(u)

    def S12_pt(self, pin, tin):
        return self._get().S12_pt(pin, tin)

    def _get_m(self):
        return np.sqrt(self.eps / self.mu)

    def _set_m(self, m):
        self.mu = 1.0
        self.eps = m ** 2

    m = property(_get_m, _set_m)

    def _get_m2(self):
        return np.sqrt(self.eps2) if self.eps2 is not None else None

    def _set_m2(self, m2):
        self.eps2 = m2 ** 2

    m2 = property(_get_m2, _set_m2)

    def _get_x(self):
        return self._x

    def _set_x(self, x):
        if x >= 0.0:
            self._x = x
        else:
            raise ValueError("The size x cannot be smaller than 0.")

    x = property(_get_x, _set_x)

    def _get_y(self):
        return self._y

    def _set_y(self, y):
        if y >= self.x:
            self._y = y
        else:
            raise ValueError("The size y cannot be smaller than x.")

    y = property(_get_y, _set_y)


class _S12Rows(object):
    """Per-size view of S1/S2 shaped like the reference's list of lists of
    (S1, S2) tuples: ``ret['s12'][i][k]`` is (S1, S2) at size i, cosine k."""

    def __init__(self, s1, s2):
        self.s1 = s1
        self.s2 = s2
        self._pairs = np.stack([s1, s2], axis=-1)

    def __len__(self):
        return self.s1.shape[0]

    def __getitem__(self, i):
        return self._pairs[i]

    def __iter__(self):
        return iter(self._pairs)


class MultipleMie(object):
    """pymiecoated.MultipleMie (mie_coated.py:41-179) on the GPU."""

    def __init__(self, xArr, yArr, costarr, device=0):
        self.xArr = np.asarray(xArr, dtype=np.float64)
        self.yArr = None if yArr is None else np.asarray(yArr, dtype=np.float64)
        self.costarr = np.asarray(costarr, dtype=np.float64)
        self.device = device
        self._dx = None
        self._dcost = None

    def preCalculate(self):
        """Stage the size and cosine arrays on the device (the reference's
        Bessel and pi/tau caches, mie_coated.py:149-179, are built on the GPU
        inside each sweep)."""
        ctx = _native.context(self.device)
        self._dx = _dev(self.xArr, torch.float64, ctx.device)
        self._dcost = _dev(self.costarr, torch.float64, ctx.device)

    def calculateS12(self, xx, eps, mu, jvarr=(), yvarr=()):
        """(S1, S2) at every cosine of costarr for one size parameter xx and
        permittivity/permeability eps, mu (mie_coated.py:51-53): a [nang, 2]
        complex array whose row k unpacks as (S1, S2).  jvarr/yvarr are
        accepted and ignored (Bessel functions are computed on the device)."""
        off, an, bn, _ = coefficients([float(xx)], complex(eps), None if mu is None else complex(mu),
                                      device=self.device, with_eff=False)
        s1, s2 = s12(off, an, bn, self.costarr, self.device)
        return np.stack([s1[0].cpu().numpy(), s2[0].cpu().numpy()], axis=-1)

    def calculateS12WithParams(self, xx, jvarr, yvarr, params):
        """(S1, S2) at every cosine of costarr from given coefficients
        params = (an, bn, nmax), as returned by pymiecoated's
        single_mie_coeff_numba (mie_coated.py:55-59): the scaled pi/tau rows
        of nmax at costarr (the reference's parr/tarr) are built on the
        device and the sums run there (gbmie_s12_pt)."""
        an, bn, nmax = params
        nmax = int(nmax)
        an = np.asarray(an, np.complex128)[:nmax]
        bn = np.asarray(bn, np.complex128)[:nmax]
        if an.size != nmax or bn.size != nmax:
            raise ValueError("params must hold nmax coefficients a_n and b_n")
        dv = _native.context(self.device).device
        off = torch.tensor([0, nmax], dtype=torch.int64, device=dv)
        pin, tin = pitau(self.costarr, nmax, self.device)
        s1, s2 = s12_pt(off, _dev(an, torch.complex128, dv), _dev(bn, torch.complex128, dv), pin, tin,
                        self.device)
        return np.stack([s1[0].cpu().numpy(), s2[0].cpu().numpy()], axis=-1)

    def calculateS12SizeRange(self, mr, mi):
        """S1/S2 at every cosine and the six efficiencies for every size,
        eps = (mr + i mi)^2, mu = 1 (mie_coated.py:61-89).  Returns the
        reference's dict: 's12' indexable as [size][angle] -> (S1, S2),
        and arrays for 'qext', 'qsca', 'qabs', 'asy', 'qb', 'qratio'."""
        if self._dx is None:
            self.preCalculate()
        ctx = _native.context(self.device)
        n, nang = self.xArr.size, self.costarr.size
        if self.yArr is not None:
            eps = complex(mr, mi) ** 2
            off, an, bn, eff = coefficients(self.xArr, eps, None, self.yArr, eps, self.device)
            s1, s2 = s12(off, an, bn, self.costarr, self.device)
        else:
            s1 = torch.empty((n, nang), dtype=torch.complex128, device=ctx.device)
            s2 = torch.empty_like(s1)
            eff = torch.empty((n, 6), dtype=torch.float64, device=ctx.device)
            ctx.call("gbmie_size_range", _native._I64(n), _native.ptr(self._dx), _native._D(mr), _native._D(mi),
                     _native._I32(nang), _native.ptr(self._dcost), _native.ptr(s1), _native.ptr(s2),
                     _native.ptr(eff))
            ctx.sync()
        e = eff.cpu().numpy()
        ret = {"s12": _S12Rows(s1.cpu().numpy(), s2.cpu().numpy())}
        for j, k in enumerate(["qext", "qsca", "qabs", "qb", "asy", "qratio"]):
            ret[k] = e[:, j].copy()
        return ret
