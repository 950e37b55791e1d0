"""Optics-table generation: the runoptics / dointegration.fun drop-in.

``fun(partID0, datatype, oppfx, oppclassic)`` and ``run_table(params, mlist,
waterm)`` follow geosmie/dointegration.py:672-1036: per size bin the
reference's size-parameter grid (initializeXarr :425-463), per wavelength the
interpolated refractive index (:700-710, :813-816), per RH the growth factor
and volume-mixed index (getHumidRefractiveIndex :493-536), PSD weights
(calculatePSD :539-664), Mie + Mueller + size integration (rawMie,
integratePSD :1064-1254) and the phase normalisation (:950-1001).

The host does the bookkeeping on small arrays (grids, indices, growth
factors); every per-size and per-angle number is computed by libgbmie.so
through ``gbmie_table_plan_create`` / ``gbmie_table_run``.  The NetCDF
writer of the reference (createNCDF :205-422) is not part of this module:
results come back as arrays with the reference file's variable names and its
non-legacy dimension order (bin, wavelength, rh, ...).
"""
import ctypes
import json
import os

import numpy as np
import torch

from . import _native, growth
from ._native import GRID_RADIUS, GRID_X, PSD_LOGNORM, PSD_POWER4, PSD_WEIGHTS  # noqa: F401

SCATKEYS = ["p11", "p12", "p22", "p33", "p34", "p44"]
SCALARKEYS = ["qext", "qsca", "qabs", "qb", "g", "csca", "cext"]
EXTRAKEYS = ["ssa", "bsca", "bext", "bbck", "refreal", "refimag", "lidar_ratio"]
NLSCALARKEYS = ["mass", "volume", "area", "rEff", "rMass", "rhop", "growth_factor", "rLow", "rUp"]
# order of the scalar block returned by the C ABI (GBMIE_S_*) and of the
# wavelength-independent block (GBMIE_N_*)
SCALAR_ORDER = ["qext", "qsca", "qabs", "qb", "g", "csca", "cext", "ssa", "bsca", "bext", "bbck",
                "refreal", "refimag", "lidar_ratio"]
NL_ORDER = ["mass", "volume", "area", "rEff", "rMass", "rhop", "growth_factor", "rLow", "rUp"]


class _Desc(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in
                ["n_lambda", "n_rh", "n_size", "n_bin", "n_comp", "n_ang", "grid_kind", "psd_kind",
                 "precision", "n_gsf"]] + \
               [(n, ctypes.c_void_p) for n in ["lambda_", "grid", "dgrid", "m", "psd_param", "gf_psd"]] + \
               [("rh0_index", ctypes.c_int32), ("n_gsf_nodes", ctypes.c_int32)] + \
               [(n, ctypes.c_void_p) for n in ["frac", "weights", "rhop", "rhop0", "gf", "rlow", "rup",
                                                "cos_theta", "theta", "m_core", "core_ratio"]]


class _Out(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ["phase", "pback", "scalar", "nl", "pmom"]]


def angmie():
    """The reference's 371 output angles (dointegration.py:739-742), degrees."""
    return np.concatenate([np.linspace(0.0, 1.0, 100, endpoint=False),
                           np.linspace(1.0, 10.0, 100, endpoint=False),
                           np.linspace(10.0, 180.0, 171, endpoint=True)])


def check_spec(spec):
    """Raise ValueError unless every array of a TablePlan spec has the size
    its dimensions (nl, nrh, ncomp from m; nbin from frac; ns from grid) ask
    for: the C plan takes plain pointers and cannot check them."""
    m = np.asarray(spec["m"])
    if m.ndim != 3:
        raise ValueError("spec['m']: [nl, nrh, ncomp] expected, got shape %s" % (m.shape,))
    nl, nrh, ncomp = m.shape
    frac = np.asarray(spec["frac"])
    if frac.ndim != 2 or frac.shape[1] != ncomp:
        raise ValueError("spec['frac']: [nbin, %d] expected, got shape %s" % (ncomp, frac.shape))
    nbin = frac.shape[0]
    ns = np.asarray(spec["grid"]).size
    need = [("lambda", (nl,)), ("dgrid", (ns,)), ("rhop", (nbin, nrh)), ("rhop0", (nbin,)), ("gf", (nrh,)),
            ("rlow", (nbin,)), ("rup", (nbin,))]
    if int(spec["psd_kind"]) == PSD_WEIGHTS:
        need.append(("weights", (nl, nrh, nbin, ncomp, ns)))
    else:
        need += [("psd_param", (nbin, ncomp, 4)), ("gf_psd", (nrh,))]
    if spec.get("m_core") is not None:
        need += [("m_core", (nl, nrh, ncomp)), ("core_ratio", (nrh,))]
    for k, shape in need:
        n = np.asarray(spec[k]).size
        if n != int(np.prod(shape)):
            raise ValueError("spec[%r]: %d values, %s = %d expected" % (k, n, list(shape), int(np.prod(shape))))


class TablePlan(object):
    """One planned table on the GPU (a C ``gbmie_table_plan``).

    ``spec`` holds host arrays (numpy) with the fields of gbmie_table_desc:
    lambda [nl] m, grid [ns], dgrid [ns], grid_kind, m [nl, nrh, ncomp]
    complex, psd_kind, psd_param [nbin, ncomp, 4], gf_psd [nrh], rh0_index,
    frac [nbin, ncomp], weights [nl, nrh, nbin, ncomp, ns] (psd_kind
    PSD_WEIGHTS), rhop [nbin, nrh], rhop0 [nbin], gf [nrh], rlow [nbin],
    rup [nbin], ang (degrees) [nang]; for coated spheres also m_core [nl,
    nrh, ncomp] complex (the core index; m is then the shell index and the
    grid the outer size) and core_ratio [nrh] (core / outer size parameter).
    Inputs are copied to the device once;
    ``run()`` launches the whole pipeline on the current stream (no host
    synchronisation, capturable in a CUDA graph).
    """

    def __init__(self, spec, precision=_native.GBMIE_PLAIN_FP64, n_gsf=0, device=0, n_gsf_nodes=0,
                 setup_stream=None):
        """setup_stream: a torch CUDA stream for the plan's own setup (input
        copy, layout kernels, operand tables), so that creating a plan does not
        wait for tables in flight on the caller's stream (run_tables)."""
        check_spec(spec)
        self.ctx = _native.context(device)
        dv = self.ctx.device
        self._run_stream = None
        ang = np.asarray(spec["ang"], np.float64)
        theta = np.radians(ang)
        lam = np.asarray(spec["lambda"], np.float64)
        m = np.asarray(spec["m"], np.complex128)
        nl, nrh, ncomp = m.shape
        frac = np.asarray(spec["frac"], np.float64)
        nbin = frac.shape[0]
        ns = len(spec["grid"])
        f64 = torch.float64

        # every input array in one page-locked staging block (256-byte aligned
        # parts) and one host -> device copy
        arrays = {
            "lambda": lam, "grid": spec["grid"], "dgrid": spec["dgrid"], "m": m, "frac": frac,
            "rhop": spec["rhop"], "rhop0": spec["rhop0"], "gf": spec["gf"], "rlow": spec["rlow"],
            "rup": spec["rup"], "cos_theta": np.cos(theta), "theta": theta,
        }
        if spec.get("m_core") is not None:   # coated spheres: core index per unit, core/outer size per RH
            arrays["m_core"] = np.asarray(spec["m_core"], np.complex128).reshape(m.shape)
            arrays["core_ratio"] = spec["core_ratio"]
        psd_kind = int(spec["psd_kind"])
        if psd_kind == PSD_WEIGHTS:
            arrays["weights"] = spec["weights"]
        else:
            arrays["psd_param"] = spec["psd_param"]
            arrays["gf_psd"] = spec["gf_psd"]
        parts, off = {}, 0
        for k, a in arrays.items():
            a = np.ascontiguousarray(a, np.complex128 if k in ("m", "m_core") else np.float64)
            parts[k] = (off, a)
            off += (a.nbytes + 255) // 256 * 256
        host = torch.empty(max(off, 256), dtype=torch.uint8, pin_memory=True)
        hv = host.numpy()
        for k, (o, a) in parts.items():
            hv[o:o + a.nbytes] = a.reshape(-1).view(np.uint8)
        setup = setup_stream if setup_stream is not None else torch.cuda.current_stream(dv)
        with torch.cuda.stream(setup):
            self._inputs = torch.empty(host.shape, dtype=torch.uint8, device=dv)
            self._inputs.copy_(host, non_blocking=True)
        setup.synchronize()   # the plan's kernels run on the context's stream
        self.t = {}
        for k, (o, a) in parts.items():
            dt = torch.complex128 if a.dtype == np.complex128 else f64
            self.t[k] = self._inputs[o:o + a.nbytes].view(dt).view(a.shape)
        desc = _Desc()
        desc.n_lambda, desc.n_rh, desc.n_size, desc.n_bin, desc.n_comp = nl, nrh, ns, nbin, ncomp
        desc.n_ang = ang.size
        desc.grid_kind = int(spec["grid_kind"])
        desc.psd_kind = psd_kind
        desc.precision = int(precision)
        desc.n_gsf = int(n_gsf)
        desc.n_gsf_nodes = int(n_gsf_nodes)   # 0: n_gsf nodes, as the reference
        desc.rh0_index = int(spec.get("rh0_index", 0))

        def p(k):
            t = self.t.get(k)
            return None if t is None else t.data_ptr()
        desc.lambda_ = p("lambda")
        for k in ["grid", "dgrid", "m", "psd_param", "gf_psd", "frac", "weights", "rhop", "rhop0", "gf",
                  "rlow", "rup", "cos_theta", "theta", "m_core", "core_ratio"]:
            setattr(desc, k, p(k))
        self.desc = desc
        self.shape = (nbin, nl, nrh)
        self.nang = ang.size
        self.ang = ang
        self.n_gsf = int(n_gsf)
        h = ctypes.c_void_p()
        nbytes = ctypes.c_int64()
        with torch.cuda.stream(setup):   # synchronises the setup stream only
            self.ctx.call("gbmie_table_plan_create", ctypes.byref(desc), ctypes.byref(h), ctypes.byref(nbytes))
        self.h = h
        self.scratch_bytes = nbytes.value
        ne = nbin * nl * nrh
        # all outputs in one device block (one device -> host copy in results())
        shapes = {"phase": (nbin, nl, nrh, 6, ang.size), "pback": (nbin, nl, nrh, 6),
                  "scalar": (nbin, nl, nrh, _native.NSCALAR), "nl": (nbin, nl, nrh, _native.NNL)}
        if n_gsf:
            shapes["pmom"] = (nbin, nl, nrh, 6, n_gsf)
        self._out_off, n = {}, 0
        for k, shp in shapes.items():
            self._out_off[k] = (n, shp)
            n += (int(np.prod(shp)) + 31) // 32 * 32   # 256-byte aligned parts
        self._out_block = torch.empty(n, dtype=f64, device=dv)
        self.out_t = {k: self._out_block[o:o + int(np.prod(shp))].view(shp) for k, (o, shp) in self._out_off.items()}
        out = _Out()
        for k, v in self.out_t.items():
            setattr(out, k, v.data_ptr())
        self.out = out
        self.n_entries = ne
        self.n_instances = nl * nrh * ncomp * ns

    def run(self, graph=False):
        """Launch the table pipeline on the context stream.  graph=True
        replays it as one CUDA graph (captured on the first such call,
        gbmie_table_run_graph)."""
        rs = torch.cuda.current_stream(self.ctx.device)
        if self._run_stream is None or rs != self._run_stream:
            self._inputs.record_stream(rs)   # the inputs may come from another (setup) stream
        self._run_stream = rs
        self.ctx.call("gbmie_table_run_graph" if graph else "gbmie_table_run", self.h, ctypes.byref(self.out))
        self._run_done = torch.cuda.Event()   # this run's end (later work on rs is not waited for)
        self._run_done.record(rs)

    def autotune(self):
        """Tune the launch parameters on this plan's data (synchronous; ends
        with a run of the tuned table) and return them (see tuning())."""
        self.ctx.call("gbmie_table_plan_autotune", self.h, ctypes.byref(self.out))
        return self.tuning()

    def set_wait_limit(self, tries):
        """Tries of every pipeline wait of the mixed path's tensor-core
        contraction before it gives up and reports a device timeout (raised
        by the next sync()); None restores the default.  0 makes every wait
        give up at once: a way to test timeout handling without a hang."""
        self.ctx.check(self.ctx.lib.gbmie_table_plan_set_wait_limit(self.h, -1 if tries is None else int(tries)),
                       "gbmie_table_plan_set_wait_limit")

    def set_dn_fp64(self, enable):
        """Mixed plans of homogeneous spheres: run the D_n recurrence in FP64
        from the reference's start (True) or in double-float pairs with the
        shortened warm-up (False, the default)."""
        self.ctx.check(self.ctx.lib.gbmie_table_plan_set_dn_fp64(self.h, int(bool(enable))),
                       "gbmie_table_plan_set_dn_fp64")

    def tuning(self):
        """{'tuned', 'plain_per_bucket', 'plain_chunk' [5], 'plain_threads'
        [5], 'coef_block', 'tc_window'}: the plan's launch parameters (nmax
        buckets <= 16, <= 64, <= 256, more, then the whole-grid launch)."""
        q = (ctypes.c_int32 * 16)()
        self.ctx.check(self.ctx.lib.gbmie_table_plan_tuning(self.h, q), "gbmie_table_plan_tuning")
        return {"tuned": bool(q[0]), "plain_per_bucket": bool(q[1]), "plain_chunk": list(q[2:7]),
                "plain_threads": list(q[7:12]), "coef_block": int(q[12]), "tc_window": int(q[13])}

    def set_tuning(self, tun):
        """Launch parameters in the form tuning() returns (those of an earlier
        autotuning, say): a table's bits depend only on them, so saved
        parameters reproduce a table exactly in another process."""
        q = (ctypes.c_int32 * 16)()
        q[1] = int(bool(tun["plain_per_bucket"]))
        for b in range(5):
            q[2 + b] = int(tun["plain_chunk"][b])
            q[7 + b] = int(tun["plain_threads"][b])
        q[12] = int(tun["coef_block"])
        q[13] = int(tun["tc_window"])
        self.ctx.check(self.ctx.lib.gbmie_table_plan_set_tuning(self.h, q), "gbmie_table_plan_set_tuning")

    def sync(self):
        """Wait for the plan's last run (on its stream) and raise on a device
        error flag."""
        rs = self._run_stream if self._run_stream is not None else torch.cuda.current_stream(self.ctx.device)
        with torch.cuda.stream(rs):
            self.ctx.bind_stream()
            self.ctx.sync()

    def close(self):
        """Destroy the plan: its arrays are freed in order on the stream of its
        last run (no wait for the device)."""
        if getattr(self, "h", None) is not None and self.h.value:
            rs = self._run_stream if self._run_stream is not None else torch.cuda.current_stream(self.ctx.device)
            with torch.cuda.stream(rs):
                self.ctx.bind_stream()
                self.ctx.lib.gbmie_table_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def results_async(self, copy_stream):
        """Start the device -> host copy of the tables after the last run, on
        copy_stream; returns a PendingResults whose get() waits for the copy
        only (tables launched afterwards keep running)."""
        hb = torch.empty(self._out_block.shape, dtype=self._out_block.dtype, pin_memory=True)
        if self._run_stream is None:
            copy_stream.wait_stream(torch.cuda.current_stream(self.ctx.device))
        else:
            copy_stream.wait_event(self._run_done)
        with torch.cuda.stream(copy_stream):
            hb.copy_(self._out_block, non_blocking=True)
        self._out_block.record_stream(copy_stream)
        done = torch.cuda.Event()
        done.record(copy_stream)
        return PendingResults(self, hb, done, copy_stream)

    def _unpack(self, hb):
        host = {k: hb[o:o + int(np.prod(shp))].view(shp) for k, (o, shp) in self._out_off.items()}
        ph = host["phase"].numpy()
        sc = host["scalar"].numpy()
        nlv = host["nl"].numpy()
        res = {k: ph[..., i, :] for i, k in enumerate(SCATKEYS)}
        res.update({k: sc[..., i] for i, k in enumerate(SCALAR_ORDER)})
        res.update({"nl_" + k: nlv[..., i] for i, k in enumerate(NL_ORDER)})
        res["pback"] = host["pback"].numpy()
        if "pmom" in host:
            res["pmom"] = host["pmom"].numpy()
        return res

    def results(self):
        """Host dict: scatkeys [nbin, nl, nrh, nang], scalar keys [nbin, nl,
        nrh], pback [nbin, nl, nrh, 6], wavelength-independent keys [nbin, nl,
        nrh] (per wavelength), pmom [nbin, nl, nrh, 6, n_gsf] (p order P11
        P12 P33 P34 P22 P44, i.e. alpha1 beta1 alpha3 beta2 alpha2 alpha4)."""
        self.sync()
        # the output block -> a page-locked host block in one copy (about 5x
        # the bandwidth of pageable copies for the 130 MB sulfate table); a
        # fresh block per call, so earlier results stay valid (torch caches
        # page-locked blocks)
        hb = torch.empty(self._out_block.shape, dtype=self._out_block.dtype, pin_memory=True)
        cs = torch.cuda.current_stream(self.ctx.device)
        with torch.cuda.stream(cs):
            hb.copy_(self._out_block, non_blocking=True)
        cs.synchronize()
        return self._unpack(hb)


class PendingResults(object):
    """A table's results on their way to the host (TablePlan.results_async)."""

    def __init__(self, plan, hb, done, stream):
        self.plan, self.hb, self.done, self.stream = plan, hb, done, stream

    def get(self):
        """Wait for the copy; the device status (error flags) is read on the
        copy stream, so that tables in flight elsewhere are not waited for."""
        self.done.synchronize()
        with torch.cuda.stream(self.stream):
            self.plan.ctx.bind_stream()
            self.plan.ctx.sync()
        return self.plan._unpack(self.hb)


def run_tables(specs, precision=_native.GBMIE_MIXED, n_gsf=0, device=0, n_gsf_nodes=0):
    """Tables of a sequence of specs, pipelined on one GPU: plan i + 1 is
    created (host work, input copy and setup kernels on a setup stream) while
    table i runs, and table i's results are copied back (on a copy stream)
    while table i + 1 runs; plans are closed without waiting for the device.
    Yields each table's results dict (TablePlan.results) in order."""
    dv = _native.context(device).device
    setup = torch.cuda.Stream(dv)
    copy = torch.cuda.Stream(dv)
    it = iter(specs)
    try:
        spec = next(it)
    except StopIteration:
        return
    plan = TablePlan(spec, precision=precision, n_gsf=n_gsf, device=device, n_gsf_nodes=n_gsf_nodes,
                     setup_stream=setup)
    nxt = None
    try:
        plan.run()
        while plan is not None:
            try:
                spec = next(it)
                nxt = TablePlan(spec, precision=precision, n_gsf=n_gsf, device=device, n_gsf_nodes=n_gsf_nodes,
                                setup_stream=setup)
                nxt.run()
            except StopIteration:
                nxt = None
            pend = plan.results_async(copy)
            res = pend.get()
            plan.close()
            yield res
            plan, nxt = nxt, None
    finally:
        # a consumer that stops early, or an error: the open plans are
        # destroyed now (in order on their run streams), not at collection
        for p_ in (plan, nxt):
            if p_ is not None:
                p_.close()


# ---------------------------------------------------------------------------
# reference-style host bookkeeping (small arrays only)
# ---------------------------------------------------------------------------
def _get_dr(arr):
    """Centred differences (dointegration.py:93-101)."""
    arr = np.asarray(arr, np.float64)
    d = np.empty_like(arr)
    d[0] = arr[1] - arr[0]
    d[1:-1] = ((arr[1:-1] - arr[:-2]) + (arr[2:] - arr[1:-1])) / 2.0
    d[-1] = arr[-1] - arr[-2]
    return d


def _carma_grid(minx, maxx, nbinperdecade):
    """Volume-ratio size grid and widths (dointegration.py:103-153).

    The powers are taken one grid point at a time as scalars, as the
    reference does: numpy's vectorised power rounds differently (by an ulp
    here and there, and differently per CPU), and the grid then no longer
    equals the reference's bit for bit."""
    rat = maxx / minx
    nbin = np.log10(maxx / minx) * nbinperdecade
    rmrat = (rat ** 3) ** (1.0 / nbin)
    rmin = minx * ((1.0 + rmrat) / 2.0) ** (1.0 / 3.0)
    cpi = 4.0 / 3.0 * np.pi
    rvolmin = cpi * rmin ** 3.0
    vrfact = ((3.0 / 2.0 / np.pi / (rmrat + 1)) ** (1.0 / 3.0)) * (rmrat ** (1.0 / 3.0) - 1.0)
    n = int(nbin)
    r = np.empty(n)
    dr = np.empty(n)
    for k in range(n):
        rvol = rvolmin * rmrat ** k
        r[k] = (rvol / cpi) ** (1.0 / 3.0)
        dr[k] = vrfact * rvol ** (1.0 / 3.0)
    return r, dr


def _x_grid(params, b, minlam, maxlam):
    """initializeXarr (dointegration.py:425-463)."""
    pp = params["psd"]["params"]
    t = params["psd"]["type"]
    if t == "lognorm":
        return _carma_grid(pp["rmin0"][b][0] * 2 * np.pi / maxlam, pp["rmax0"][b][-1] * 2 * np.pi / minlam * 3.0,
                           pp["numperdec"][b])
    if t == "ss":
        return _carma_grid(pp["rMinMaj"][b] * 2 * np.pi / maxlam, pp["rMaxMaj"][b] * 2 * np.pi / minlam * 10,
                           pp["numperdec"][b])
    if t == "du":
        minx = pp["rMinMaj"][b][0] * 2 * np.pi / maxlam
        maxx = pp["rMaxMaj"][b][-1] * 2 * np.pi / minlam
        return (np.linspace(np.log10(minx), np.log10(maxx), 1000)) ** 10.0, None
    raise ValueError("unknown psd type %s" % t)


def _growth(rhdep, siz0, rh, allrh):
    """humidityGrowth (particleparams.py:85-108): 'simple', 'trivial', 'ss'
    (Gerber) and 'su' (CARMA sulfate, growth.grow_v75)."""
    rhi = list(allrh).index(rh)
    t = rhdep["type"]
    p = rhdep["params"]
    if t in ("simple", "trivial"):
        return siz0 * p["gf"][rhi]
    if t == "ss":
        if rh == 0.0:
            return siz0
        siz = siz0 * 100
        return (p["c1"] * siz ** p["c2"] / (p["c3"] * siz ** p["c4"] - np.log10(rh)) + siz ** 3.0) ** (1.0 / 3.0) / 100.0
    if t == "su":
        if rh == 0.0:
            return siz0
        return siz0 * float(growth.grow_v75(rh, siz0, temp=p["temp"]))
    raise NotImplementedError("growth law '%s' is not implemented" % t)


def _lognorm_weights(params, b, rh_list, x, dx, lams):
    """Lognormal PSD weights of bin b with size-dependent growth ('su'):
    calculatePSD's lognorm branch (dointegration.py:549-583) -- every mode
    radius and upper bound grown by humidityGrowth at its own dry size,
    getLogNormPSD (particleparams.py:113-128) in size-parameter space, times
    the grid's dx, normalised -- [nl, nrh, ncomp, ns]."""
    pp = params["psd"]["params"]
    ncomp = len(pp["r0"][b])
    out = np.zeros((lams.size, len(rh_list), ncomp, x.size))
    for li, lam in enumerate(lams):
        xconv = 2 * np.pi / lam
        for ri, onerh in enumerate(rh_list):
            for k in range(ncomp):
                rmode = _growth(params["rhDep"], pp["r0"][b][k], onerh, rh_list)
                rmax = _growth(params["rhDep"], pp["rmax0"][b][k], onerh, rh_list)
                rmin = pp["rmin0"][b][k]
                sig = pp["sigma"][b][k]
                xmode, xmax, xmin = rmode * xconv, rmax * xconv, rmin * xconv
                d = 1. / (x * (2 * np.pi) ** 0.5 * np.log(sig)) * np.exp(-(np.log(x / xmode) ** 2) /
                                                                         (2. * np.log(sig) ** 2))
                d[np.where(x >= xmax)] = 0.
                d[np.where(x <= xmin)] = 0.
                d = d * dx
                out[li, ri, k] = d / np.sum(d)
    return out


def _ss_weights(params, b, rh_list, x, lams):
    """Gong sea-salt PSD weights (dointegration.py:585-624) [nl, nrh, ns]."""
    pp = params["psd"]["params"]
    rminmaj, rmaxmaj = pp["rMinMaj"][b], pp["rMaxMaj"][b]
    out = np.zeros((lams.size, len(rh_list), x.size))
    for li, lam in enumerate(lams):
        rarr = x / (2 * np.pi / lam)
        dr = _get_dr(rarr)
        for ri, onerh in enumerate(rh_list):
            rminuse = _growth(params["rhDep"], rminmaj, onerh, rh_list)
            rmaxuse = _growth(params["rhDep"], rmaxmaj, onerh, rh_list)
            rrat = rminmaj / rminuse
            r80rat = 1.65 * rrat
            r80 = rarr * r80rat * 1e6
            afac = 4.7 * (1.0 + 30.0 * r80) ** (-0.017 * r80 ** (-1.44))
            bfac = (0.433 - np.log10(r80)) / 0.433
            dndr = 1.373 * r80 ** (-afac) * (1.0 + 0.057 * r80 ** 3.45) * 10.0 ** (1.607 * np.exp(-bfac ** 2.0)) * r80rat
            dndr[rarr < rminuse] = 0.0
            dndr[rarr > rmaxuse] = 0.0
            dndr = dndr / np.sum(dndr)
            w = dndr * dr
            out[li, ri] = w / np.sum(w)
    return out


def bin_spec(params, b, mlist, waterm, ang, lambdas=None):
    """The TablePlan spec of size bin b of a reference particle definition."""
    lam = np.asarray(mlist[0][0], np.float64) if lambdas is None else np.asarray(lambdas, np.float64)
    rh = list(params["rh"])
    if "maxrh" in params:
        rh = list(np.minimum(np.array(rh, dtype=np.float64), params["maxrh"]))
    rtype = params["rhDep"]["type"]
    ptype = params["psd"]["type"]
    pp = params["psd"]["params"]
    trivial = rtype == "trivial"
    rh_run = rh[:1] if trivial else rh
    x, dx = _x_grid(params, b, lam[0], lam[-1])
    # refractive indices: particle (imaginary sign flipped, :813-816) and water
    n0 = np.array([[complex(np.interp(l_, t[0], t[1]), -np.interp(l_, t[0], t[2])) for t in mlist] for l_ in lam])
    if trivial:
        nw = np.ones(lam.size, np.complex128)
    else:
        nw = np.array([complex(np.interp(l_, waterm[0], waterm[1]), np.interp(l_, waterm[0], waterm[2]))
                       for l_ in lam])
    nrh = len(rh_run)
    gf = np.zeros(nrh)
    rrat = np.zeros(nrh)
    for ri in range(nrh):
        if rtype in ("simple", "trivial"):
            gf[ri] = params["rhDep"]["params"]["gf"][ri]
            rrat[ri] = 1.0 / gf[ri]
        elif rtype in ("ss", "su"):   # getHumidRefractiveIndex :512-531
            rminmaj = pp["rMinMaj"][b] if (rtype == "ss" and "rMinMaj" in pp) else pp["rmin0"][b][0]
            rminuse = _growth(params["rhDep"], rminmaj, rh[ri], rh)
            rrat[ri] = rminmaj / rminuse
            gf[ri] = 1.0 / rrat[ri]
        else:
            raise NotImplementedError("growth law '%s' is not implemented" % rtype)
    # volume mixing (dointegration.py:505); components follow the PSD (one RI
    # table is shared by every component, as the reference replicates it)
    fr = list(pp["fracs"][b])
    ncomp = len(fr)
    mix = nw[:, None, None] + (n0[:, None, :] - nw[:, None, None]) * (rrat[None, :, None] ** 3.0)
    if mix.shape[2] == 1 and ncomp > 1:
        mix = np.repeat(mix, ncomp, axis=2)
    rhop0v = params["rhop0"][b] if isinstance(params["rhop0"], list) else params["rhop0"]
    spec = {
        "lambda": lam, "grid": x, "grid_kind": GRID_X, "m": mix, "frac": np.array([fr]),
        "rhop": (rrat ** 3.0 * rhop0v + (1.0 - rrat ** 3.0) * 1000.0)[None, :], "rhop0": np.array([rhop0v]),
        "gf": gf, "ang": np.asarray(ang, np.float64), "rh0_index": rh.index(0.0) if 0.0 in rh else 0,
    }
    if ptype == "lognorm" and rtype == "su":
        # growth depends on the dry size: host-side weights of the grown modes
        spec["psd_kind"] = PSD_WEIGHTS
        spec["dgrid"] = dx
        spec["weights"] = _lognorm_weights(params, b, rh_run, x, dx, lam)[:, :, None, :, :]
        spec["psd_param"] = np.array([[[pp["r0"][b][k], pp["rmin0"][b][k], pp["rmax0"][b][k], pp["sigma"][b][k]]
                                       for k in range(ncomp)]])
        spec["rlow"] = np.array([pp["rmin0"][b][0]])
        spec["rup"] = np.array([pp["rmax0"][b][0]])
    elif ptype == "lognorm":
        spec["psd_kind"] = PSD_LOGNORM
        spec["dgrid"] = dx
        spec["psd_param"] = np.array([[[pp["r0"][b][k], pp["rmin0"][b][k], pp["rmax0"][b][k], pp["sigma"][b][k]]
                                       for k in range(ncomp)]])
        # growth of r0/rmax0 looks the RH up by value (particleparams.py:86)
        spec["gf_psd"] = np.array([params["rhDep"]["params"]["gf"][rh.index(v)] for v in rh_run])
        spec["rlow"] = np.array([pp["rmin0"][b][0]])
        spec["rup"] = np.array([pp["rmax0"][b][0]])
    elif ptype == "du":
        spec["psd_kind"] = PSD_POWER4
        spec["dgrid"] = _get_dr(x)
        spec["psd_param"] = np.array([[[pp["rMinMaj"][b][k], pp["rMaxMaj"][b][k], 0.0, 0.0]
                                       for k in range(ncomp)]])
        spec["gf_psd"] = np.ones(nrh)
        spec["rlow"] = np.array([pp["rMinMaj"][b][-1]])
        spec["rup"] = np.array([pp["rMaxMaj"][b][-1]])
    elif ptype == "ss":
        spec["psd_kind"] = PSD_WEIGHTS
        spec["dgrid"] = _get_dr(x)
        spec["weights"] = _ss_weights(params, b, rh_run if not trivial else rh[:1], x, lam)[:, :, None, None, :]
        spec["rlow"] = np.array([pp["rMinMaj"][b]])
        spec["rup"] = np.array([pp["rMaxMaj"][b]])
    else:
        raise ValueError("unknown psd type %s" % ptype)
    spec["trivial_nrh"] = len(rh) if trivial else 0
    return spec


def run_table(params, mlist, waterm, ang=None, lambdas=None, precision=_native.GBMIE_PLAIN_FP64, n_gsf=0,
              device=0):
    """The (bin x wavelength x RH) table of a reference particle definition.

    Returns {key: array} with the reference file's variables and
    non-legacy dimensions: scatkeys (bin, wavelength, rh, ang), scalar keys
    (bin, wavelength, rh), pback (bin, wavelength, rh, p), and the
    wavelength-independent keys (bin, rh) holding the last wavelength's
    values as the reference file does; with n_gsf > 0 also 'pmom'
    (bin, wavelength, rh, p, m) as written by rungsf (pygeos mode).
    """
    ang = angmie() if ang is None else np.asarray(ang, np.float64)
    pp = params["psd"]["params"]
    nbin = len(pp["r0"]) if params["psd"]["type"] == "lognorm" else len(pp["rMinMaj"])
    parts = []
    for b in range(nbin):
        spec = bin_spec(params, b, mlist, waterm, ang, lambdas)
        plan = TablePlan(spec, precision=precision, n_gsf=n_gsf, device=device)
        plan.run()
        res = plan.results()
        plan.close()
        nrh_full = spec["trivial_nrh"]
        if nrh_full:   # 'trivial': every RH copies the dry values (copyDryValues)
            res = {k: np.repeat(v, nrh_full, axis=2) for k, v in res.items()}
        parts.append(res)
    out = {k: np.concatenate([p_[k] for p_ in parts], axis=0) for k in parts[0]}
    for k in NLSCALARKEYS:
        out[k] = out.pop("nl_" + k)[:, -1, :]
    return out


def load_particle(path, data_dir=None):
    """particleparams.getPPJSON (particleparams.py:18-56): the JSON dict, the
    refractive-index tables (wavelength in metres) and the water table."""
    with open(path) as fp:
        params = json.load(fp)
    base = data_dir or os.getcwd()
    ri = params["ri"]

    def rel(p):
        return p if os.path.isabs(p) else os.path.join(base, p)
    if ri["format"] == "gads":
        mlist = [np.loadtxt(rel(p), skiprows=17, max_rows=61, comments=None, unpack=True, usecols=[1, 8, 9])
                 for p in ri["path"]]
    elif ri["format"] in ("csv", "wsv"):
        mlist = [np.loadtxt(rel(p), unpack=True, delimiter="," if ri["format"] == "csv" else None)
                 for p in ri["path"]]
    else:
        raise ValueError("refractive index format %s not supported" % ri["format"])
    for t in mlist:
        t[0] *= 1e-6
    waterm = np.loadtxt(rel("data/refrac.water.txt"), skiprows=13, unpack=True, usecols=[0, 1, 2])
    waterm[0] *= 1e-6
    return params, mlist, waterm


def fun(partID0, datatype="json", oppfx=".", oppclassic=False, data_dir=None, n_gsf=0,
        precision=_native.GBMIE_PLAIN_FP64, write=True, version=2):
    """dointegration.fun (:672): computes the table and, like the reference,
    writes oppfx/optics_<id>.nomom.nc4 (legacy layout: .nomom.legacy.nc4)
    as a NetCDF classic file (lutfile); returns the table dict."""
    if datatype != "json":
        raise ValueError("bad datatype: %s" % datatype)
    params, mlist, waterm = load_particle(partID0, data_dir)
    if params.get("mode", "mie") != "mie":
        raise NotImplementedError("kernel (GRASP) mode is not a Mie table")
    out = run_table(params, mlist, waterm, n_gsf=n_gsf, precision=precision)
    if write:
        from . import lutfile
        path = os.path.join(oppfx, lutfile.optics_filename(partID0, oppclassic))
        lutfile.write_optics(path, out, params["rh"], mlist[0][0], angmie(), oppclassic, version=version)
    return out
