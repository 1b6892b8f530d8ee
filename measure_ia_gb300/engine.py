"""Host driver of the CUDA pair counter.

``PairCounter`` holds one measurement configuration (binning, jackknife,
precision) and runs ``mia_measure`` on device-resident catalogues.  PyTorch
supplies the device buffers and the stream; all arithmetic happens in the
CUDA library.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from . import binning as B

_CONTEXTS: dict[int, C.c_void_p] = {}


def context(device: int) -> C.c_void_p:
    lib = L.load()
    if device not in _CONTEXTS:
        h = C.c_void_p()
        rc = lib.mia_create(device, C.byref(h))
        if rc != L.MIA_OK:
            raise L.MiaError(rc, "mia_create failed")
        _CONTEXTS[device] = h
    return _CONTEXTS[device]


def profile_pairs(device: int, n_slots: int) -> None:
    """Record CUDA events around the next pair-kernel launches of this device's
    context (a ring of n_slots; 0 switches recording off)."""
    lib = L.load()
    ctx = context(device)
    rc = lib.mia_profile_pairs(ctx, int(n_slots))
    if rc != L.MIA_OK:
        raise L.MiaError(rc, lib.mia_last_error(ctx).decode())


def pair_kernel_ms(device: int, n: int) -> list:
    """Durations (ms) of the last n recorded pair-kernel launches, oldest first."""
    lib = L.load()
    ctx = context(device)
    buf = (C.c_float * max(int(n), 1))()
    got = C.c_int()
    rc = lib.mia_profile_read(ctx, buf, int(n), C.byref(got))
    if rc != L.MIA_OK:
        raise L.MiaError(rc, lib.mia_last_error(ctx).decode())
    return [float(buf[i]) for i in range(got.value)]


def jackknife_cross_cov(real_a, real_b=None, device: int = 0, stream=None):
    """Jackknife covariance and std of two datasets' realisations (n_real x
    n_bins each; ``real_b=None`` = ``real_a`` with itself), computed on the
    device by ``mia_jackknife_cross_cov`` (measure_jackknife.py:485-571).
    Inputs are CUDA tensors (rows may be strided) or host arrays; returns
    (cov, std) as CUDA tensors."""
    import torch
    dev = torch.device("cuda", device)

    def dev2d(x):
        t = x if isinstance(x, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64))
        t = t.to(device=dev, dtype=torch.float64)
        if t.dim() != 2 or t.stride(1) != 1:
            t = t.reshape(t.shape[0], -1).contiguous()
        return t

    a = dev2d(real_a)
    b = a if real_b is None else dev2d(real_b)
    if a.shape != b.shape:
        raise ValueError(f"realisation shapes differ: {tuple(a.shape)} vs {tuple(b.shape)}")
    n_real, n_bins = a.shape
    cov = torch.empty((n_bins, n_bins), dtype=torch.float64, device=dev)
    std = torch.empty(n_bins, dtype=torch.float64, device=dev)
    st = stream if stream is not None else torch.cuda.current_stream(dev)
    lib = L.load()
    ctx = context(device)
    rc = lib.mia_jackknife_cross_cov(ctx, int(n_real), int(n_bins), C.c_void_p(a.data_ptr()), int(a.stride(0)),
                                     C.c_void_p(b.data_ptr()), int(b.stride(0)), C.c_void_p(cov.data_ptr()),
                                     C.c_void_p(std.data_ptr()), C.c_void_p(st.cuda_stream))
    if rc != L.MIA_OK:
        raise L.MiaError(rc, lib.mia_last_error(ctx).decode())
    return cov, std


def _dptr(ptr):
    return C.cast(ptr, C.POINTER(C.c_double))


@dataclass
class Measurement:
    """Products of one measurement, as host arrays (layout of the reference's outputs)."""
    kind: str
    n_r: int
    n_p: int
    J: int
    arrays: dict
    npairs: np.ndarray          # (1+J, n_r, n_p) int64: [0] all pairs, [1+i] region i
    stats: dict

    def __getitem__(self, k):
        return self.arrays[k]


class PairCounter:
    """One configuration of the box pair count (w or multipoles)."""

    def __init__(self, kind, *, boxsize, r_bins, r_min, r_max, p_bins, los=2, l_subboxes=0, precision="fp64",
                 membership="tree", ellipticity="distortion", want_variance=False, volume=None, rp_cut=0.0,
                 cell_size=0.0, shapes_per_unit=0, cell_refine=0, cell_size_los=0.0, cell_refine_los=0, device=0):
        if kind not in ("w", "m"):
            raise ValueError(kind)
        self._args = dict(boxsize=boxsize, r_bins=r_bins, r_min=r_min, r_max=r_max, p_bins=p_bins, los=los,
                          l_subboxes=l_subboxes, precision=precision, membership=membership, ellipticity=ellipticity,
                          want_variance=want_variance, volume=volume, rp_cut=rp_cut, device=device)
        self.knobs = dict(cell_size=cell_size, cell_refine=cell_refine, shapes_per_unit=shapes_per_unit,
                          cell_size_los=cell_size_los, cell_refine_los=cell_refine_los)
        self.membership = membership
        self.kind = kind
        self.device = device
        self.n_r = len(r_bins) - 1
        self.n_p = len(p_bins) - 1
        if self.n_r > L.MAX_BINS_R or self.n_p > L.MAX_BINS_P:
            raise ValueError(f"at most {L.MAX_BINS_R} r bins and {L.MAX_BINS_P} pi/mu bins are supported")
        self.J = l_subboxes ** 3 if l_subboxes > 0 else 0
        self._r_edges = np.ascontiguousarray(r_bins, dtype=np.float64)
        self._p_edges = np.ascontiguousarray(p_bins, dtype=np.float64)
        qt = B.r_table(kind, self._r_edges, r_min, r_max, self.n_r, membership, rp_cut)
        pt = B.pi_table(self._p_edges, self.n_p) if kind == "w" else B.mu_table(self._p_edges, self.n_p)
        self.q_table, self.p_table = qt, pt
        self._qb = np.ascontiguousarray(qt.breaks, dtype=np.float64)
        self._qn = np.ascontiguousarray(qt.bins, dtype=np.int32)
        self._pb = np.ascontiguousarray(pt.breaks, dtype=np.float64)
        self._pn = np.ascontiguousarray(pt.bins, dtype=np.int32)
        cfg = L.Config()
        cfg.kind = L.MIA_KIND_W if kind == "w" else L.MIA_KIND_MULTIPOLES
        cfg.membership = L.MIA_TREE if membership == "tree" else L.MIA_BRUTE
        cfg.precision = L.MIA_MIXED if precision == "mixed" else L.MIA_FP64
        cfg.los = int(los)
        cfg.l_subboxes = int(l_subboxes)
        cfg.ellipticity = L.MIA_DISTORTION if ellipticity == "distortion" else L.MIA_ELLIPTICITY
        cfg.want_variance = int(bool(want_variance))
        cfg.n_r, cfg.n_p = self.n_r, self.n_p
        cfg.n_qbreak, cfg.n_pbreak = len(self._qb), len(self._pb)
        cfg.shapes_per_unit = int(shapes_per_unit)
        cfg.cell_refine = int(cell_refine)
        cfg.boxsize = float(boxsize)
        cfg.volume = float(boxsize ** 3 if volume is None else volume)
        cfg.r_min, cfg.r_max = float(r_min), float(r_max)
        cfg.rp_cut = float(rp_cut)
        cfg.cell_size = float(cell_size)
        cfg.cell_size_los = float(cell_size_los)
        cfg.cell_refine_los = int(cell_refine_los)
        cfg.r_edges = self._r_edges.ctypes.data_as(C.POINTER(C.c_double))
        cfg.p_edges = self._p_edges.ctypes.data_as(C.POINTER(C.c_double))
        cfg.q_break = self._qb.ctypes.data_as(C.POINTER(C.c_double))
        cfg.q_bin = self._qn.ctypes.data_as(C.POINTER(C.c_int))
        cfg.p_break = self._pb.ctypes.data_as(C.POINTER(C.c_double))
        cfg.p_bin = self._pn.ctypes.data_as(C.POINTER(C.c_int))
        self.cfg = cfg
        self.precision = precision
        lib = L.load()
        lay = L.Layout()
        rc = lib.mia_output_layout(C.byref(cfg), C.byref(lay))
        if rc != L.MIA_OK:
            raise L.MiaError(rc, "invalid configuration")
        self.layout = lay

    # ---- sizes ---------------------------------------------------------------
    def workspace_bytes(self, n_pos, n_shape):
        lib = L.load()
        n = C.c_size_t()
        rc = lib.mia_workspace_size(C.byref(self.cfg), int(n_pos), int(n_shape), C.byref(n))
        if rc != L.MIA_OK:
            raise L.MiaError(rc, "invalid configuration")
        return n.value

    def allocate(self, n_pos, n_shape):
        """Device buffers for one run: (workspace, out, npairs) torch tensors."""
        import torch
        dev = torch.device("cuda", self.device)
        ws = torch.empty(self.workspace_bytes(n_pos, n_shape), dtype=torch.uint8, device=dev)
        out = torch.empty(self.layout.total, dtype=torch.float64, device=dev)
        npairs = torch.empty((1 + self.J) * self.n_r * self.n_p, dtype=torch.int64, device=dev)
        return ws, out, npairs

    # ---- run -----------------------------------------------------------------
    def run(self, cat, buffers, stream=None):
        """Enqueue mia_measure on device tensors and wait for it.

        ``cat``: dict with CUDA float64 contiguous tensors 'Position' (N,3),
        'weight', 'Position_shape_sample' (M,3), 'Axis_Direction' (M,2), 'q',
        'weight_shape_sample'."""
        import torch
        ws, out, npairs = buffers
        c = L.Catalog()
        c.position = cat["Position"].data_ptr()
        c.weight = cat["weight"].data_ptr()
        c.position_shape = cat["Position_shape_sample"].data_ptr()
        c.axis_direction = cat["Axis_Direction"].data_ptr()
        c.q = cat["q"].data_ptr()
        c.weight_shape = cat["weight_shape_sample"].data_ptr()
        c.n_pos = cat["Position"].shape[0]
        c.n_shape = cat["Position_shape_sample"].shape[0]
        r = L.Result()
        r.out = out.data_ptr()
        r.npairs = npairs.data_ptr()
        if stream is None:
            stream = torch.cuda.current_stream(self.device)
        lib = L.load()
        ctx = context(self.device)
        rc = lib.mia_measure(ctx, C.byref(self.cfg), C.byref(c), C.c_void_p(ws.data_ptr()), ws.numel(),
                             C.byref(r), C.c_void_p(stream.cuda_stream))
        if rc != L.MIA_OK:
            msg = lib.mia_last_error(ctx).decode()
            if rc in (L.MIA_ERR_ARG, L.MIA_ERR_RANGE):
                raise ValueError(msg)
            raise L.MiaError(rc, msg)

    def fetch(self, buffers):
        """Copy the products to the host and slice them by the output layout."""
        _, out, npairs = buffers
        o = out.cpu().numpy()
        cnt = npairs.cpu().numpy().reshape(1 + self.J, self.n_r, self.n_p)
        lay = self.layout
        nb, nr, npp, J = self.n_r * self.n_p, self.n_r, self.n_p, self.J

        a = {}
        a["DD_all"] = o[lay.dd:lay.dd + (1 + J) * nb].reshape(1 + J, nr, npp)
        a["Splus_all"] = o[lay.splus:lay.splus + (1 + J) * nb].reshape(1 + J, nr, npp)
        for k in ("scross", "variance", "rr", "xi_gp", "xi_gx", "xi_gg", "splusd", "scrossd", "sigmasq"):
            off = getattr(lay, k)
            a[k] = o[off:off + nb].reshape(nr, npp)
        a["DD"] = a["DD_all"][0]
        for k in ("rr_jk", "xi_gp_jk", "splusd_jk", "xi_gg_jk", "dd_jk"):
            off = getattr(lay, k)
            a[k] = o[off:off + J * nb].reshape(J, nr, npp)
        for k in ("proj_gp", "proj_gg", "mean_gp", "std_gp", "mean_gg", "std_gg"):
            off = getattr(lay, k)
            a[k] = o[off:off + nr]
        for k in ("proj_gp_jk", "proj_gg_jk"):
            off = getattr(lay, k)
            a[k] = o[off:off + J * nr].reshape(J, nr)
        for k in ("cov_gp", "cov_gg"):
            off = getattr(lay, k)
            a[k] = o[off:off + nr * nr].reshape(nr, nr)
        a["R"] = o[lay.R]
        a["R_jk"] = o[lay.R_jk:lay.R_jk + J]
        a["npos_jk"] = o[lay.npos_jk:lay.npos_jk + J]
        a["nshape_jk"] = o[lay.nshape_jk:lay.nshape_jk + J]
        st = o[lay.stats:lay.stats + 8]
        stats = dict(n_pos=int(st[0]), n_shape=int(st[1]), binned_pairs=int(st[2]), edge_pairs=int(st[3]),
                     work_units=int(st[4]))
        return Measurement(self.kind, nr, npp, J, a, cnt, stats)

    def with_knobs(self, **knobs):
        """The same measurement with other launch knobs (identical results)."""
        return PairCounter(self.kind, **self._args, **{**self.knobs, **knobs})

    def search_ranges(self):
        r = max(float(self._args["r_max"]), float(self._r_edges[-1]))
        if self.kind == "w":
            return r, max(abs(float(self._p_edges[0])), abs(float(self._p_edges[-1])))
        return r, r

    def tuned(self, dcat, cache=True, log=None):
        """A counter with autotuned launch knobs for this catalogue (see autotune.py)."""
        import torch
        from . import autotune
        rp, rl = self.search_ranges()
        key = None
        if cache:
            key = autotune.workload_key(self.kind, self.precision, dcat["Position"].shape[0],
                                        dcat["Position_shape_sample"].shape[0], float(self._args["boxsize"]),
                                        self.n_r, self.n_p, rp, rl, int(self._args["l_subboxes"]), self.membership,
                                        torch.cuda.get_device_name(self.device))
        best = autotune.tune(lambda **k: self.with_knobs(**k), dcat, rp, rl, key=key, log=log)
        return self.with_knobs(**{k: best[k] for k in autotune.KNOBS})

    def to_device(self, cat):
        import torch
        dev = torch.device("cuda", self.device)
        out = {}
        for k in ("Position", "weight", "Position_shape_sample", "Axis_Direction", "q", "weight_shape_sample"):
            v = cat[k]
            if isinstance(v, torch.Tensor):
                out[k] = v.to(device=dev, dtype=torch.float64).contiguous()
            else:
                out[k] = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).to(dev)
        return out

    def measure(self, cat, stream=None):
        """Convenience: copy host arrays (numpy) or use device tensors, run, fetch."""
        import torch
        dev = torch.device("cuda", self.device)
        dcat = {}
        for k in ("Position", "weight", "Position_shape_sample", "Axis_Direction", "q", "weight_shape_sample"):
            v = cat[k]
            if isinstance(v, torch.Tensor):
                t = v.to(device=dev, dtype=torch.float64).contiguous()
            else:
                t = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).to(dev)
            dcat[k] = t
        bufs = self.allocate(dcat["Position"].shape[0], dcat["Position_shape_sample"].shape[0])
        self.run(dcat, bufs, stream)
        return self.fetch(bufs)


class BatchCounter:
    """Many catalogues measured with one configuration in one persistent
    pair-kernel launch (``mia_batch_*``).  ``prepare`` uploads tables once;
    ``enqueue`` only enqueues memsets and kernels, so ``capture`` can record it
    in a CUDA graph that ``replay`` re-runs."""

    def __init__(self, counter: PairCounter, dcats):
        import torch
        self.pc = counter
        self.dcats = list(dcats)
        self.n = len(self.dcats)
        lib = L.load()
        n_pos = (C.c_int64 * self.n)(*[d["Position"].shape[0] for d in self.dcats])
        n_shape = (C.c_int64 * self.n)(*[d["Position_shape_sample"].shape[0] for d in self.dcats])
        nbytes = C.c_size_t()
        rc = lib.mia_batch_workspace_size(C.byref(counter.cfg), self.n, n_pos, n_shape, C.byref(nbytes))
        if rc != L.MIA_OK:
            raise L.MiaError(rc, "invalid batch configuration")
        dev = torch.device("cuda", counter.device)
        self.ws = torch.empty(nbytes.value, dtype=torch.uint8, device=dev)
        self.outs = [torch.empty(counter.layout.total, dtype=torch.float64, device=dev) for _ in range(self.n)]
        self.cnts = [torch.empty((1 + counter.J) * counter.n_r * counter.n_p, dtype=torch.int64, device=dev)
                     for _ in range(self.n)]
        self.cats = (L.Catalog * self.n)()
        self.res = (L.Result * self.n)()
        for i, d in enumerate(self.dcats):
            c = self.cats[i]
            c.position, c.weight = d["Position"].data_ptr(), d["weight"].data_ptr()
            c.position_shape = d["Position_shape_sample"].data_ptr()
            c.axis_direction, c.q = d["Axis_Direction"].data_ptr(), d["q"].data_ptr()
            c.weight_shape = d["weight_shape_sample"].data_ptr()
            c.n_pos, c.n_shape = d["Position"].shape[0], d["Position_shape_sample"].shape[0]
            self.res[i].out = self.outs[i].data_ptr()
            self.res[i].npairs = self.cnts[i].data_ptr()
        self.graph = None

    def tuned(self, cache=True, log=None):
        """A batch of the same catalogues with launch knobs autotuned on the
        batch as a whole (the time of one batched run per candidate; cached per
        batch shape): the best geometry for many small catalogues differs from
        that of the largest one."""
        import torch
        from . import autotune
        pc = self.pc
        rp, rl = pc.search_ranges()
        key = None
        if cache:
            sizes = [(d["Position"].shape[0], d["Position_shape_sample"].shape[0]) for d in self.dcats]
            key = autotune.workload_key(pc.kind, pc.precision, sum(a for a, _ in sizes), sum(b for _, b in sizes),
                                        float(pc._args["boxsize"]), pc.n_r, pc.n_p, rp, rl,
                                        int(pc._args["l_subboxes"]), pc.membership,
                                        torch.cuda.get_device_name(pc.device)) + f"|batch{self.n}"

        def run(**knobs):
            b = BatchCounter(pc.with_knobs(**knobs), self.dcats)
            b.prepare()
            return lambda: (b.enqueue(), b.status())

        best = autotune.tune(pc.with_knobs, None, rp, rl, key=key, log=log, run=run)
        return BatchCounter(pc.with_knobs(**{k: best[k] for k in autotune.KNOBS}), self.dcats)

    def _call(self, name, stream):
        import torch
        lib = L.load()
        ctx = context(self.pc.device)
        if stream is None:
            stream = torch.cuda.current_stream(self.pc.device)
        rc = getattr(lib, name)(ctx, C.byref(self.pc.cfg), self.n, self.cats, C.c_void_p(self.ws.data_ptr()),
                                self.ws.numel(), self.res, C.c_void_p(stream.cuda_stream))
        if rc != L.MIA_OK:
            raise L.MiaError(rc, lib.mia_last_error(ctx).decode())

    def prepare(self, stream=None):
        self._call("mia_batch_prepare", stream)

    def enqueue(self, stream=None):
        self._call("mia_batch_enqueue", stream)

    def status(self, stream=None):
        import torch
        lib = L.load()
        ctx = context(self.pc.device)
        if stream is None:
            stream = torch.cuda.current_stream(self.pc.device)
        rc = lib.mia_batch_status(ctx, self.n, C.c_void_p(self.ws.data_ptr()), C.c_void_p(stream.cuda_stream))
        if rc != L.MIA_OK:
            msg = lib.mia_last_error(ctx).decode()
            if rc in (L.MIA_ERR_ARG, L.MIA_ERR_RANGE):
                raise ValueError(msg)
            raise L.MiaError(rc, msg)

    def run(self, stream=None):
        self.enqueue(stream)
        self.status(stream)

    def capture(self):
        """Record ``enqueue`` in a CUDA graph (after ``prepare``)."""
        self.graph = capture_batches([self])
        return self.graph

    def replay(self):
        self.graph.replay()
        self.status()

    def fetch(self, i):
        return self.pc.fetch((None, self.outs[i], self.cnts[i]))

    def realisations(self, i, key="gp"):
        """Catalogue i's jackknife realisations of w (or the multipoles),
        key 'gp' or 'gg': a (J, n_r) view of its device output."""
        off = getattr(self.pc.layout, f"proj_{key}_jk")
        J, nr = self.pc.J, self.pc.n_r
        return self.outs[i][off:off + J * nr].view(J, nr)

    def cross_covariance(self, i, j=None, key="gp"):
        """Jackknife covariance between catalogues i and j (i with itself
        when j is None) straight from the device outputs: (cov, std) CUDA
        tensors."""
        b = None if j is None else self.realisations(j, key)
        return jackknife_cross_cov(self.realisations(i, key), b, device=self.pc.device)

    def full_covariance(self, key="gp"):
        """Jackknife covariance of all catalogues' realisations at once, in one
        launch: an (n n_r) x (n n_r) matrix whose (i, j) block of n_r x n_r is
        cross_covariance(i, j), and std its diagonal's root."""
        import torch
        reals = torch.cat([self.realisations(i, key) for i in range(self.n)], dim=1)
        return jackknife_cross_cov(reals, None, device=self.pc.device)


def capture_batches(batches):
    """One CUDA graph that runs every batch's ``enqueue`` (e.g. the w and the
    multipole measurement of the same catalogues), after each batch's
    ``prepare``.  Replaying it re-measures all of them; ``status()`` of each
    batch then reports its errors."""
    import torch
    dev = batches[0].pc.device
    s = torch.cuda.Stream(dev)
    s.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(s):  # one eager run on the capture stream first
        for b in batches:
            b.enqueue(s)
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
        for b in batches:
            b.enqueue(s)
    return g
