"""Benchmark: binned pairs/s of the w_gg + w_g+ measurement with 27 jackknife
regions on the clustered 4M-galaxy catalogue, mixed form vs plain FP64 form.

Workload (seeded synthetic, no dataset download): Neyman-Scott catalogue in a
205 Mpc/h periodic box, 80,000 parents x Poisson(50) children with sigma = 1
Mpc/h Gaussian offsets (~4.0M positions), shape sample a random 1M subset,
axis towards the parent in the projected plane + von Mises(kappa=2) noise,
q ~ Beta(4,2), lognormal weights (sigma 0.3), plus 2,000 injected pairs on
bin edges.  Binning: 10 log r_p bins 0.1-20 Mpc/h, 8 linear Pi bins over
|Pi| <= 20 Mpc/h, LOS = z, 27 jackknife sub-boxes.

A step is one full measurement (cell-list build, pair counts with
jackknife parts, FP64 edge re-test, analytic RR, realisations, w, covariance)
on catalogues resident in HBM.  Binned pair: one (shape, position) pair that
lands in an (r_p, Pi) bin, counted once.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "binned pairs/s, wg+&wgg 4M gal 27JK: mixed vs FP64 GPU form at <=1e-6 rel err"
L_BOX = 205.0
R_BINS = np.logspace(-1, np.log10(20.0), 11)
PI_BINS = np.linspace(-20.0, 20.0, 9)
LANE_OPS_PER_PAIR = 32          # FP32 lane-ops per binned (r_p, Pi) pair (fixed recipe)
# FP64 operations per binned (r_p, Pi) pair in the plain FP64 form (fixed recipe):
# separations 3, squares 2, r_p^2 1, dot and crs against the axis 2 x 2, crs^2 1,
# the sin^2 phi guard 1, e / r_p^2 8 (a division counted as 8, its Newton steps),
# e cos 2phi 2, e sin 2phi 3, weight products 3.  (The reference's arccos route,
# with two square roots and two more divisions, runs only for near-collinear
# pairs.)
FP64_OPS_PER_PAIR = 28


def make_catalog(seed=2026, n_centres=80000, n_shape=1_000_000, n_edge=2000):
    from measure_ia_gb300.catalogs import neyman_scott_catalog, add_edge_pairs
    d = neyman_scott_catalog(n_centres, L_BOX, n_shape, seed, mean_children=50, sigma=1.0, kappa=2.0)
    return add_edge_pairs(d, L_BOX, seed + 1, R_BINS, PI_BINS, n_edge)


def world():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU reference (the oracle's restatement of the reference's tree + Pool path)
# ---------------------------------------------------------------------------

def cpu_sample_shapes(n_shape, n_sample, seed=7):
    """The seeded sample of shape indices the CPU reference measures."""
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n_shape, size=min(n_sample, n_shape), replace=False))


def cpu_reference(data, n_sample_shapes, processes):
    """The reference algorithm of measure_xi_w's multiprocessing backend
    (measure_w_box_jk.py:648-857) on a seeded sample of ``n_sample_shapes``
    shapes against all positions: labels and responsivity, the periodic
    position KD-tree built once (:764), then a fork Pool over chunks of
    shapes (:765-768) whose workers query that tree and bin the pairs with
    the reference's numpy sequence (:543-646).  The chunk is the reference's
    default 1000 shapes, or sample / processes when that is smaller, so that
    every process has work.  Returns (binned pairs, seconds, tree seconds,
    chunk)."""
    from oracle import ia_oracle as O
    b = O.Binning(boxsize=L_BOX, r_min=0.1, r_max=20.0, num_bins_r=10, num_bins_pi=8, pi_max=20.0)
    idx = cpu_sample_shapes(len(data["Position_shape_sample"]), n_sample_shapes)
    pos, spos = data["Position"], data["Position_shape_sample"][idx]
    axis_raw, q, ws = data["Axis_Direction"][idx], data["q"][idx], data["weight_shape_sample"][idx]
    chunk = max(1, min(1000, -(-len(idx) // processes)))
    t0 = time.perf_counter()
    axis = axis_raw / np.sqrt((axis_raw ** 2).sum(1))[:, None]
    e = O.ellipticity_size(q)
    R = O.responsivity(ws, e)
    lab_p = O.jackknife_labels(pos, b.L_0p5, 3)
    lab_s = O.jackknife_labels(spos, b.L_0p5, 3)
    c, t_tree = O.count_pairs_parallel("w", b, 2, pos, data["weight"], spos, axis, e, ws, R, lab_p, lab_s, 27,
                                       (0, len(idx)), processes=processes, chunk=chunk)
    dt = time.perf_counter() - t0
    return int(c.npairs.sum()), dt, t_tree, chunk


def cpu_model():
    """The host CPU's model name (for the record), or the machine type."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def cpu_line(data, pairs, secs, t_tree, chunk, n_sample, cores, steps=1):
    """The cpu_baseline object of a CPU-reference measurement."""
    v = pairs / secs
    n_shape = len(data["Position_shape_sample"])
    per_step, tree = secs / steps, t_tree / steps
    return {"value": v, "unit": "binned pairs/s", "cores": cores, "kind": "port",
            "sample": (f"{n_sample} seeded shapes x all {len(data['Position'])} positions per step, fork Pool of "
                       f"{cores} processes over chunks of {chunk} shapes, one position KD-tree build per step "
                       f"({tree:.2f} s of {per_step:.2f} s); {cpu_model()}"),
            "extrapolated_full_step_s": tree + (per_step - tree) * n_shape / n_sample,
            "note": ("the oracle's restatement of the reference's multiprocessing backend: scipy KD-tree "
                     "pre-selection, per-pair numpy binning (np.bincount where the reference uses the slower "
                     "np.add.at); extrapolated_full_step_s = one tree build plus the sample's pair time scaled "
                     "linearly to all shapes (labelled extrapolated: not run at full size)")}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def _errors(ref, got, keys):
    out = {}
    for k, name in keys:
        a, b = ref[k], got[k]
        out[name] = {"max_rel_per_bin": float(np.max(np.abs(b - a) / np.maximum(np.abs(a), 1e-300))),
                     "max_rel_to_vector_scale": float(np.max(np.abs(b - a)) / np.max(np.abs(a)))}
    return out


def time_counter(pc, dcat, steps, warmup, stream, ws=1, kernel_ms=None):
    """ms per step (CUDA events on the launching stream), per-step list, products.
    With a list ``kernel_ms``, the pair kernel's own launch durations in the
    timed steps (CUDA events the library records around that launch, on the
    same stream) are appended to it."""
    import torch
    from measure_ia_gb300 import engine
    n_pos, n_shape = dcat["Position"].shape[0], dcat["Position_shape_sample"].shape[0]
    bufs = pc.allocate(n_pos, n_shape)
    for _ in range(warmup):
        pc.run(dcat, bufs, stream)
    torch.cuda.synchronize()
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    if kernel_ms is not None:
        engine.profile_pairs(pc.device, steps)
    torch.cuda.synchronize()
    evs[0].record(stream)
    for i in range(steps):
        pc.run(dcat, bufs, stream)
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    ms = evs[0].elapsed_time(evs[-1]) / steps
    per = [evs[i].elapsed_time(evs[i + 1]) for i in range(steps)]
    if kernel_ms is not None:
        kernel_ms.extend(engine.pair_kernel_ms(pc.device, steps))
        engine.profile_pairs(pc.device, 0)
    return ms, per, pc.fetch(bufs)


def profiled_traffic(kernel="k_pairs", workload="config2_w_jk27"):
    """DRAM bytes (read + write) per launch of the pair kernel on this
    workload from one ncu capture, as recorded in profiles/traffic.json (the
    capture's command and summary are named there), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            rec = json.load(f).get(f"{kernel}/{workload}")
        return int(rec["dram_bytes_per_launch"]) if rec else None
    except (OSError, ValueError, KeyError, TypeError):
        return None


def aggregate_ranks(t_step, binned, ws, device="cuda"):
    """Whole-job figures of ws replicas: the slowest rank's step time and the
    binned pairs of all ranks together (one all-reduce each; no data path)."""
    if ws == 1:
        return t_step, binned
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(t_step)], dtype=torch.float64, device=device)
    b = torch.tensor([float(binned)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(b, op=dist.ReduceOp.SUM)
    return float(t.item()), int(round(b.item()))


def _pick(pc, dcat, args):
    """Launch knobs: pinned by --knobs, else autotuned on this catalogue
    (outside the timed region; cached per workload shape), else the defaults."""
    if args.knobs:
        v = args.knobs.split(",")
        k = dict(cell_size=float(v[0]), cell_refine=int(v[1]), shapes_per_unit=int(v[2]))
        if len(v) == 5:
            k.update(cell_size_los=float(v[3]), cell_refine_los=int(v[4]))
        return pc.with_knobs(**k)
    return pc if args.no_tune else pc.tuned(dcat)


def run_gpu(args, data, rank, ws, local):
    import torch
    from measure_ia_gb300.engine import PairCounter
    from measure_ia_gb300 import MeasureIABox

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    keys = ("Position", "weight", "Position_shape_sample", "Axis_Direction", "q", "weight_shape_sample")
    dcat = {k: torch.from_numpy(np.ascontiguousarray(data[k], dtype=np.float64)).to(dev) for k in keys}
    stream = torch.cuda.current_stream(dev)
    common = dict(boxsize=L_BOX, r_bins=R_BINS, r_min=0.1, r_max=20.0, p_bins=PI_BINS, l_subboxes=3, device=local)

    # launch knobs tuned on this catalogue (outside the timed region; cached per workload shape)
    pcm = _pick(PairCounter("w", precision="mixed", **common), dcat, args)
    knobs = dict(pcm.knobs)

    with ClockSampler(local) as clk:
        kms = []
        msm, per_m, mm = time_counter(pcm, dcat, args.steps, args.warmup, stream, ws, kernel_ms=kms)
    clocks = clk.summary()
    per_step = {"mixed": per_m}
    if args.only_mixed:
        m64, ms64 = mm, float("nan")
    else:
        pc64 = PairCounter("w", precision="fp64", **common, **knobs)
        ms64, per_step["fp64"], m64 = time_counter(pc64, dcat, max(1, min(args.steps, 2)), 1, stream, ws)

    binned = mm.stats["binned_pairs"]
    assert binned == m64.stats["binned_pairs"], "mixed and FP64 forms binned different pairs"
    counts_exact = bool(np.array_equal(mm.npairs, m64.npairs))
    err = _errors(m64, mm, (("proj_gp", "w_g+"), ("proj_gg", "w_gg"), ("cov_gp", "cov w_g+"), ("cov_gg", "cov w_gg")))
    err["w_g+ in jackknife sigma"] = float(np.max(np.abs(mm["proj_gp"] - m64["proj_gp"]) / m64["std_gp"]))

    # multipoles on the same catalogue (10 log r bins 0.1-20, 20 mu bins over [-1, 1]): rate and accuracy
    mult = None
    if not args.only_mixed and not args.no_multipoles:
        mc = dict(common, p_bins=np.linspace(-1.0, 1.0, 21))
        pmm = PairCounter("m", precision="mixed", **mc)
        pmm = _pick(pmm, dcat, args)
        mms, _, mmm = time_counter(pmm, dcat, 2, 1, stream, ws)
        pm64 = PairCounter("m", precision="fp64", **mc, **dict(pmm.knobs))
        mms64, _, mm64 = time_counter(pm64, dcat, 1, 0, stream, ws)
        mult = {"binned_pairs_per_step": mmm.stats["binned_pairs"],
                "mixed": {"value": mmm.stats["binned_pairs"] / (mms / 1e3), "ms_per_step": mms},
                "fp64": {"value": mm64.stats["binned_pairs"] / (mms64 / 1e3), "ms_per_step": mms64},
                "counts_bit_exact_mixed_vs_fp64": bool(np.array_equal(mmm.npairs, mm64.npairs)),
                "accuracy_mixed_vs_fp64": _errors(mm64, mmm, (("proj_gp", "multipole g+ (l=2)"),
                                                              ("proj_gg", "multipole gg (l=0)"),
                                                              ("cov_gp", "cov g+"), ("cov_gg", "cov gg")))}

    res = dict(binned=binned, ms=msm, kernel_ms=kms, ms64=ms64, clocks=clocks, counts_exact=counts_exact, err=err,
               stats=mm.stats, stats64=m64.stats, per_step=per_step, knobs=knobs, mult=mult,
               e2e_s=float("nan"), h2d=0, d2h=0)
    if args.no_e2e:
        return res
    # end to end through the public API with host buffers: H2D copies, the
    # measurement, D2H of every product and the dataset writes, every step.
    # The catalogue sits in pinned (page-locked) host memory, handed over as
    # numpy arrays like the reference's inputs.
    host = {}
    for k in keys:
        a = np.ascontiguousarray(data[k], dtype=np.float64)
        pinned = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
        pinned.numpy()[...] = a
        host[k] = pinned.numpy()
    host["LOS"] = 2
    import tempfile
    out_dir = tempfile.mkdtemp(prefix="mia_bench_")
    out_file = os.path.join(out_dir, "bench_output.hdf5")  # the products' HDF5 file, rewritten every step
    box = MeasureIABox(dict(host), out_file, None, None, [0.1, 20.0], 10, 8, 20.0, boxsize=L_BOX, num_nodes=2,
                       precision="mixed", device=local, autotune=not args.no_tune)
    box.measure_xi_w("bench", "both", 27, temp_file_path="/tmp")  # warm-up (tuner cache hit)
    e2e_steps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        box.measure_xi_w("bench", "both", 27, temp_file_path="/tmp")
    torch.cuda.synchronize()
    res["e2e_s"] = (time.perf_counter() - t0) / e2e_steps
    res["e2e_file_bytes"] = os.path.getsize(out_file)
    import shutil
    shutil.rmtree(out_dir, ignore_errors=True)
    res["h2d"] = sum(np.asarray(data[k]).nbytes for k in keys)
    res["d2h"] = pcm.layout.total * 8 + (1 + 27) * 80 * 8
    return res


def _time_graph(g, steps, warmup, stream):
    """ms per replay of a CUDA graph (CUDA events on the replay stream)."""
    import torch
    for _ in range(warmup):
        g.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        g.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def run_batch48(args, local):
    """48 catalogues (12 mass bins x 4 snapshots), sizes log-uniform in
    [5e3, 2e6] galaxies, each drawn with the clustered recipe (parents = N/50,
    shapes = N/4, independent seeds), w_gg + w_g+ and the multipoles (20 mu_r
    bins) of every catalogue with 27 jackknife regions: both measurements'
    batches (one persistent pair-kernel launch each) in one CUDA graph,
    against the same catalogues measured one after the other."""
    import torch
    from measure_ia_gb300.catalogs import neyman_scott_catalog
    from measure_ia_gb300.engine import BatchCounter, PairCounter, capture_batches
    rng = np.random.default_rng(48)
    sizes = np.exp(rng.uniform(np.log(5e3), np.log(2e6), 48))
    cats = [neyman_scott_catalog(max(2, int(n / 50)), L_BOX, max(100, int(n / 4)), 1000 + i, mean_children=50,
                                 sigma=1.0) for i, n in enumerate(sizes)]
    common = dict(boxsize=L_BOX, r_bins=R_BINS, r_min=0.1, r_max=20.0, l_subboxes=3, precision="mixed", device=local)
    pcs = {"w": PairCounter("w", p_bins=PI_BINS, **common),
           "m": PairCounter("m", p_bins=np.linspace(-1.0, 1.0, 21), **common)}
    dcats = [pcs["w"].to_device(c) for c in cats]
    if args.knobs or args.no_tune:
        pcs = {k: _pick(pc, dcats[0], args) for k, pc in pcs.items()}
    else:  # launch knobs tuned on the batch as a whole (outside the timed region; cached per batch shape)
        pcs = {k: BatchCounter(pc, dcats).tuned().pc for k, pc in pcs.items()}
    stream = torch.cuda.current_stream(local)
    out = {}
    batches = {}
    for kind, pc in pcs.items():
        # one after the other
        bufs = [pc.allocate(d["Position"].shape[0], d["Position_shape_sample"].shape[0]) for d in dcats]
        for d, b in zip(dcats, bufs):
            pc.run(d, b, stream)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for d, b in zip(dcats, bufs):
                pc.run(d, b, stream)
        torch.cuda.synchronize()
        seq_ms = (time.perf_counter() - t0) * 1e3 / args.steps
        singles = [pc.fetch(b) for b in bufs]
        binned = sum(m.stats["binned_pairs"] for m in singles)
        # batched, replayed from a CUDA graph of its own
        batch = BatchCounter(pc, dcats)
        batch.prepare()
        batch.run()
        batch.capture()
        ms = _time_graph(batch.graph, args.steps, args.warmup, stream)
        batch.status()
        same = all(np.array_equal(batch.fetch(i).npairs, singles[i].npairs) for i in range(len(dcats)))
        batches[kind] = batch
        out[kind] = {"value": binned / (ms / 1e3), "ms_per_step": ms, "one_after_the_other_ms": seq_ms,
                     "binned_pairs_per_step": binned, "counts_equal_to_one_by_one": bool(same), "knobs": pc.knobs}
        if args.fp64:  # the plain FP64 form, one catalogue after the other, one step
            pc64 = PairCounter(kind, **{**common, "precision": "fp64"},
                               p_bins=PI_BINS if kind == "w" else np.linspace(-1.0, 1.0, 21), **pc.knobs)
            ms64, exact, errs = 0.0, True, []
            for i, d in enumerate(dcats):
                t, _, m64 = time_counter(pc64, d, 1, 0, stream)
                ms64 += t
                exact &= bool(np.array_equal(m64.npairs, batch.fetch(i).npairs))
                errs.append(_errors(m64, batch.fetch(i), (("proj_gp", "g+"), ("proj_gg", "gg"))))
            worst = {k: max(e[k][q] for e in errs) for k in ("g+", "gg")
                     for q in ("max_rel_to_vector_scale",)}
            worst_bin = {k: max(e[k]["max_rel_per_bin"] for e in errs) for k in ("g+", "gg")}
            out[kind]["fp64_form"] = {"value": binned / (ms64 / 1e3), "ms_per_step": ms64,
                                      "counts_bit_exact_mixed_vs_fp64": exact,
                                      "max_rel_to_vector_scale_over_catalogues": worst,
                                      "max_rel_per_bin_over_catalogues": worst_bin}
    # both measurements of all 48 catalogues in one graph
    g = capture_batches([batches["w"], batches["m"]])
    ms_both = _time_graph(g, args.steps, args.warmup, stream)
    for b in batches.values():
        b.status()
    binned_both = out["w"]["binned_pairs_per_step"] + out["m"]["binned_pairs_per_step"]
    # every pairwise jackknife cross-covariance of the 48 catalogues' w_g+,
    # on the device from the batch outputs, against the oracle's numpy loop
    # on the host (on rank 0's host cores, for the record)
    batch = batches["w"]
    pairs = [(i, j) for i in range(len(dcats)) for j in range(i + 1, len(dcats))]
    for i, j in pairs[:4]:
        batch.cross_covariance(i, j)
    torch.cuda.synchronize()
    x0, x1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    x0.record(stream)
    res = [batch.cross_covariance(i, j) for i, j in pairs]
    x1.record(stream)
    torch.cuda.synchronize()
    xcov_ms = x0.elapsed_time(x1)
    from oracle import ia_oracle  # the checker and the host baseline
    reals = [batch.realisations(i).cpu().numpy() for i in range(len(dcats))]
    t0 = time.perf_counter()
    host = [ia_oracle.jackknife_cross_cov(reals[i], reals[j]) for i, j in pairs]
    host_ms = (time.perf_counter() - t0) * 1e3
    xcov_exact = all(np.array_equal(r[0].cpu().numpy(), h[0]) for r, h in zip(res, host))
    batch.full_covariance()  # all 48 catalogues in one launch (warm-up, then timed)
    x0.record(stream)
    full, _ = batch.full_covariance()
    x1.record(stream)
    torch.cuda.synchronize()
    full_ms = x0.elapsed_time(x1)
    nr = len(R_BINS) - 1
    full_exact = all(np.array_equal(full[i * nr:(i + 1) * nr, j * nr:(j + 1) * nr].cpu().numpy(), h[0])
                     for (i, j), h in zip(pairs, host))
    return {"metric": "binned pairs/s, 48 uneven catalogues, w_gg+w_g+ and multipoles 27JK in one CUDA graph, "
                      "mixed form",
            "value": binned_both / (ms_both / 1e3), "unit": "binned pairs/s", "ms_per_step": ms_both,
            "binned_pairs_per_step": binned_both, "w": out["w"], "multipoles": out["m"],
            "cross_covariances": {"pairs": len(pairs), "device_ms_pair_by_pair": xcov_ms,
                                  "device_ms_all_in_one_launch": full_ms, "host_oracle_ms": host_ms,
                                  "bit_exact_vs_oracle": bool(xcov_exact and full_exact)},
            "config": {"workload": "48 catalogues, sizes log-uniform 5e3-2e6 (config 3): w (10 x 8 bins) and "
                                   "multipoles (10 x 20 mu_r bins), 27 jackknife regions, one graph",
                       "n_positions_total": int(sum(len(c["Position"]) for c in cats)),
                       "n_shapes_total": int(sum(len(c["Position_shape_sample"]) for c in cats))}}


def run_small(args, local, which):
    """Config 0 (10,000 uniform galaxies, shape = position sample, weights 1,
    w only) or config 1 (clustered, 20,000 parents x Poisson(50), 200k shapes,
    w and multipoles with 20 mu bins over [-1, 1]); 27 jackknife regions;
    both forms, autotuned knobs."""
    import torch
    from measure_ia_gb300.catalogs import neyman_scott_catalog, uniform_catalog
    from measure_ia_gb300.engine import PairCounter
    if which == "config0":
        data = uniform_catalog(10000, L_BOX, 2024)
        kinds = [("w", PI_BINS)]
    else:
        data = neyman_scott_catalog(20000, L_BOX, 200_000, 11, mean_children=50, sigma=1.0, kappa=2.0)
        kinds = [("w", PI_BINS), ("m", np.linspace(-1.0, 1.0, 21))]
    stream = torch.cuda.current_stream(local)
    out = {}
    for kind, pbins in kinds:
        common = dict(boxsize=L_BOX, r_bins=R_BINS, r_min=0.1, r_max=20.0, p_bins=pbins, l_subboxes=3, device=local)
        pcm = PairCounter(kind, precision="mixed", **common)
        dcat = pcm.to_device(data)
        pcm = _pick(pcm, dcat, args)
        ms, _, mm = time_counter(pcm, dcat, args.steps, args.warmup, stream)
        pc64 = PairCounter(kind, precision="fp64", **common, **pcm.knobs)
        ms64, _, m64 = time_counter(pc64, dcat, max(1, min(args.steps, 3)), 1, stream)
        b = mm.stats["binned_pairs"]
        label = "w" if kind == "w" else "multipoles"
        out[label] = {"binned_pairs_per_step": b, "mixed": {"value": b / (ms / 1e3), "ms_per_step": ms},
                      "fp64": {"value": b / (ms64 / 1e3), "ms_per_step": ms64},
                      "counts_bit_exact_mixed_vs_fp64": bool(np.array_equal(mm.npairs, m64.npairs)),
                      "accuracy_mixed_vs_fp64": _errors(m64, mm, (("proj_gp", "g+"), ("proj_gg", "gg"))),
                      "knobs": pcm.knobs}
    first = out["w"]
    desc = ("10,000 uniform galaxies, w_gg+w_g+ 27JK (config 0)" if which == "config0" else
            "clustered 1M positions / 200k shapes, w and multipoles, 27JK (config 1)")
    return {"metric": f"binned pairs/s, {desc}, mixed form", "value": first["mixed"]["value"],
            "unit": "binned pairs/s", "ms_per_step": first["mixed"]["ms_per_step"], "forms": out,
            "config": {"workload": desc, "n_positions": int(len(data["Position"])),
                       "n_shapes": int(len(data["Position_shape_sample"]))}}


def run_large(args, local):
    """1000 Mpc/h box, 500,000 parents x Poisson(50) (sigma 1.5 Mpc/h),
    5M shapes, 15 log r_p bins 0.1-60, 20 Pi bins over |Pi| <= 60, 125
    jackknife regions, mixed form."""
    import torch
    from measure_ia_gb300.catalogs import neyman_scott_catalog
    from measure_ia_gb300.engine import PairCounter
    data = neyman_scott_catalog(500_000, 1000.0, 5_000_000, 4, mean_children=50, sigma=1.5)
    rb = np.logspace(-1, np.log10(60.0), 16)
    pb = np.linspace(-60.0, 60.0, 21)
    pc = PairCounter("w", boxsize=1000.0, r_bins=rb, r_min=0.1, r_max=60.0, p_bins=pb, l_subboxes=5,
                     precision="mixed", device=local)
    dcat = pc.to_device(data)
    pc = _pick(pc, dcat, args)
    ms, per, m = time_counter(pc, dcat, args.steps, max(1, args.warmup), torch.cuda.current_stream(local))
    fp64 = None
    if args.fp64:  # the plain FP64 form, one step
        pc64 = PairCounter("w", boxsize=1000.0, r_bins=rb, r_min=0.1, r_max=60.0, p_bins=pb, l_subboxes=5,
                           precision="fp64", device=local, **pc.knobs)
        ms64, _, m64 = time_counter(pc64, dcat, 1, 0, torch.cuda.current_stream(local))
        fp64 = {"value": m.stats["binned_pairs"] / (ms64 / 1e3), "ms_per_step": ms64,
                "counts_bit_exact_mixed_vs_fp64": bool(np.array_equal(m64.npairs, m.npairs)),
                "accuracy_mixed_vs_fp64": _errors(m64, m, (("proj_gp", "w_g+"), ("proj_gg", "w_gg")))}
    return {"metric": "binned pairs/s, w_gg+w_g+ 125JK, 1000 Mpc/h box, mixed form",
            "value": m.stats["binned_pairs"] / (ms / 1e3), "unit": "binned pairs/s", "ms_per_step": ms,
            "step_ms": per, "binned_pairs_per_step": m.stats["binned_pairs"],
            "edge_pairs_retested": m.stats.get("edge_pairs"), "knobs": pc.knobs, "fp64_form": fp64,
            "config": {"workload": "25M positions / 5M shapes, 1000 Mpc/h, 15x20 bins, 125 jackknife (config 4)",
                       "n_positions": int(len(data["Position"])), "n_shapes": int(len(data["Position_shape_sample"]))}}


# ---------------------------------------------------------------------------
# lightcone workload (MeasureIALightcone.measure_xi_w, clusters estimator)
# ---------------------------------------------------------------------------

LC_DESC = ("lightcone survey 40 x 25 deg (1000 deg^2), 0.1 < z < 0.5: 200k clustered galaxies (100k shapes), "
           "1M randoms; w_gg + w_g+ (clusters estimator: S+D, S+R, RD, RR counters), 10 log r_p bins 0.1-60 Mpc, "
           "20 Pi bins |Pi| < 60 Mpc, 50 jackknife patches (10 x 5 RA/DEC grid)")
# Fixed FP32 recipe per binned lightcone pair, lane-ops (an FMA is one), in the
# box path's terms: separation 3, projection by chi cos(dec) and chi 2,
# r_p^2 2, range tests 3, r bin 3, Pi bin 2 = 15 counts only; the shape
# terms add cos/sin 2phi of the separation 5, the combination with the
# shape's angle 4, weight products and scaling 4 = 28.  Multipoles: r^2 +1,
# range tests -1, mu bin +2 (17 and 30).
LC_LANE_OPS = {("w", False): 15, ("w", True): 28, ("m", False): 17, ("m", True): 30}


def lightcone_catalogue(seed=77, n_par=10000, n_rand=1_000_000, n_shape=100_000):
    rng = np.random.default_rng(seed)
    cen = np.c_[rng.uniform(0, 40, n_par), rng.uniform(-12.5, 12.5, n_par), rng.uniform(0.1, 0.5, n_par)]
    kids = rng.poisson(20, n_par)
    par = np.repeat(np.arange(n_par), kids)
    n = len(par)
    data = {"RA": np.clip(cen[par, 0] + rng.normal(0, 0.05, n), 0, 40),
            "DEC": np.clip(cen[par, 1] + rng.normal(0, 0.05, n), -12.5, 12.5),
            "Redshift": np.clip(cen[par, 2] + rng.normal(0, 0.0005, n), 0.1, 0.5)}
    k = np.sort(rng.choice(n, min(n_shape, n), replace=False))
    eps, ang = rng.uniform(0, 0.6, len(k)), rng.uniform(0, np.pi, len(k))
    data.update(RA_shape_sample=data["RA"][k], DEC_shape_sample=data["DEC"][k], Redshift_shape_sample=data["Redshift"][k],
                e1=eps * np.cos(2 * ang), e2=eps * np.sin(2 * ang))
    rnd = {"RA": rng.uniform(0, 40, n_rand), "DEC": rng.uniform(-12.5, 12.5, n_rand), "Redshift": rng.uniform(0.1, 0.5, n_rand)}
    grid = lambda ra, dec: (np.minimum(9, (ra / 4.0).astype(int)) * 5 + np.minimum(4, ((dec + 12.5) / 5.0).astype(int)))
    jk = {"position": grid(data["RA"], data["DEC"]), "shape": grid(data["RA_shape_sample"], data["DEC_shape_sample"]),
          "randoms": grid(rnd["RA"], rnd["DEC"])}
    return data, rnd, jk


def _lc_counters(data, rnd, jk, kind="w"):
    """The four counters of measure_xi_w (kind 'w') or measure_xi_multipoles
    (kind 'm') with 'clusters' and corr_type 'both', with their host inputs,
    as MeasureIALightcone prepares them."""
    from measure_ia_gb300 import MeasureIALightcone
    from measure_ia_gb300.cosmology import default_cosmology
    from measure_ia_gb300.lightcone import _Run
    lc = MeasureIALightcone(dict(data), dict(rnd), None, separation_limits=[0.1, 60.0], num_bins_r=10,
                            num_bins_pi=20, pi_max=60.0)
    r = dict(lc.randoms_data)
    r.update(RA_shape_sample=r["RA"], DEC_shape_sample=r["DEC"], Redshift_shape_sample=r["Redshift"],
             weight=np.ones(len(r["RA"])))
    r["weight_shape_sample"] = r["weight"]
    cosmo = default_cosmology()
    run = _Run(lc, kind, "clusters", "lc", "both", lc.data, r, lambda z: cosmo.comoving_radial_distance(1 / (1 + z)),
               0.7, False, None, None, None)
    out = []
    for name, pf, sf, shapes, pp, sp in (("S+D", "D", "D", True, "position", "shape"),
                                         ("S+R", "R", "D", True, "randoms", "shape"),
                                         ("RD", "D", "R", False, "position", "randoms"),
                                         ("RR", "R", "R", False, "randoms", "randoms")):
        sel = run._select(run._combo(pf, sf, shapes), None, shapes)
        lo, hi = int(np.min(jk[pp])), int(np.max(jk[pp]))
        pos, shp = run._samples(sel, shapes, np.asarray(jk[pp]) - lo, run._shape_labels(jk[sp], lo, hi))
        out.append((name, shapes, run._counter(shapes), pos, shp, hi - lo + 1))
    return lc, out


def measured_dgemm_tflops(device):
    import torch
    a = torch.randn(4096, 4096, dtype=torch.float64, device=device)
    b = torch.randn(4096, 4096, dtype=torch.float64, device=device)
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize(device)
    best = 1e9
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize(device)
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2 * 4096 ** 3 / best / 1e12


def lightcone_cpu(data, rnd, n_sample, processes=None):
    """The oracle's restatement of the reference's brute-force RR counter
    (measure_w_lightcone.py:216-343, a numpy loop over positions) on the
    first n_sample random positions against all random shapes: (binned
    pairs, seconds)."""
    from measure_ia_gb300.cosmology import default_cosmology
    from oracle import lightcone_oracle as LO
    cosmo = default_cosmology()
    b = LO.LcBinning(0.1, 60.0, 10, 20, 60.0)
    sel = {"RA": rnd["RA"][:n_sample], "DEC": rnd["DEC"][:n_sample], "Redshift": rnd["Redshift"][:n_sample],
           "weight": np.ones(n_sample), "RA_shape_sample": rnd["RA"], "DEC_shape_sample": rnd["DEC"],
           "Redshift_shape_sample": rnd["Redshift"], "weight_shape_sample": np.ones(len(rnd["RA"]))}
    t0 = time.perf_counter()
    _, _, dd = LO.pair_counts("w", False, b, sel, lambda a: cosmo.comoving_radial_distance(a), 0.7, False,
                              empty_to_one=False)
    secs = time.perf_counter() - t0
    return float(dd.sum()), secs   # unit weights: DD = pair counts


def run_lightcone(args, local):
    import torch
    data, rnd, jk = lightcone_catalogue(n_par=args.lc_parents, n_rand=args.lc_randoms,
                                        n_shape=min(100_000, args.lc_parents * 10))
    cores = 1
    cpu = None
    if not args.no_cpu:
        pairs, secs = lightcone_cpu(data, rnd, args.lc_cpu_sample)
        cpu = {"value": pairs / secs, "unit": "binned pairs/s", "cores": cores, "kind": "port",
               "sample": f"RR counter: first {args.lc_cpu_sample} random positions x all 1M random shapes, "
                         f"{secs:.1f} s (the reference's per-position numpy loop, one process)"}
    lc, counters = _lc_counters(data, rnd, jk)
    jobs = [(name, shapes, c, c.prepare(pos, shp, npatch)) for name, shapes, c, pos, shp, npatch in counters]
    stream = torch.cuda.current_stream(local)
    for _ in range(max(3, args.warmup)):
        for _, _, c, j in jobs:
            c.run(j, stream.cuda_stream)
    torch.cuda.synchronize(local)
    binned = {}
    for name, shapes, c, j in jobs:
        sums, counts = c.fetch(j)
        binned[name] = (shapes, int(counts[0].sum()))
    per, per_counter = [], {name: [] for name, *_ in jobs}
    with ClockSampler(local) as clk:
        torch.cuda.synchronize(local)
        for _ in range(args.steps):
            evs = []
            t0 = torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            for name, _, c, j in jobs:
                c.run(j, stream.cuda_stream)
                e = torch.cuda.Event(enable_timing=True)
                e.record(stream)
                evs.append((name, e))
            torch.cuda.synchronize(local)
            prev = t0
            for name, e in evs:
                per_counter[name].append(prev.elapsed_time(e))
                prev = e
            per.append(t0.elapsed_time(evs[-1][1]))
    ms = float(np.mean(per))
    total_binned = sum(v[1] for v in binned.values())
    # the multipole counters (r, mu_r bins: 10 log r bins 0.1-60, 20 mu_r bins), same catalogue
    _, mcounters = _lc_counters(data, rnd, jk, kind="m")
    mjobs = [(name, c, c.prepare(pos, shp, npatch)) for name, shapes, c, pos, shp, npatch in mcounters]
    for _ in range(max(3, args.warmup)):
        for _, c, j in mjobs:
            c.run(j, stream.cuda_stream)
    torch.cuda.synchronize(local)
    mbinned = sum(int(c.fetch(j)[1][0].sum()) for _, c, j in mjobs)
    mper = []
    for _ in range(args.steps):
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _, c, j in mjobs:
            c.run(j, stream.cuda_stream)
        t1.record(stream)
        torch.cuda.synchronize(local)
        mper.append(t0.elapsed_time(t1))
    del mjobs
    ops = sum(LC_LANE_OPS[("w", s)] * n for s, n in binned.values())
    props = torch.cuda.get_device_properties(local)
    peak = props.multi_processor_count * 128 * 2070e6 / 1e12
    achieved = ops / (ms / 1e3) / 1e12
    dgemm = measured_dgemm_tflops(local)
    # end to end through the public API: host arrays in, HDF5-layout products out (in memory)
    from measure_ia_gb300 import MeasureIALightcone
    e2e = []
    for _ in range(max(1, min(2, args.steps))):
        lc2 = MeasureIALightcone(dict(data), dict(rnd), None, separation_limits=[0.1, 60.0], num_bins_r=10,
                                 num_bins_pi=20, pi_max=60.0, num_nodes=2)
        torch.cuda.synchronize(local)
        t = time.perf_counter()
        lc2.measure_xi_w("clusters", "lc", "both", jk_patches={k: np.array(v) for k, v in jk.items()})
        torch.cuda.synchronize(local)
        e2e.append(time.perf_counter() - t)
    h2d = sum(j.h2d for *_, j in jobs)
    d2h = sum(j.out.numel() * 8 + j.cnt.numel() * 8 + 4 for *_, j in jobs)
    return {"metric": "binned pairs/s, lightcone w_gg+w_g+ (MeasureIALightcone.measure_xi_w, clusters, 50 patches)",
            "value": total_binned / (ms / 1e3), "unit": "binned pairs/s", "ms_per_step": ms, "step_ms": per,
            "counter_ms": {k: float(np.mean(v)) for k, v in per_counter.items()},
            "binned_pairs_per_step": {k: v[1] for k, v in binned.items()}, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "config": {"workload": LC_DESC, "n_positions": len(data["RA"]),
                                        "n_shapes": len(data["RA_shape_sample"]), "n_randoms": len(rnd["RA"]),
                                        "l2": "inputs larger than L2 (RR: 1M x 1M sorted samples, 8 x 8 MB arrays)"},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                         "traffic": None, "kernel": "k_lc_pairs (+ cell-list build), all four counters",
                         "note": "achieved = FP32 lane-ops of a fixed recipe per binned pair (15 counts only, 28 "
                                 "with shapes) x binned pairs / device time of the four counters; peak = nominal "
                                 "SMs x 128 x 2070 MHz (no FP32 figure in MEASURED_PEAKS.json).  The counters are "
                                 "issue-bound (RR ~71% issue, 13.0 warp instructions per binned pair: candidate tests, "
                                 "guard-band decisions, jackknife attribution), the shape terms FP64",
                         "fp64_dgemm_tflops": dgemm},
            "cpu_baseline": cpu,
            "e2e": {"value": total_binned / float(np.mean(e2e)), "unit": "binned pairs/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "seconds": e2e},
            "multipoles": {"value": mbinned / (float(np.mean(mper)) / 1e3), "unit": "binned pairs/s",
                           "ms_per_step": float(np.mean(mper)), "binned_pairs_per_step": mbinned,
                           "note": "the four counters of measure_xi_multipoles('clusters', 'both'), same catalogue"},
            "gpu_launches": 4 * 14 * args.steps,
            "clocks": clk.summary()}


def lightcone_reference_line(args):
    data, rnd, jk = lightcone_catalogue(n_par=args.lc_parents, n_rand=args.lc_randoms,
                                        n_shape=min(100_000, args.lc_parents * 10))
    res = [lightcone_cpu(data, rnd, args.lc_cpu_sample) for _ in range(args.steps)]
    pairs, secs = sum(r[0] for r in res), sum(r[1] for r in res)
    v = pairs / secs
    return {"metric": "binned pairs/s, lightcone w_gg+w_g+ (MeasureIALightcone.measure_xi_w, clusters, 50 patches)",
            "value": v, "unit": "binned pairs/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference", "config": {"workload": LC_DESC},
            "cpu_baseline": {"value": v, "unit": "binned pairs/s", "cores": 1, "kind": "port",
                             "sample": f"RR counter: first {args.lc_cpu_sample} random positions x all 1M random "
                                       "shapes per step"},
            "e2e": {"value": v, "unit": "binned pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------
# ingestion workload (ReadData.read_cat into GPU memory)
# ---------------------------------------------------------------------------

def run_ingest(args, local):
    """A config-2-sized catalogue (4M positions, 1M shapes: Position,
    weight, Position_shape_sample, Axis_Direction, q, weight_shape_sample)
    written as one HDF5 file, then read into GPU memory with
    ReadData.read_cat(device=...): file -> pinned buffer -> device.  The file
    is re-read every step (its pages may sit in the OS cache: 'data' says
    so); the host arm reads the same datasets into numpy arrays and copies
    them to the device from pageable memory."""
    import tempfile
    import torch
    from measure_ia_gb300 import hdf5
    from measure_ia_gb300.read_data import ReadData
    rng = np.random.default_rng(11)
    n_p, n_s = 4_000_000, 1_000_000
    cat = {"Snapshot_99/cat/Position": rng.uniform(0, 205, (n_p, 3)), "Snapshot_99/cat/weight": rng.uniform(size=n_p),
           "Snapshot_99/cat/Position_shape_sample": rng.uniform(0, 205, (n_s, 3)),
           "Snapshot_99/cat/Axis_Direction": rng.normal(size=(n_s, 2)), "Snapshot_99/cat/q": rng.uniform(size=n_s),
           "Snapshot_99/cat/weight_shape_sample": rng.uniform(size=n_s)}
    nbytes = sum(v.nbytes for v in cat.values())
    d = tempfile.mkdtemp(prefix="mia_ingest_")
    hdf5.write_file(os.path.join(d, "catalogue.hdf5"), cat)
    rd = ReadData("TNG300", "catalogue", 99, sub_group="cat", data_path=d)
    names = [k.split("/")[-1] for k in cat]
    dev = torch.device("cuda", local)

    def step_pinned():
        return [rd.read_cat(nm, device=dev) for nm in names]

    def step_host():
        return [torch.from_numpy(np.ascontiguousarray(rd.read_cat(nm))).to(dev) for nm in names]

    out = {}
    for label, fn in (("pinned", step_pinned), ("host", step_host)):
        for _ in range(max(1, args.warmup)):
            fn()
        torch.cuda.synchronize(dev)
        ts = []
        for _ in range(args.steps):
            t = time.perf_counter()
            got = fn()
            torch.cuda.synchronize(dev)
            ts.append(time.perf_counter() - t)
        out[label] = float(np.median(ts))
    ok = all(np.array_equal(g.cpu().numpy(), cat[k]) for g, k in zip(step_pinned(), cat))
    import shutil
    shutil.rmtree(d, ignore_errors=True)
    return {"metric": "catalogue ingestion GB/s, ReadData.read_cat into GPU memory (config-2 catalogue)",
            "value": nbytes / out["pinned"] / 1e9, "unit": "GB/s", "ms_per_step": 1e3 * out["pinned"],
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "config": {"workload": "4M positions + 1M shapes, 6 datasets, 176 MB in one HDF5 file (contiguous)",
                       "bytes": nbytes, "cache": "file re-read every step; pages may be in the OS page cache"},
            "bit_exact": bool(ok),
            "host_path": {"value": nbytes / out["host"] / 1e9, "unit": "GB/s", "ms_per_step": 1e3 * out["host"],
                          "note": "read into numpy, pageable copy to the device"},
            "e2e": {"value": nbytes / out["pinned"] / 1e9, "unit": "GB/s", "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=1600, help="seeded shapes in the CPU-baseline sample")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--only-mixed", action="store_true", help="time the mixed form only (profiling runs)")
    ap.add_argument("--no-tune", action="store_true", help="default launch knobs instead of the autotuner's")
    ap.add_argument("--knobs", default="", help="CELL,REFINE,SPU[,CELL_LOS,REFINE_LOS] launch knobs instead of tuning (profiling runs)")
    ap.add_argument("--no-multipoles", action="store_true", help="skip the multipole rate and accuracy report")
    ap.add_argument("--fp64", action="store_true", help="batch48 / large: also time the plain FP64 form")
    ap.add_argument("--lc-cpu-sample", type=int, default=60, help="lightcone: random positions in the CPU sample")
    ap.add_argument("--lc-randoms", type=int, default=1_000_000, help="lightcone: randoms (profiling runs)")
    ap.add_argument("--lc-parents", type=int, default=10000, help="lightcone: clustered parents (profiling runs)")
    ap.add_argument("--workload", default="config2",
                    choices=["config2", "batch48", "large", "config0", "config1", "lightcone", "ingest"],
                    help="config2 = the headline line; batch48 and large print their own lines")
    ap.add_argument("--centres", type=int, default=80000, help="Neyman-Scott parents (profiling runs)")
    ap.add_argument("--shapes", type=int, default=1_000_000, help="shape-sample size (profiling runs)")
    args = ap.parse_args()
    rank, ws, local = world()
    if args.impl == "reference" and rank != 0:
        return  # the CPU reference arm runs on rank 0 only
    if args.impl == "reference" and args.workload == "lightcone":
        print(json.dumps(lightcone_reference_line(args)))
        return
    if args.workload != "config2":
        import torch
        torch.cuda.set_device(local)
        if args.workload == "batch48":
            line = run_batch48(args, local)
        elif args.workload == "lightcone":
            line = run_lightcone(args, local)
        elif args.workload == "ingest":
            line = run_ingest(args, local)
        elif args.workload == "large":
            line = run_large(args, local)
        else:
            line = run_small(args, local, args.workload)
        line.update({"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                     "data": "synthetic"})
        if rank == 0:
            print(json.dumps(line))
        return
    data = make_catalog(n_centres=args.centres, n_shape=args.shapes)
    n_pos, n_shape = len(data["Position"]), len(data["Position_shape_sample"])
    config = {"workload": "clustered 4M positions / 1M shapes, w_gg+w_g+, 27 jackknife regions (config 2)",
              "n_positions": n_pos, "n_shapes": n_shape, "boxsize": L_BOX, "r_p_bins": "10 log 0.1-20",
              "pi_bins": "8 linear |Pi|<=20", "membership": "kd-tree (r_min < r_p <= r_max)",
              "l2": "inputs larger than L2 (sorted working set > 129 MB)"}
    cores = os.cpu_count() or 1

    if args.impl == "reference":
        results = []
        for _ in range(args.warmup):  # the same per-step work on a smaller sample
            cpu_reference(data, max(cores, args.cpu_sample // 8), cores)
        for _ in range(args.steps):
            results.append(cpu_reference(data, args.cpu_sample, cores))
        pairs = sum(r[0] for r in results)
        secs = sum(r[1] for r in results)
        cpu = cpu_line(data, pairs, secs, sum(r[2] for r in results), results[0][3], args.cpu_sample, cores,
                       args.steps)
        v = cpu["value"]
        line = {"metric": METRIC, "value": v, "unit": "binned pairs/s", "n_gpus": 0, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
                "config": config, "cpu_baseline": cpu,
                "e2e": {"value": v, "unit": "binned pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    # CPU baseline first, before any CUDA context exists (the pool forks)
    cpu = None
    if rank == 0 and not args.no_cpu:
        pairs, secs, t_tree, chunk = cpu_reference(data, args.cpu_sample, cores)
        cpu = cpu_line(data, pairs, secs, t_tree, chunk, args.cpu_sample, cores)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    r = run_gpu(args, data, rank, ws, local)
    t_step, binned_all = aggregate_ranks(r["ms"] / 1e3, r["binned"], ws)
    value = binned_all / t_step
    import torch
    props = torch.cuda.get_device_properties(local)
    peak = props.multi_processor_count * 128 * 2070e6 / 1e12
    # the pair kernel's own average launch time in the timed steps (its share
    # of the step is the rest of the device time: preparation, re-test, post)
    k_ms = float(np.mean(r["kernel_ms"])) if r["kernel_ms"] else r["ms"]
    achieved = LANE_OPS_PER_PAIR * r["binned"] / (k_ms / 1e3) / 1e12
    traffic = profiled_traffic()
    fp64_form = {"value": r["binned"] / (r["ms64"] / 1e3), "ms_per_step": r["ms64"]}
    if np.isfinite(r["ms64"]):
        # the FP64 form against the FP64 pipe: a fixed recipe of FP64 operations
        # per binned pair over the step, and cuBLAS DGEMM's FMA rate measured here
        dgemm = measured_dgemm_tflops(local)
        fp64_ops = FP64_OPS_PER_PAIR * r["binned"] / (r["ms64"] / 1e3) / 1e12
        fp64_form.update({"fp64_ops_per_binned_pair": FP64_OPS_PER_PAIR, "achieved_fp64_tops": fp64_ops,
                          "dgemm_tflops_measured": dgemm, "dgemm_fma_rate_tops": dgemm / 2,
                          "frac_of_dgemm_fma_rate": fp64_ops / (dgemm / 2),
                          "note": "plain FP64 form: an FP32 range test, then the reference's FP64 separations "
                                  "and bin decisions for the survivors with all lanes busy, the S+D terms from "
                                  "a short FP64 chain; ops per pair from the fixed recipe in bench.py (a "
                                  "division counted as 8)"})
    if rank != 0:
        return
    launches_per_step = 22  # prep 16 (prep 2, scans 9, scatter 2, responsivity sums 1, work units 2), work prefix 1, pairs 1, edge re-test 1, fixed-point sums 1, post 1, status 1
    line = {
        "metric": METRIC, "value": value, "unit": "binned pairs/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 pair arithmetic, f64 edge re-test and reductions", "data": "synthetic",
        "config": config,
        "fp64_form": fp64_form,
        "mixed_over_fp64": r["ms64"] / r["ms"],
        "accuracy_mixed_vs_fp64": r["err"], "counts_bit_exact_mixed_vs_fp64": r["counts_exact"],
        "binned_pairs_per_step": r["binned"], "edge_pairs_retested": r["stats"]["edge_pairs"],
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "k_pairs (persistent pair kernel)", "kernel_ms": k_ms,
                     "kernel_share_of_step": k_ms / r["ms"],
                     "note": "achieved = 32 FP32 lane-ops per binned pair / the pair kernel's mean launch time "
                             "(CUDA events on the launching stream, timed steps); peak = nominal SMs x 128 x "
                             "2070 MHz (no FP32 figure in MEASURED_PEAKS.json); traffic = DRAM bytes per "
                             "launch from one ncu capture (profiles/traffic.json)"},
        "cpu_baseline": cpu,
        "e2e": {"value": r["binned"] / r["e2e_s"], "unit": "binned pairs/s", "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"], "hdf5_file_bytes": r.get("e2e_file_bytes"),
                "note": "MeasureIABox.measure_xi_w from pinned host arrays: H2D of the catalogue, the measurement, "
                        "D2H of every product and the HDF5 output file written, every step"},
        "gpu_launches": launches_per_step * args.steps,
        "step_ms": r["per_step"],
        "launch_knobs": r["knobs"],
        "multipoles": r["mult"],
        "clocks": r["clocks"],
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
