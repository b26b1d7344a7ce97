"""Benchmark of the CENTRE entropy hot path on GB300.

One step = the whole hot path over one synthetic trajectory already resident
in HBM: histogram discretisation of every bond/angle/torsion, 1-D counts and
entropies, 2-D joint counts and entropies of every DOF pair, MI, MIE sums and
the MIST spanning tree.  Workload: a 1000-atom chain (999 bonds, 998 angles,
997 torsions = 2994 DOFs, 4,480,521 pairs), 100,000 frames, 50 bins per DOF,
10 convergence steps, ML estimator, Jacobian on.  The metric is MI pairs/s.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--form tc|atomic|auto]
    python bench.py --impl reference      # the CPU implementation of the path

Multi-GPU (torchrun): every rank runs its own independent trajectory
(replicas; no collective on the data path); value = all ranks' pairs / the
slowest rank's time.

Besides the contract keys, the line carries `roofline` (the dominant
pair-count kernel against its own hardware ceiling: increments/s of the
shared-memory histogram against one conflict-free shared-atomic wavefront of
32 increments per SM and cycle, or FP8 one-hot FLOP/s for the tensor-core
form), `tc_roofline` (the tensor-core form's own run against the FP8 rate),
`discretize_roofline` (HBM GB/s) and `parity` (each count form's S2 against
the oracle on a sampled sub-system, and the two forms against each other on
every pair).
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

METRIC = "MI pairs/s"
UNIT = "pairs/s"
NBINS = 50      # set from the workload in main()
NSTEPS = 10


SM_COUNT = 152
# Conflict-free shared-memory atomics: one wavefront of 32 increments per SM
# and cycle is the ceiling of the histogram form (the data pipe retires one
# wavefront per cycle).
INCREMENTS_PER_SM_CYCLE = 32
# DRAM bytes (read + written) of one pair-count launch of the default
# workload (2994 DOFs, 100,000 frames, 50 bins, 10 steps, ML), from an ncu
# capture of that launch: gpu__time_duration and the two dram__bytes
# metrics, one pass (profiles/pairs_hist_chain1000_dram.md).  Algorithmic
# bytes of the launch: the 0.30 GB bin matrix read once and 0.36 GB of
# 64-bit moments written.
PAIR_HIST_TRAFFIC = 1.10e9 + 0.354e9
PAIR_HIST_TRAFFIC_NOTE = ("dram__bytes_read.sum 1.10 GB + dram__bytes_write.sum 0.354 GB of one "
                          "ncu capture of this launch on this workload (algorithmic: 0.30 GB "
                          "of bins read once + 0.36 GB of moments written)")


def slowest_rank(value, dist, device="cpu"):
    """The largest of every rank's value (a step time): the job runs as fast
    as its slowest replica."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, step_s, world):
    """Whole-job units per second: every rank processed its own units in a
    step that lasted `step_s` (the slowest rank's)."""
    return world * units_per_rank / step_s


def workload(name):
    from centre_gb300.synth import WORKLOADS
    w = dict(WORKLOADS[name])
    na = w["natoms"]
    w["ndof"] = 3 * na - 6
    w["npairs"] = w["ndof"] * (w["ndof"] - 1) // 2
    return w


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
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
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------- CPU port --
def subsystem(tr, kper):
    """The first `kper` bonds, angles and torsions of a chain: a complete
    sub-system of the workload (same frames, distributions and couplings)
    with 3*kper DOFs.  Returns the blocks and the DOFs' indices in the full
    system (bonds, then angles, then torsions)."""
    blocks, glob, base = [], [], 0
    for typ, blk in tr.blocks():
        k = min(kper, len(blk))
        blocks.append((typ, np.ascontiguousarray(blk[:k])))
        glob += list(range(base, base + k))
        base += len(blk)
    return blocks, np.array(glob, np.int64)


def cpu_pass(orc, blocks, nthreads):
    """One complete pass of the path on the CPU oracle (the C restatement of
    the reference, OpenMP over DOFs and pairs): discretise every DOF, 1-D
    entropies, joint entropies of every pair i<j, MI, MIE-2 sums and the MIST
    tree of every step.  Returns (seconds, pairs, S2 [pairs][steps])."""
    t0 = time.perf_counter()
    bins_l, ext_l, types_l = [], [], []
    for typ, blk in blocks:
        b, e = orc.discretize(typ, blk, [NBINS], nthreads=nthreads)
        bins_l.append(b)
        ext_l.append(e)
        types_l += [typ] * len(blk)
    bins, ext = np.concatenate(bins_l), np.concatenate(ext_l)
    types = np.array(types_l, np.uint8)
    n = len(types)
    s1 = orc.entropy1d(types, bins, ext, NSTEPS, [NBINS], [0], True, nthreads=nthreads)
    ii, jj = np.triu_indices(n, 1)
    pairs = np.stack([ii, jj], 1).astype(np.uint32)
    s2 = orc.entropy2d(pairs, types, bins, ext, NSTEPS, [NBINS], [0], True, nthreads=nthreads)
    s1 = s1[:, 0, 0, :]
    s2 = s2[:, 0, 0, :]
    mi = s1[ii] + s1[jj] - s2
    mie = s1.sum(axis=0) - mi.sum(axis=0)
    mist = np.empty(NSTEPS)
    for t in range(NSTEPS):
        tree = orc.mst(n, pairs[:, 0], pairs[:, 1], mi[:, t])
        mist[t] = s1[:, t].sum() - mi[tree, t].sum()
    dt = time.perf_counter() - t0
    assert np.all(np.isfinite(mie)) and np.all(np.isfinite(mist))
    return dt, len(pairs), s2


def oracle_check(orc, tr, kper, s2_by_form, ndof, nthreads):
    """The GPU's joint entropies (one array per count form, all pairs of the
    full system) against the oracle on every pair of a sub-system."""
    blocks, glob = subsystem(tr, kper)
    dt, npairs, s2o = cpu_pass(orc, blocks, nthreads)
    ii, jj = np.triu_indices(len(glob), 1)
    gi, gj = glob[ii], glob[jj]
    idx = gi * ndof - gi * (gi + 1) // 2 + (gj - gi - 1)
    out = {}
    for form, s2g in s2_by_form.items():
        g = s2g[idx]
        err = np.abs(g - s2o)
        big = np.abs(s2o) > 1e-6
        rel = err[big] / np.abs(s2o[big]) if big.any() else np.zeros(1)
        out[form] = {"pairs": int(npairs), "pair_steps": int(err.size),
                     # relative error where |S2| > 1e-6; absolute error
                     # everywhere (joint entropies with Jacobian terms can sit
                     # within rounding of zero)
                     "max_rel_error": float(rel.max()), "max_abs_error": float(err.max()),
                     "within_test_tolerance": bool(np.all(err <= 1e-9 * np.abs(s2o) + 1e-13))}
    return dt, npairs, out


# ------------------------------------------------------------ our GPU arm --
def run_ours(args):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from centre_gb300.api import Context, make_params
    from centre_gb300.synth import chain_trajectory

    w = workload(args.workload)
    tr = chain_trajectory(w["natoms"], w["nframes"], seed=1000 + rank, coupling=w["coupling"])
    dev = torch.device("cuda", local)
    blocks = [(typ, torch.from_numpy(blk).to(dev)) for typ, blk in tr.blocks()]
    ndof = sum(b.shape[0] for _, b in blocks)
    n = tr.nframes
    npairs = ndof * (ndof - 1) // 2
    types = torch.tensor(sum([[t] * b.shape[0] for t, b in blocks], []), dtype=torch.uint8,
                         device=dev)
    bins = torch.empty((ndof, 1, n), dtype=torch.uint8, device=dev)
    ext = torch.empty((ndof, 4), dtype=torch.float64, device=dev)
    s1 = torch.empty((ndof, 1, 1, NSTEPS), dtype=torch.float64, device=dev)
    s2 = torch.empty((npairs, 1, 1, NSTEPS), dtype=torch.float64, device=dev)
    mi = torch.empty_like(s2)
    form = {"auto": 0, "atomic": 1, "tc": 2}[args.form]

    ctx = Context(local)
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)

    def step(f, s2buf=s2):
        p = make_params(n, NSTEPS, [NBINS], [0], True, counts_form=f)
        off = 0
        for typ, data in blocks:
            k = data.shape[0]
            ctx.discretize_dev(typ, data, [NBINS], bins[off:off + k], ext[off:off + k])
            off += k
        ctx.entropy1d_dev(p, types, bins, ext, s1)
        ctx.entropy2d_dev(p, types, bins, ext, s2buf)
        return ctx.score_dev(p, types, s1, s2buf, None, True, mi)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()

    for _ in range(args.warmup):
        step(form)
    barrier()
    ctx.enable_timing(True)
    launches0 = ctx.launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(stream)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            res = step(form)
        ev1.record(stream)
        barrier()
        wall = time.perf_counter() - t0
    ms = ev0.elapsed_time(ev1)
    # score_dev synchronises internally for the tree, so the device clock
    # and the host clock agree up to launch gaps; report the larger
    step_ms = max(ms, wall * 1e3) / args.steps
    launches = ctx.launches - launches0
    t_disc, n_disc = ctx.timer(0)
    t_1d, n_1d = ctx.timer(1)
    t_pairs, n_pairs = ctx.timer(2)
    t_score, n_score = ctx.timer(3)
    ctx.enable_timing(False)

    step_ms = slowest_rank(step_ms, dist, dev)
    value = job_throughput(npairs, step_ms / 1e3, world)

    hbm, bf16, src = peaks()
    fp8_peak = 2.0 * bf16
    used = NSTEPS * (n // NSTEPS)
    flops_per_launch = 2.0 * used * NBINS * NBINS * npairs   # one-hot contraction
    incr_per_launch = float(used) * npairs                    # histogram increments
    pair_ms = t_pairs / max(n_pairs, 1)
    disc_ms = t_disc / max(n_disc, 1)
    # discretise launches cover one DOF block each; bytes per launch averaged
    disc_bytes = 5.0 * ndof * n / 3
    uses_tc = form == 2 or (form == 0 and NBINS > 217)
    clocks = clk.summary()
    mhz = (clocks or {}).get("sm_mhz") or 2070.0

    def tc_line(ms):
        a = flops_per_launch / (ms / 1e3) / 1e12
        return {"bound": "tensor", "kernel": "pairs_tc_kernel (FP8 one-hot O^T O)",
                "achieved": a, "peak": fp8_peak, "unit": "TFLOP/s", "frac": a / fp8_peak,
                "traffic": None,
                "note": f"2*N*B^2 flops per pair (B={NBINS} real bins, N={used} frames), "
                        f"{npairs} pairs per launch; peak = 2 x {src} bf16 {bf16:.0f} TF/s "
                        "(no FP8 figure is measured: the dense FP8 rate is taken as twice "
                        "the bf16 one)"}

    if uses_tc:
        roofline = tc_line(pair_ms)
    else:
        a = incr_per_launch / (pair_ms / 1e3)
        peak = SM_COUNT * mhz * 1e6 * INCREMENTS_PER_SM_CYCLE
        roofline = {"bound": "shared-memory atomics", "kernel": "pairs_hist_kernel<4,4>",
                    "achieved": a, "peak": peak, "unit": "increments/s", "frac": a / peak,
                    "traffic": PAIR_HIST_TRAFFIC,
                    "note": f"N={used} increments per pair (one per frame), {npairs} pairs "
                            f"per launch; ceiling = {SM_COUNT} SMs x {mhz:.0f} MHz (sampled "
                            f"SM clock) x {INCREMENTS_PER_SM_CYCLE} increments (one "
                            "conflict-free shared-atomic wavefront per SM and cycle), derived "
                            "from the hardware (no shared-memory figure is measured)"}
        if PAIR_HIST_TRAFFIC_NOTE:
            roofline["traffic_note"] = PAIR_HIST_TRAFFIC_NOTE
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded BAT chain, float32)",
        "config": {"workload": f"chain{w['natoms']}: {ndof} DOFs, {n} frames, {NBINS} bins, "
                               f"{NSTEPS} steps, ML, all {npairs} pairs, MIE-2 + MIST",
                   "counts_form": args.form, "l2": "inputs (1.2 GB) larger than L2",
                   "parallelism": f"replicas x{world}"},
        "mist_wall_ms": t_score / max(args.steps, 1),
        "kernel_ms_per_step": {"discretize": t_disc / args.steps, "counts1d": t_1d / args.steps,
                               "pair_counts": t_pairs / args.steps,
                               "score_mst": t_score / args.steps},
        "roofline": roofline,
        "discretize_roofline": {"bound": "hbm", "achieved": disc_bytes / (disc_ms / 1e3) / 1e9,
                                "peak": hbm, "unit": "GB/s",
                                "frac": disc_bytes / (disc_ms / 1e3) / 1e9 / hbm,
                                "note": f"5 B per DOF-frame; {src} peak"},
        "gpu_launches": launches,
    }
    s2_by_form = {("tc" if uses_tc else "histogram"): s2}
    # end to end right after the device-resident steps, before the other
    # count form's comparison run (seconds of tensor-core work); it leaves
    # the device outputs above untouched
    if not args.no_e2e:
        out["e2e"] = run_e2e(ctx, tr, args, w, world, dist, dev)
    if args.compare_atomic:
        # both count forms on the same data (the metric compares them): the
        # one the timed steps did not use runs one more (warm, timed) step
        # into its own S2 buffer, so that each form's output is checked
        other = 1 if uses_tc else 2
        s2_other = torch.empty_like(s2)
        try:
            step(other, s2_other)
            barrier()
            ctx.enable_timing(True)
            step(other, s2_other)
            to, no_ = ctx.timer(2)
            ctx.enable_timing(False)
            torch.cuda.synchronize(dev)
            other_ms = to / max(no_, 1)
            tc_ms, at_ms = (pair_ms, other_ms) if uses_tc else (other_ms, pair_ms)
            out["tc_pair_counts_ms"] = tc_ms
            out["atomic_pair_counts_ms"] = at_ms
            out["tc_over_atomic"] = at_ms / tc_ms if tc_ms > 0 else None
            out["tc_roofline"] = tc_line(tc_ms)
            s2_by_form["histogram" if uses_tc else "tc"] = s2_other
            # the two forms produce the same integers, hence the same
            # entropies to the last bit, on every pair and step
            out["forms_bit_identical"] = bool(torch.equal(s2, s2_other))
        except Exception as e:   # e.g. a bin count the tensor-core form does not take
            ctx.enable_timing(False)
            out["tc_pair_counts_ms"] = None
            out["tc_note"] = str(e)
    if clocks:
        out["clocks"] = clocks

    if world == 1 and not args.no_screen:
        # the learned screen on the 5000-atom chain (two timed steps after
        # one warm-up), carried as a sub-record of the default line
        out["screen5000"], _ = screen_measure(5000, 2, 1, local)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        oracle.build(with_ref=False)
        orc = oracle.Oracle()
        cores = os.cpu_count()
        host = {k: v.reshape(npairs, NSTEPS).cpu().numpy() for k, v in s2_by_form.items()}
        dt, np_sub, checks = oracle_check(orc, tr, args.cpu_kper, host, ndof, cores)
        out["cpu_baseline"] = {
            "value": np_sub / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"one complete pass (discretise, 1-D, all {np_sub} pairs, MI, MIE-2, "
                      f"MIST of every step) over the sub-system of the first {args.cpu_kper} "
                      f"bonds, angles and torsions ({3 * args.cpu_kper} DOFs, {n} frames, "
                      f"{NBINS} bins, {NSTEPS} steps): {dt:.2f} s on {cores} host threads",
            "extrapolated": False}
        out["parity"] = {"vs_oracle": checks,
                         "forms_bit_identical_all_pairs": out.get("forms_bit_identical")}
    ctx.close()
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def run_e2e(ctx, tr, args, w, world, dist, dev):
    """The same step through the host-pointer C ABI (the stage-by-stage
    drop-in): pinned host BAT in, bins/entropies/MI back to host."""
    import torch
    from centre_gb300.api import make_params
    n = tr.nframes
    blocks = []
    for typ, blk in tr.blocks():
        h = torch.from_numpy(blk).pin_memory()
        blocks.append((typ, h.numpy()))
    ndof = sum(b.shape[0] for _, b in blocks)
    npairs = ndof * (ndof - 1) // 2
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    bins = pin((ndof, 1, n), torch.uint8)
    ext = pin((ndof, 4), torch.float64)
    s1 = pin((ndof, 1, 1, NSTEPS), torch.float64)
    s2 = pin((npairs, 1, 1, NSTEPS), torch.float64)
    mi = pin((npairs, 1, 1, NSTEPS), torch.float64)
    types = np.array(sum([[t] * b.shape[0] for t, b in blocks], []), np.uint8)
    form = {"auto": 0, "atomic": 1, "tc": 2}[args.form]
    p = make_params(n, NSTEPS, [NBINS], [0], True, counts_form=form)

    stage_s = {"discretize": 0.0, "entropy1d": 0.0, "entropy2d": 0.0, "score": 0.0}

    def step():
        # each stage call returns with its outputs in host memory
        t = time.perf_counter()
        off = 0
        for typ, data in blocks:
            k = data.shape[0]
            ctx.discretize(typ, data, [NBINS], bins_out=bins[off:off + k], ext_out=ext[off:off + k])
            off += k
        t1 = time.perf_counter()
        ctx.entropy1d(p, types, bins, ext, out=s1)
        t2 = time.perf_counter()
        ctx.entropy2d(p, types, bins, ext, out=s2)
        t3 = time.perf_counter()
        res = ctx.score(p, types, s1, s2, None, True, True, mi_out=mi)
        t4 = time.perf_counter()
        for key, a, b in (("discretize", t, t1), ("entropy1d", t1, t2), ("entropy2d", t2, t3),
                          ("score", t3, t4)):
            stage_s[key] += b - a
        return res

    for _ in range(2):      # warm-up (first-touch of the pinned buffers)
        step()
    for key in stage_s:
        stage_s[key] = 0.0
    steps = max(1, min(args.steps, 3))
    if dist:
        dist.barrier()
    with ClockSampler(dev.index if dev.index is not None else 0) as clk:
        t0 = time.perf_counter()
        for _ in range(steps):
            step()
        dt = (time.perf_counter() - t0) / steps
    dt = slowest_rank(dt, dist, dev)
    h2d = sum(b.nbytes for _, b in blocks) + 2 * bins.nbytes + 2 * ext.nbytes + s1.nbytes \
        + s2.nbytes + 3 * types.nbytes
    d2h = bins.nbytes + ext.nbytes + s1.nbytes + s2.nbytes + mi.nbytes
    out = {"value": world * npairs / dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": dt * 1e3, "steps": steps,
           "stage_wall_ms": {k: v / steps * 1e3 for k, v in stage_s.items()}}
    clocks = clk.summary()
    if clocks:
        out["clocks"] = clocks
    return out


# ----------------------------------------------- batched trajectories ----
def run_batch(args):
    """Many trajectories of uneven length scored in one captured graph
    (centre_gpu_entropy_batch_dev): 1-D and all-pairs joint entropies at 10
    frame prefixes, MI, MIE-2 and MIST sums per trajectory.  Metric: MI pairs
    (summed over trajectories) per second of the whole batch."""
    import torch
    from centre_gb300.api import Context, make_params
    from centre_gb300.synth import BATCHES, batch_specs, chain_blocks_torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    b = BATCHES[args.workload]
    nb, nsteps = b["nbins"], b["nsteps"]
    ctx = Context(local)
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    specs = batch_specs(args.workload, seed=1 + rank)
    systems, host_bins = [], []
    tot_pairs = tot_incr = 0
    with torch.cuda.stream(stream):
        for natoms, nframes, seed in specs:
            blocks = chain_blocks_torch(natoms, nframes, seed, dev, coupling=b["coupling"])
            ndof = sum(x.shape[0] for _, x in blocks)
            npairs = ndof * (ndof - 1) // 2
            bins = torch.empty((ndof, 1, nframes), dtype=torch.uint8, device=dev)
            ext = torch.empty((ndof, 4), dtype=torch.float64, device=dev)
            off = 0
            for typ, data in blocks:
                k = data.shape[0]
                ctx.discretize_dev(typ, data, [nb], bins[off:off + k], ext[off:off + k])
                off += k
            del blocks
            types = torch.tensor(sum([[t] * k for t, k in ((1, natoms - 1), (2, natoms - 2),
                                                          (3, natoms - 3))], []),
                                 dtype=torch.uint8, device=dev)
            systems.append({"types": types, "bins": bins, "ext": ext,
                            "s1": torch.empty((ndof, nsteps), dtype=torch.float64, device=dev),
                            "s2": torch.empty((npairs, nsteps), dtype=torch.float64, device=dev),
                            "mi": torch.empty((npairs, nsteps), dtype=torch.float64, device=dev)})
            tot_pairs += npairs
            tot_incr += npairs * nsteps * (nframes // nsteps)
    torch.cuda.synchronize(dev)
    p = make_params(0, nsteps, [nb], [0], True)

    def step():
        return ctx.entropy_batch_dev(p, systems)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()

    t0 = time.perf_counter()
    step()           # tunes the count kernel and captures the graph
    first_ms = (time.perf_counter() - t0) * 1e3
    for _ in range(args.warmup):
        step()
    barrier()
    ctx.enable_timing(True)
    launches0 = ctx.launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(stream)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            res = step()
        ev1.record(stream)
        barrier()
        wall = time.perf_counter() - t0
    ms = ev0.elapsed_time(ev1)
    step_ms = max(ms, wall * 1e3) / args.steps
    launches = ctx.launches - launches0
    graph_ms, ngraph = ctx.timer(2)
    ctx.enable_timing(False)
    step_ms = slowest_rank(step_ms, dist, dev)
    # the count kernel's increments (one per pair and frame used) over the
    # whole graph's time, against the shared-atomic ceiling of the histogram
    # form: the graph also holds the 1-D, finalize and scoring kernels, so
    # this is a lower bound on the count kernel's own fraction
    clocks = clk.summary()
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    achieved = tot_incr / (step_ms / 1e3)
    ceiling = SM_COUNT * mhz * 1e6 * INCREMENTS_PER_SM_CYCLE
    ndofs = [3 * a - 6 for a, _, _ in specs]
    out = {
        "metric": METRIC, "value": world * tot_pairs / (step_ms / 1e3), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded BAT chains drawn on the device, float32)",
        "config": {"workload": f"{args.workload}: {len(specs)} chains, {min(ndofs)}..{max(ndofs)} "
                               f"DOFs, {min(f for _, f, _ in specs)}..{max(f for _, f, _ in specs)} "
                               f"frames, {nb} bins, {nsteps} prefixes, ML, all pairs "
                               f"({tot_pairs} in total), MIE-2 + MIST per chain",
                   "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"},
        "first_call_ms": first_ms,
        "increments_per_s": tot_incr / (step_ms / 1e3),
        "graph_ms_per_step": graph_ms / max(ngraph, 1),
        "roofline": {"bound": "shared-memory atomics", "kernel": "pairs_hist_batch_kernel "
                     "(time of the whole batch graph)", "achieved": achieved, "peak": ceiling,
                     "unit": "increments/s", "frac": achieved / ceiling, "traffic": None,
                     "note": f"one increment per pair and frame used ({tot_incr} per step); "
                             f"ceiling = {SM_COUNT} SMs x {mhz:.0f} MHz (sampled SM clock) x "
                             f"{INCREMENTS_PER_SM_CYCLE} increments (one conflict-free "
                             "shared-atomic wavefront per SM and cycle), derived from the "
                             "hardware"},
        "gpu_launches": launches,
    }
    if clocks:
        out["clocks"] = clocks
    if not args.no_e2e:
        # host bins in (pinned), the batch, the sums back on the host
        pins = [torch.empty(sd["bins"].shape, dtype=torch.uint8, pin_memory=True)
                for sd in systems]
        for h, sd in zip(pins, systems):
            h.copy_(sd["bins"])
        torch.cuda.synchronize(dev)
        steps = max(1, min(args.steps, 3))
        t0 = time.perf_counter()
        for _ in range(steps):
            with torch.cuda.stream(stream):
                for h, sd in zip(pins, systems):
                    sd["bins"].copy_(h, non_blocking=True)
            step()
        dt = (time.perf_counter() - t0) / steps
        G = nsteps
        out["e2e"] = {"value": world * tot_pairs / dt, "unit": UNIT,
                      "h2d_bytes_per_step": int(sum(h.numel() for h in pins)),
                      "d2h_bytes_per_step": int(len(systems) * 2 * G * 17 * 8),
                      "ms_per_step": dt * 1e3, "steps": steps}
    ctx.close()
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


# ------------------------------------------------- von Mises KDE path ----
def run_kde(args):
    """The KDE discretisation path on the 1000-atom chain: the reference's
    von Mises KDE conformer binning (Real2Int::getMinimaPositions; kappa 1,
    up to 5 conformers, 361-point grid) of its 997 torsions over 100,000
    frames, then KDE entropies (bin width 1), all 496,506 torsion pairs and
    MIE/MIST, as the reference runs pdfmethod = vonMisesKDE (torsions only).
    The BAT torsions come from host memory each step (the KDE entry takes
    host buffers), so the step includes their upload."""
    import torch
    from centre_gb300.api import Context, make_params
    from centre_gb300.synth import chain_blocks_torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    natoms, nframes, nsteps, nconf = 1000, 100_000, 10, 5
    ctx = Context(local)
    tors = chain_blocks_torch(natoms, nframes, 2000, dev, coupling="block8")[2][1]
    h_tors = tors.cpu().numpy()
    del tors
    ndof = h_tors.shape[0]
    npairs = ndof * (ndof - 1) // 2
    types = torch.full((ndof,), 3, dtype=torch.uint8, device=dev)
    ext = torch.full((ndof, 4), 1000.0, dtype=torch.float64, device=dev)
    p = make_params(nframes, nsteps, [nconf], [0], True, kde=True)
    s1 = torch.empty((ndof, nsteps), dtype=torch.float64, device=dev)
    s2 = torch.empty((npairs, nsteps), dtype=torch.float64, device=dev)
    mi = torch.empty_like(s2)
    times = {"kde": 0.0, "entropy": 0.0, "score": 0.0}

    def step():
        t0 = time.perf_counter()
        b, minima, nfound = ctx.discretize_vmkde(h_tors, nconf, 1.0, 5, 1e-4, 1000)
        bins = torch.from_numpy(b).to(dev)
        torch.cuda.synchronize(dev)
        t1 = time.perf_counter()
        ctx.entropy1d_dev(p, types, bins, ext, s1)
        ctx.entropy2d_dev(p, types, bins, ext, s2)
        torch.cuda.synchronize(dev)
        t2 = time.perf_counter()
        out = ctx.score_dev(p, types, s1, s2, None, True, mi)
        t3 = time.perf_counter()
        times["kde"] += t1 - t0
        times["entropy"] += t2 - t1
        times["score"] += t3 - t2
        return out

    for _ in range(args.warmup):
        step()
    for k in times:
        times[k] = 0.0
    torch.cuda.synchronize(dev)
    launches0 = ctx.launches
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
    step_ms = wall * 1e3 / args.steps
    # grid work: 361 kernel terms per frame per torsion (FP64 exp each)
    terms = 361.0 * nframes * ndof
    out = {
        "metric": METRIC, "value": npairs / (step_ms / 1e3), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded BAT chain, float32 torsions in host memory)",
        "config": {"workload": f"kde1000: {ndof} torsions, {nframes} frames, von Mises KDE "
                               f"(kappa 1, <= {nconf} conformers, 361-point grid), {nsteps} "
                               f"steps, ML, all {npairs} pairs, MIE-2 + MIST",
                   "l2": "inputs (0.4 GB) larger than L2", "parallelism": "replicas x1"},
        "stage_ms_per_step": {k: v * 1e3 / args.steps for k, v in times.items()},
        "kde_terms_per_s": terms / times["kde"] * args.steps,
        "gpu_launches": ctx.launches - launches0,
    }
    clocks = clk.summary()
    if clocks:
        out["clocks"] = clocks
    ctx.close()
    print(json.dumps(out))


def run_kdegrid(args):
    """The grid-KDE path on the 1000-atom chain (2994 DOFs, 100,000 frames):
    every torsion binned by a von Mises KDE (kappa 50, 72-point grid) and
    every bond and angle by a Gaussian KDE (Silverman bandwidth, 50-point
    grid) into conformer intervals between the density's grid minima
    (centre_gpu_discretize_gridkde_dev), then KDE entropies (bin width 1) of
    all 4,480,521 pairs at 10 steps and MIE/MIST.  The trajectory is resident
    on the device; a step is the whole path."""
    import torch
    from centre_gb300.api import Context, make_params
    from centre_gb300.synth import chain_blocks_torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    natoms, nframes, nsteps = 1000, 100_000, 10
    grids = {1: 50, 2: 50, 3: 72}
    kappa = 50.0
    ctx = Context(local)
    blocks = chain_blocks_torch(natoms, nframes, 2000, dev, coupling="block8")
    ndof = sum(b.shape[0] for _, b in blocks)
    npairs = ndof * (ndof - 1) // 2
    types = torch.cat([torch.full((b.shape[0],), t, dtype=torch.uint8, device=dev)
                       for t, b in blocks])
    ext = torch.full((ndof, 4), 1000.0, dtype=torch.float64, device=dev)
    bins = torch.empty((ndof, 1, nframes), dtype=torch.uint8, device=dev)
    minima = [torch.empty((b.shape[0], grids[t]), dtype=torch.float64, device=dev)
              for t, b in blocks]
    nmin = torch.empty(ndof, dtype=torch.uint8, device=dev)
    nbins = torch.empty(ndof, dtype=torch.uint8, device=dev)
    s1 = torch.empty((ndof, nsteps), dtype=torch.float64, device=dev)
    s2 = torch.empty((npairs, nsteps), dtype=torch.float64, device=dev)
    mi = torch.empty_like(s2)
    times = {"kde": 0.0, "entropy": 0.0, "score": 0.0}

    def step():
        t0 = time.perf_counter()
        off = 0
        for (typ, data), mins in zip(blocks, minima):
            k = data.shape[0]
            ctx.discretize_gridkde_dev(typ, data, grids[typ], kappa, bins[off:off + k, 0], mins,
                                       nmin[off:off + k], nbins[off:off + k])
            off += k
        # histograms as wide as the most conformers any DOF has
        p = make_params(nframes, nsteps, [int(nbins.max().item())], [0], True, kde=True)
        t1 = time.perf_counter()
        ctx.entropy1d_dev(p, types, bins, ext, s1)
        ctx.entropy2d_dev(p, types, bins, ext, s2)
        torch.cuda.synchronize(dev)
        t2 = time.perf_counter()
        out = ctx.score_dev(p, types, s1, s2, None, True, mi)
        t3 = time.perf_counter()
        times["kde"] += t1 - t0
        times["entropy"] += t2 - t1
        times["score"] += t3 - t2
        return out

    for _ in range(args.warmup):
        step()
    for k in times:
        times[k] = 0.0
    torch.cuda.synchronize(dev)
    launches0 = ctx.launches
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
    step_ms = wall * 1e3 / args.steps
    terms = float(nframes) * sum(grids[t] * b.shape[0] for t, b in blocks)
    nb_used = nbins.cpu().numpy()
    out = {
        "metric": METRIC, "value": npairs / (step_ms / 1e3), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded BAT chain drawn on the device, float32)",
        "config": {"workload": f"kdegrid1000: {ndof} DOFs, {nframes} frames, grid KDE "
                               f"(torsions von Mises kappa {kappa:g} on 72 points, bonds/angles "
                               f"Gaussian on 50 points), {nsteps} steps, ML (KDE form), all "
                               f"{npairs} pairs, MIE-2 + MIST",
                   "l2": "inputs (1.2 GB) larger than L2", "parallelism": "replicas x1"},
        "stage_ms_per_step": {k: v * 1e3 / args.steps for k, v in times.items()},
        "kde_terms_per_s": terms / times["kde"] * args.steps,
        "conformers_per_dof": {"max": int(nb_used.max()), "mean": float(nb_used.mean())},
        "gpu_launches": ctx.launches - launches0,
    }
    clocks = clk.summary()
    if clocks:
        out["clocks"] = clocks
    ctx.close()
    print(json.dumps(out))


# ------------------------------------------------ learned pair screen ----
def screen_measure(natoms, steps, warmup, local, seed=4000):
    """A-MIST with the learned pair screen (centre_gpu_screen_dev) on an
    natoms chain, 100,000 frames, 50 bins, 10 steps: each step trains the
    network on exact MI of 200,000 random pairs over the first 20 % of
    frames, keeps 64 partners per DOF, computes their exact joint entropies
    over all frames and runs MIE sums and MIST.  The plain all-pairs MIST of
    the same data is timed once beside it and is the yardstick of the
    total-entropy error.  Returns the measurements and a clock sampler."""
    import torch
    from centre_gb300.api import Context, make_params, make_screen_params
    from centre_gb300.synth import chain_blocks_torch
    dev = torch.device("cuda", local)
    nframes, nb, nsteps = 100_000, 50, 10
    ctx = Context(local)
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        blocks = chain_blocks_torch(natoms, nframes, seed, dev, coupling="block8")
        ndof = sum(x.shape[0] for _, x in blocks)
        bins = torch.empty((ndof, 1, nframes), dtype=torch.uint8, device=dev)
        ext = torch.empty((ndof, 4), dtype=torch.float64, device=dev)
        off = 0
        for typ, data in blocks:
            k = data.shape[0]
            ctx.discretize_dev(typ, data, [nb], bins[off:off + k], ext[off:off + k])
            off += k
        del blocks
    torch.cuda.synchronize(dev)
    types = torch.tensor(sum([[t] * k for t, k in ((1, natoms - 1), (2, natoms - 2),
                                                  (3, natoms - 3))], []),
                         dtype=torch.uint8, device=dev)
    nall = ndof * (ndof - 1) // 2
    p = make_params(nframes, nsteps, [nb], [0], True)
    sp = make_screen_params(feat_div=5, ntrain=200_000, nprefilter=256, nneigh=64, epochs=3,
                            batch=4096, lr=2e-3, seed=17)
    s1 = torch.empty((ndof, nsteps), dtype=torch.float64, device=dev)

    def mist(pairs):
        ctx.entropy1d_dev(p, types, bins, ext, s1)
        n = pairs.shape[0] if pairs is not None else nall
        s2 = torch.empty((n, nsteps), dtype=torch.float64, device=dev)
        ctx.entropy2d_dev(p, types, bins, ext, s2, pairs)
        out = ctx.score_dev(p, types, s1, s2, pairs, True)
        del s2
        return out

    def step():
        pairs, w, losses = ctx.screen_dev(p, sp, types, bins, ext)
        return mist(pairs), pairs.shape[0], losses

    # the yardstick: plain all-pairs MIST, timed once after one warm-up
    full = mist(None)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    full = mist(None)
    torch.cuda.synchronize(dev)
    t_full = time.perf_counter() - t0
    for _ in range(warmup):
        step()
    torch.cuda.synchronize(dev)
    launches0 = ctx.launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize(dev)
        ev0.record(stream)
        t0 = time.perf_counter()
        for _ in range(steps):
            res, npairs, losses = step()
        ev1.record(stream)
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
    step_ms = max(ev0.elapsed_time(ev1), wall * 1e3) / steps
    launches = ctx.launches - launches0
    ctx.close()
    # total MIST entropy (S2 column of the MIST sums) per convergence prefix
    s2_full = full["mist"][:, 16]
    s2_scr = res["mist"][:, 16]
    conv = s2_full[-1]     # all pairs over the whole trajectory: the least biased value
    rec = {
        "workload": f"chain{natoms}: {ndof} DOFs, {nframes} frames, {nb} bins, {nsteps} steps, "
                    "ML, A-MIST over the learned screen's pairs",
        "screen": "train 200000 pairs on first 20% frames, 3 epochs, prefilter 256, keep 64 "
                  "per DOF",
        "ms_per_step": step_ms, "exact_pairs": int(npairs), "all_pairs": nall,
        "all_pairs_mist_ms": t_full * 1e3, "speedup_vs_all_pairs": t_full * 1e3 / step_ms,
        "total_entropy_rel_error": {
            "per_prefix": (np.abs(s2_scr - s2_full) / np.abs(s2_full)).tolist(),
            "max_over_steps": float(np.max(np.abs(s2_scr - s2_full) / np.abs(s2_full))),
            "last_step": float(abs(s2_scr[-1] - s2_full[-1]) / abs(s2_full[-1]))},
        # both estimates at each prefix against the all-pairs value over the
        # whole trajectory: at short prefixes the all-pairs tree (a maximum
        # over every noisy plug-in MI) moves away from it by more than the
        # screened tree does
        "distance_to_full_trajectory_all_pairs": {
            "screened": (np.abs(s2_scr - conv) / abs(conv)).tolist(),
            "all_pairs": (np.abs(s2_full - conv) / abs(conv)).tolist()},
        "train_loss_first_last": [float(losses[0]), float(losses[-1])],
        "gpu_launches": launches,
    }
    return rec, clk.summary()


def run_screen(args):
    """The learned-screen workload on its own line (screen5000: the
    5000-atom chain, 14,994 DOFs; screen1000: the 1000-atom chain)."""
    natoms = 1000 if args.workload == "screen1000" else 5000
    local = int(os.environ.get("LOCAL_RANK", "0"))
    rec, clocks = screen_measure(natoms, args.steps, args.warmup, local)
    nall = rec["all_pairs"]
    out = {
        "metric": METRIC, "value": nall / (rec["ms_per_step"] / 1e3), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": rec["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded BAT chain drawn on the device, float32)",
        "config": {"workload": f"{args.workload}: {rec['workload']} (value = all-pairs count / "
                               "step time)",
                   "screen": rec["screen"], "l2": "inputs larger than L2",
                   "parallelism": "replicas x1"},
        **{k: rec[k] for k in ("exact_pairs", "all_pairs", "all_pairs_mist_ms",
                               "speedup_vs_all_pairs", "total_entropy_rel_error",
                               "distance_to_full_trajectory_all_pairs", "train_loss_first_last",
                               "gpu_launches")},
    }
    if clocks:
        out["clocks"] = clocks
    print(json.dumps(out))


# ------------------------------------------------------- reference arm ----
def run_reference(args):
    """The CPU implementation of the path on this machine's host cores: the
    oracle (plain-C restatement of the reference's Real2Int, binData1D/2D,
    entropy1D/2D and boruvkaMST, OpenMP over DOFs and pairs, every host
    thread).  The reference's own sources are not available here, so its
    compiled form cannot run.  A step is one complete pass of the path over a
    sub-system of the workload: the first K bonds, angles and torsions of the
    same chain (same frames, bins and steps) with all their pairs, MI, MIE-2
    sums and MIST trees.  The value is that pass's pairs per second, measured
    for every step (nothing is extrapolated)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    from centre_gb300.synth import chain_trajectory
    oracle.build(with_ref=False)
    orc = oracle.Oracle()
    w = workload(args.workload)
    tr = chain_trajectory(w["natoms"], w["nframes"], seed=1000, coupling=w["coupling"])
    blocks, glob = subsystem(tr, args.cpu_kper)
    cores = os.cpu_count()
    for _ in range(args.warmup):
        cpu_pass(orc, blocks, cores)
    times = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dt, npairs, _ = cpu_pass(orc, blocks, cores)
        times.append(dt)
    wall = time.perf_counter() - t0
    ms = 1e3 * wall / args.steps
    v = npairs / (ms / 1e3)
    ndof = len(glob)
    sample = (f"per step one complete pass over the sub-system of the first {args.cpu_kper} "
              f"bonds, angles and torsions of chain{w['natoms']} ({ndof} DOFs, all {npairs} "
              f"pairs, {w['nframes']} frames, {NBINS} bins, {NSTEPS} steps): discretise, 1-D, "
              "joint entropies, MI, MIE-2 sums and the MIST tree of every step")
    out = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded BAT chain, float32)",
        "config": {"workload": f"chain{w['natoms']}: {w['ndof']} DOFs, {w['nframes']} frames, "
                               f"{NBINS} bins, {NSTEPS} steps, ML, MIE-2 + MIST; CPU steps "
                               f"run its {ndof}-DOF sub-system",
                   "implementation": "CPU restatement of the reference path (oracle/), "
                                     "OpenMP over DOFs and pairs"},
        "pairs_per_step": npairs, "step_seconds": times,
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample, "extrapolated": False},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="auto", choices=["auto", "tc", "atomic"])
    ap.add_argument("--workload", default="chain1000")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-screen", action="store_true",
                    help="leave the learned-screen sub-record out of the default line")
    ap.add_argument("--no-compare-atomic", dest="compare_atomic", action="store_false")
    ap.add_argument("--cpu-kper", type=int, default=200,
                    help="bonds, angles and torsions of the CPU sub-system pass")
    ap.add_argument("--nbins", type=int, default=0,
                    help="override the workload's bin count (bin-count sweeps)")
    args = ap.parse_args()
    global NBINS, NSTEPS
    from centre_gb300.synth import BATCHES
    if args.workload == "kde1000":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the KDE path is measured "
                              "against the histogram reference arm only"}))
            return
        run_kde(args)
        return
    if args.workload == "kdegrid1000":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the grid KDE has no "
                              "reference counterpart (the reference's KDE is torsion-only)"}))
            return
        run_kdegrid(args)
        return
    if args.workload in ("screen5000", "screen1000"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the learned screen has no "
                              "reference counterpart (the reference reads neighbour files)"}))
            return
        run_screen(args)
        return
    if args.workload in BATCHES:
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "batched workloads are "
                              "measured against the single-trajectory reference arm"}))
            return
        run_batch(args)
        return
    w = workload(args.workload)
    NBINS, NSTEPS = w["nbins"], w["nsteps"]
    if args.nbins:
        NBINS = args.nbins
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
