#!/usr/bin/env python3
"""Benchmark: Dual Marching Cubes throughput on one GB300.

Default workload: 1024^3 uint16 lattice value noise (4 octaves, base period
128 voxels, persistence 0.5, quantised to 0..65535), isovalue 32768 -- the
reference's plain-extractor configuration with the HBM-roofline target.
Synthetic data generated on the device from a fixed seed.

One step = one full extraction (count sweep, segment scan, emit sweep) of the
resident volume into preallocated device buffers.  The input (2 GiB) is
larger than L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload noise1024|blobs512|sphere64]

Prints one JSON line (rank 0).  --impl reference times the reference
algorithm's CPU restatement (the reference itself is CUDA-only, Fermi-era and
has no CPU path) with all host threads on a bounded z-slab sample.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (dims, dtype, iso, description)
    "noise1024": ((1024, 1024, 1024), "uint16", 32768.0,
                  "1024^3 uint16 4-octave lattice value noise (period 128, persistence 0.5), iso 32768"),
    "blobs512": ((512, 512, 512), "float32", 0.5,
                 "512^3 float32 sum of 32 Gaussian blobs (sigma 8-32, amplitude 0.5-1.5), iso 0.5"),
    "sphere64": ((64, 64, 64), "float32", 0.0,
                 "64^3 float32 sphere SDF radius 20 + uniform noise 0.01, iso 0"),
    # the 1024^3 noise field's statistics on an eighth of the volume (profiling case)
    "noise512": ((512, 512, 512), "uint16", 32768.0,
                 "512^3 uint16 4-octave lattice value noise (period 128, persistence 0.5), iso 32768"),
}


def make_volume(name, device, zrange=None):
    import torch
    from framework_gb300 import fields
    dims, dtype, iso, _ = WORKLOADS[name]
    if name in ("noise1024", "noise512"):
        vol = fields.value_noise_u16(dims, device=device)
    elif name == "blobs512":
        vol = fields.gaussian_blobs(dims, device=device)
    else:
        vol = fields.sphere_sdf(64, radius=20.0, noise=0.01, seed=1).to(device)
    if device != "cpu":
        torch.cuda.synchronize()
    return vol, iso


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(dict(sm=float(parts[1]), smax=float(parts[2]), power=float(parts[3]),
                                 hw=parts[5], hwt=parts[6], swt=parts[7], swpc=parts[8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        reasons = set()
        for r in rows:
            for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"),
                              ("swt", "sw_thermal_slowdown"), ("swpc", "sw_power_cap")):
                if r[key].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in rows), "sm_max_mhz": max(r["smax"] for r in rows),
                "reasons": sorted(reasons), "samples": len(rows)}


def combine_ranks(ms, units, dist, device):
    """Whole-job figures when every rank processed its own `units` in `ms`
    (independent volumes, weak scaling): the slowest rank's time and the
    units of all ranks.  Without a process group, the rank's own."""
    if dist is None:
        return ms, units
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# the sources of the brick kernels: a DRAM-traffic figure holds only for the
# build it was captured on
TRAFFIC_SOURCES = ("dmc_brick.cu", "dmc_device.cuh", "dmc_scan.cuh", "dmc_tables.inc", "dmc_internal.h")


def kernel_sources_sha256():
    import hashlib
    h = hashlib.sha256()
    for name in TRAFFIC_SOURCES:
        with open(os.path.join(ROOT, "framework_gb300", "csrc", name), "rb") as f:
            h.update(name.encode() + b"\0" + f.read())
    return h.hexdigest()


def profile_traffic(workload, kernel="emit"):
    """DRAM bytes per launch of a brick kernel on a workload, from the ncu
    capture recorded in profiles/traffic.json.  The record carries the
    sha256 of the kernel sources it was captured on; when the sources have
    changed since, the figure no longer describes this build: a warning goes
    to stderr and the traffic is reported as null."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    if d.get("sources_sha256") != kernel_sources_sha256():
        print("warning: profiles/traffic.json was captured on other kernel sources; traffic reported as null",
              file=sys.stderr, flush=True)
        return None
    return d.get("%s:%s" % (workload, kernel))


def cpu_model():
    """CPU model name of this host (lscpu), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_single_thread_sample(vol_host, iso, target_s=3.0):
    """The CPU restatement on one thread, on a z-slab sized for ~target_s.
    Returns (GVoxels/s, sample text); leaves the oracle on all host threads."""
    import numpy as np
    import oracle
    oracle.set_threads(1)
    try:
        nz = vol_host.shape[0]
        planes = min(nz, 4)
        t0 = time.perf_counter()
        oracle.extract(np.ascontiguousarray(vol_host[:planes]), iso=iso)
        dt = time.perf_counter() - t0
        planes = max(planes, min(nz, int(planes * target_s / max(dt, 1e-3))))
        sample = np.ascontiguousarray(vol_host[:planes])
        t0 = time.perf_counter()
        oracle.extract(sample, iso=iso)
        dt = time.perf_counter() - t0
    finally:
        oracle.set_threads(os.cpu_count() or 1)
    return sample.size / dt / 1e9, "z-slab of %d x %d x %d points (%.1f s)" % (
        sample.shape[2], sample.shape[1], sample.shape[0], dt)


def cpu_oracle_sample(vol_host, iso, target_s=10.0):
    """Time the CPU restatement with all host threads on a z-slab sample of
    the workload, sized for ~target_s of work.  Returns GVoxels/s, cores, sample text."""
    import numpy as np
    import oracle
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    nz = vol_host.shape[0]
    planes = min(nz, 34)
    t0 = time.perf_counter()
    oracle.extract(np.ascontiguousarray(vol_host[:planes]), iso=iso)
    dt = time.perf_counter() - t0
    want = int(planes * target_s / max(dt, 1e-3))
    planes = max(planes, min(nz, want))
    sample = np.ascontiguousarray(vol_host[:planes])
    t0 = time.perf_counter()
    oracle.extract(sample, iso=iso)
    dt = time.perf_counter() - t0
    return sample.size / dt / 1e9, cores, "z-slab of %d x %d x %d points (%.1f s)" % (
        sample.shape[2], sample.shape[1], sample.shape[0], dt)


def run_reference(args, rank):
    """CPU restatement of the reference algorithm, all host threads."""
    import numpy as np
    import torch
    if rank != 0:
        return
    wl = "noise1024" if args.workload == "shard1024" else args.workload   # the sharded volume is the same field
    dims, dtype, iso, desc = WORKLOADS[wl]
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    vol, iso = make_volume(wl, dev)
    from framework_gb300 import fields
    host = fields.as_u16_numpy(vol) if dtype == "uint16" else vol.cpu().numpy()
    import oracle
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    # bounded sample per step: a z-slab sized for ~10 s per step in total
    planes = min(host.shape[0], 34)
    t0 = time.perf_counter()
    oracle.extract(np.ascontiguousarray(host[:planes]), iso=iso)
    dt = time.perf_counter() - t0
    budget = 120.0 / max(1, args.steps + args.warmup)
    planes = max(2, min(host.shape[0], int(planes * budget / max(dt, 1e-3))))
    sample = np.ascontiguousarray(host[:planes])
    for _ in range(args.warmup):
        oracle.extract(sample, iso=iso)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.extract(sample, iso=iso)
        times.append(time.perf_counter() - t0)
    t = sum(times)
    value = sample.size * args.steps / t / 1e9
    line = {
        "impl": "reference", "metric": "GVoxels/s", "value": round(value, 4), "unit": "GVoxels/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * t / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u16" if dtype == "uint16" else "f32", "data": "synthetic",
        "config": {"workload": args.workload, "desc": desc, "sample_points": int(sample.size)},
        "cpu_baseline": {"value": round(value, 4), "unit": "GVoxels/s", "cores": cores, "kind": "port",
                         "sample": "z-slab %dx%dx%d of the workload" % (sample.shape[2], sample.shape[1], sample.shape[0]),
                         "cpu_model": cpu_model()},
        "e2e": {"value": round(value, 4), "unit": "GVoxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


BATCH_DESC = ("256 float32 gyroid volumes sin(fx)cos(fy)+sin(fy)cos(fz)+sin(fz)cos(fx), per-axis dims "
              "log-uniform 16-256, f uniform 0.05-0.4 rad/voxel, noise sigma 0.02, iso uniform -0.5..0.5")


def make_batch(device, count=256, lo=16, hi=256, seed=5):
    """The uneven gyroid batch in one device pool (each volume a view, 256-byte aligned)."""
    import torch
    from framework_gb300 import fields
    specs = fields.uneven_batch_specs(count=count, lo=lo, hi=hi, seed=seed)
    offs, total = [], 0
    for sp in specs:
        nx, ny, nz = sp["dims"]
        offs.append(total)
        total += (nx * ny * nz + 63) // 64 * 64
    pool = torch.empty(total, dtype=torch.float32, device=device)
    vols = []
    for sp, off in zip(specs, offs):
        nx, ny, nz = sp["dims"]
        v = pool[off:off + nx * ny * nz].view(nz, ny, nx)
        v.copy_(fields.gyroid(sp["dims"], sp["freq"], seed=sp["seed"], device=device))
        vols.append(dict(volume=v, iso=sp["iso"]))
    if device != "cpu":
        torch.cuda.synchronize()
    return pool, vols


def batch_cpu_sample(vols, target_s=10.0):
    """CPU restatement over the first volumes of the batch, all host threads, ~target_s."""
    import numpy as np
    import oracle
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    done, t_used = 0, 0.0
    for d in vols:
        host = np.ascontiguousarray(d["volume"].cpu().numpy())
        t0 = time.perf_counter()
        oracle.extract(host, iso=d["iso"])
        t_used += time.perf_counter() - t0
        done += 1
        if t_used >= target_s:
            break
    return done / t_used, cores, "first %d of %d volumes (%.1f s)" % (done, len(vols), t_used)


def run_batch(args, rank, world, dist=None):
    """Batched extraction of the uneven gyroid mix: graph-launched pipeline
    (vol/s) against one plain extraction call per volume."""
    import torch
    import framework_gb300 as fg
    from framework_gb300 import autotune
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pool, vols = make_batch("cuda")
    n = len(vols)
    N = sum(d["volume"].numel() for d in vols)
    ex = fg.Extractor(local, algo="brick")
    V, Q, res = ex.extract_batch(vols)              # count only
    vbuf = torch.empty((V, 3), device="cuda")
    qbuf = torch.empty((Q, 4), dtype=torch.int32, device="cuda")
    tune = autotune.tune(ex, vols, vbuf, qbuf)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        ex.extract_batch(vols, vbuf, qbuf, mode="graph")
        ex.batch_wait()
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        ex.extract_batch(vols, vbuf, qbuf, mode="graph")
        nv, nq, _r = ex.batch_wait()
    ev1.record(stream)
    torch.cuda.synchronize()
    ms, total_vols = combine_ranks(ev0.elapsed_time(ev1) / args.steps, n, dist, "cuda")
    clk = clocks.stop()
    assert (nv, nq) == (V, Q)
    # per-kernel split from one synchronous call
    ex.extract_batch(vols, vbuf, qbuf)
    st = ex.stats()
    # plain form: one dmc_extract_device call per volume into the same buffers
    plain_reps = max(1, min(3, args.steps))
    for d in vols:
        ex.extract_device(d["volume"], iso=d["iso"], vertices=vbuf, quads=qbuf)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(plain_reps):
        for d in vols:
            ex.extract_device(d["volume"], iso=d["iso"], vertices=vbuf, quads=qbuf)
    torch.cuda.synchronize()
    plain_s = (time.perf_counter() - t0) / plain_reps
    # the same volumes as one-volume asynchronous batches on two contexts,
    # each with its own stream: no batching across volumes, and no host wait
    # between launches (a context waits only for its own previous volume)
    exa = (ex, fg.Extractor(local, algo="brick"))
    exa[1].set_option(fg.OPT_BRICK_PLANES, int(tune["planes"]))
    sa = [torch.cuda.Stream(device=local) for _ in range(2)]
    vmax, qmax = int(res[:, 1].max()), int(res[:, 3].max())
    one_v = [torch.empty((max(vmax, 1), 3), device="cuda") for _ in range(2)]
    one_q = [torch.empty((max(qmax, 1), 4), dtype=torch.int32, device="cuda") for _ in range(2)]

    def one_by_one():
        busy = [False, False]
        for i, d in enumerate(vols):
            c = i & 1
            if busy[c]:
                exa[c].batch_wait()
            exa[c].extract_batch([d], one_v[c], one_q[c], mode="async", stream=sa[c])
            busy[c] = True
        for c in (0, 1):
            if busy[c]:
                exa[c].batch_wait()
    one_by_one()                                  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(plain_reps):
        one_by_one()
    torch.cuda.synchronize()
    single_s = (time.perf_counter() - t0) / plain_reps
    exa[1].close()
    del one_v, one_q
    # end to end: pinned host volumes in, host meshes out, per step.  The
    # volumes go up, through and down in 8 groups on two contexts (asynchronous
    # batches), so that one group's upload, another's extraction and a third's
    # download overlap.  Each group extracts into a device region of 1.25 times
    # its counts in the step before (the sizing pass for the first step); once
    # batch_wait has returned a group's counts, exactly its mesh is copied
    # down, after the meshes of the groups before it.  (The batch is the same
    # every step, so the regions are sized once.)
    host_pool = torch.empty(pool.shape, dtype=pool.dtype, pin_memory=True)
    host_pool.copy_(pool)
    hv = torch.empty((V, 3), dtype=torch.float32, pin_memory=True)
    hq = torch.empty((Q, 4), dtype=torch.int32, pin_memory=True)
    e2e_steps = max(1, min(args.e2e_steps, args.steps))
    ex2 = fg.Extractor(local, algo="brick")
    ex2.set_option(fg.OPT_BRICK_PLANES, int(tune["planes"]))
    exs = (ex, ex2)
    n_groups = 8
    groups = []
    for g in range(n_groups):
        a, b = g * n // n_groups, (g + 1) * n // n_groups
        lo = (vols[a]["volume"].data_ptr() - pool.data_ptr()) // 4
        hi = (vols[b]["volume"].data_ptr() - pool.data_ptr()) // 4 if b < n else pool.numel()
        groups.append((a, b, lo, hi))
    sizing = [(int(res[b - 1][0] + res[b - 1][1] - res[a][0]), int(res[b - 1][2] + res[b - 1][3] - res[a][2]))
              for a, b, _, _ in groups]
    caps = [(v * 5 // 4 + 64, q * 5 // 4 + 64) for v, q in sizing]
    cv = [sum(c[0] for c in caps[:g]) for g in range(n_groups)]
    cq = [sum(c[1] for c in caps[:g]) for g in range(n_groups)]
    del vbuf, qbuf
    dv = torch.empty((cv[-1] + caps[-1][0], 3), dtype=torch.float32, device=f"cuda:{local}")
    dq = torch.empty((cq[-1] + caps[-1][1], 4), dtype=torch.int32, device=f"cuda:{local}")
    s_up, s_dn = torch.cuda.Stream(), torch.cuda.Stream()
    s_ex = (torch.cuda.Stream(), torch.cuda.Stream())
    e2e_bytes = [0, 0]

    def pipelined_pass():
        pend = [None, None]
        off = [0, 0]

        def finish(c):
            g = pend[c]
            nv_g, nq_g, _ = exs[c].batch_wait()
            with torch.cuda.stream(s_dn):
                hv[off[0]:off[0] + nv_g].copy_(dv[cv[g]:cv[g] + nv_g], non_blocking=True)
                hq[off[1]:off[1] + nq_g].copy_(dq[cq[g]:cq[g] + nq_g], non_blocking=True)
            off[0] += nv_g
            off[1] += nq_g
            pend[c] = None
        t0 = time.perf_counter()
        for g, (a, b, lo, hi) in enumerate(groups):
            c = g % 2
            if pend[c] is not None:
                finish(c)                         # the group two back on this context
            up = torch.cuda.Event()
            with torch.cuda.stream(s_up):
                pool[lo:hi].copy_(host_pool[lo:hi], non_blocking=True)
                up.record(s_up)
            s_ex[c].wait_event(up)
            exs[c].extract_batch(vols[a:b], dv[cv[g]:cv[g] + caps[g][0]], dq[cq[g]:cq[g] + caps[g][1]],
                                 mode="async", stream=s_ex[c])
            pend[c] = g
        for c in (n_groups % 2, (n_groups + 1) % 2):
            if pend[c] is not None:
                finish(c)
        torch.cuda.synchronize()
        e2e_bytes[0], e2e_bytes[1] = off
        return time.perf_counter() - t0

    pipelined_pass()                             # warm-up (second context, streams)
    e2e_s = sum(pipelined_pass() for _ in range(e2e_steps)) / e2e_steps
    # the host meshes are the whole batch's, bit for bit
    assert tuple(e2e_bytes) == (V, Q)
    del dv, dq
    vbuf = torch.empty((V, 3), dtype=torch.float32, device=f"cuda:{local}")
    qbuf = torch.empty((Q, 4), dtype=torch.int32, device=f"cuda:{local}")
    ex.extract_batch(vols, vbuf, qbuf)
    assert torch.equal(hv, vbuf.cpu()) and torch.equal(hq, qbuf.cpu())
    ex2.close()
    line = None
    if rank == 0:
        hbm, peak_kind = peaks()
        alg_bytes = 4 * N + 12 * V + 16 * Q
        value = total_vols / (ms * 1e-3)
        achieved = alg_bytes / (st["emit_ms"] * 1e-3) / 1e9 if st["emit_ms"] > 0 else None
        cpu = None
        if not args.no_cpu_baseline:
            v, cores, sample = batch_cpu_sample(vols)
            cpu = {"value": round(v, 3), "unit": "volumes/s", "cores": cores, "kind": "port", "sample": sample}
        line = {
            "metric": "volumes/s", "value": round(value, 2), "unit": "volumes/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batch256", "desc": BATCH_DESC, "volumes": n, "points": N,
                       "vertices": V, "quads": Q, "mode": "graph", "autotune": tune,
                       "gvox_per_s": round(N / (ms * 1e-3) / 1e9, 3),
                       "plain_volumes_per_s": round(n / plain_s, 2),
                       "batched_over_plain": round((n / (ms * 1e-3)) / (n / plain_s), 2),
                       "single_async_volumes_per_s": round(n / single_s, 2),
                       "batched_over_single_async": round((n / (ms * 1e-3)) / (n / single_s), 2),
                       "kernel_ms": {"count": round(st["count_ms"], 4), "scan": round(st["scan_ms"], 4),
                                     "emit": round(st["emit_ms"], 4)},
                       "l2": "batch input %.0f MB > L2 (no flush needed)" % (4 * N / 1e6)},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1) if achieved else None, "peak": hbm,
                         "unit": "GB/s", "frac": round(achieved / hbm, 4) if achieved else None,
                         "traffic": profile_traffic("batch256"), "kernel": "brick_emit", "peak_kind": peak_kind,
                         "algorithmic_bytes": alg_bytes,
                         "pipeline_frac": round(alg_bytes / (ms * 1e-3) / 1e9 / hbm, 4)},
            "cpu_baseline": cpu,
            "e2e": {"value": round(n / e2e_s, 2), "unit": "volumes/s", "h2d_bytes_per_step": 4 * N,
                    "d2h_bytes_per_step": 12 * V + 16 * Q, "steps": e2e_steps,
                    "call": "dmc_extract_batch (asynchronous, 8 groups on two contexts) with page-locked "
                            "host volumes and meshes; uploads, batches and downloads overlap; each group's "
                            "download is sized by its own counts, after its batch_wait"},
            "gpu_launches": 7 * args.steps,
            "clocks": clk,
        }
    ex.close()
    return line if rank == 0 else None


def run_batch_reference(args, rank):
    """CPU restatement on the batch: volumes/s over a bounded prefix."""
    if rank != 0:
        return
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    _pool, vols = make_batch(dev)
    budget = 120.0 / max(1, args.steps + args.warmup)
    v, cores, sample = batch_cpu_sample(vols, target_s=min(budget, 20.0))
    line = {
        "impl": "reference", "metric": "volumes/s", "value": round(v, 3), "unit": "volumes/s",
        "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": round(1e3 / v, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batch256", "desc": BATCH_DESC},
        "cpu_baseline": {"value": round(v, 3), "unit": "volumes/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": round(v, 3), "unit": "volumes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


SERVED_DESC = ("device-resident pool of 64 volumes, per-axis dims log-uniform 32-512 with the upper tail "
               "weighted to a ~6 GB pool (each draw kept with probability (points/512^3)^1.4), f32 blobs / u16 "
               "lattice noise / f32 gyroid; requests (volume, iso uniform in that field's 5th-95th percentile) "
               "with seeded Poisson arrivals; admission by worst-case output bound")


# output arenas of the served bench: 4.0 G vertices (48 GB) and 2.1 G quads (34 GB)
SERVED_VERTEX_ARENA, SERVED_QUAD_ARENA = 0xF0000000, 0x80000000


def make_pool(device="cuda"):
    """The serving pool and each volume's 5th/95th percentile (from a 1M-sample draw)."""
    import torch
    from framework_gb300 import fields
    specs = fields.served_pool_specs()
    vols = []
    g = torch.Generator(device="cpu")
    g.manual_seed(77)
    for sp in specs:
        t = fields.make_pool_volume(sp, device=device)
        flat = t.reshape(-1)
        idx = torch.randint(0, flat.numel(), (min(flat.numel(), 1 << 20),), generator=g).to(device)
        smp = flat[idx].to(torch.int32) & 0xFFFF if t.dtype == torch.int16 else flat[idx]
        lo, hi = torch.quantile(smp.to(torch.float32), torch.tensor([0.05, 0.95], device=device)).tolist()
        vols.append(dict(volume=t, lo=lo, hi=hi, kind=sp["kind"], u16=t.dtype == torch.int16))
    torch.cuda.synchronize()
    return vols


def request_trace(vols, n, rate, seed):
    """n requests: uniform volume, iso uniform in [P5, P95]; Poisson arrivals at `rate`/s (0: all at once)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    vid = rng.integers(0, len(vols), n)
    iso = np.array([rng.uniform(vols[v]["lo"], vols[v]["hi"]) for v in vid], np.float32)
    arr = np.cumsum(rng.exponential(1.0 / rate, n)) if rate > 0 else np.zeros(n)
    return vid.astype(np.uint32), iso, arr


def _lat_summary(lat, arrivals, n):
    import numpy as np
    ok = lat[lat >= 0]
    span = float(np.max(arrivals + lat)) if len(lat) else 0.0
    return {"p50_ms": round(1e3 * float(np.percentile(ok, 50)), 3), "p99_ms": round(1e3 * float(np.percentile(ok, 99)), 3),
            "throughput": round(n / span, 2) if span > 0 else None}


def _warm(srv, idmap, vols):
    """Every pool volume once, at its median-ish isovalue (graph capture, scratch growth)."""
    import numpy as np
    iso = np.array([0.5 * (d["lo"] + d["hi"]) for d in vols], np.float32)
    srv.replay(idmap, iso, np.zeros(len(vols)))


def served_measure(vols, n_req=600, quick=False, device=0):
    """Saturation throughput and a Poisson load sweep for the batched server
    and the plain per-request server on the same traces."""
    import numpy as np
    import framework_gb300 as fg
    out = {}
    servers = {"served": dict(lanes=2, max_batch=64), "plain": dict(plain=True)}
    for name, kw in servers.items():
        with fg.Server(device, vertex_arena=SERVED_VERTEX_ARENA, quad_arena=SERVED_QUAD_ARENA, **kw) as srv:
            ids = [srv.add_volume(d["volume"]) for d in vols]
            idmap = np.array(ids, np.uint32)
            _warm(srv, idmap, vols)
            n_sat = n_req if name == "served" else max(64, n_req // 4)
            vid, iso, arr = request_trace(vols, n_sat, 0, seed=2)
            t0 = time.perf_counter()
            lat, st = srv.replay(idmap[vid], iso, arr)
            wall = time.perf_counter() - t0
            if (st != 0).any():
                print("%s saturation: failed requests by status %s" % (
                    name, dict(zip(*[x.tolist() for x in np.unique(st[st != 0], return_counts=True)]))),
                    file=sys.stderr, flush=True)
            cap = n_sat / wall
            out[name] = {"capacity_rps": round(cap, 2), "saturation": _lat_summary(lat, arr, n_sat),
                         "stats": srv.stats()}
    # offered loads: fractions of each server's own capacity, and the plain
    # server's 80% load offered to both
    loads = [("plain@0.8plain", "plain", 0.8 * out["plain"]["capacity_rps"]),
             ("served@0.8plain", "served", 0.8 * out["plain"]["capacity_rps"]),
             ("served@0.8served", "served", 0.8 * out["served"]["capacity_rps"])]
    if not quick:
        loads.insert(2, ("served@0.5served", "served", 0.5 * out["served"]["capacity_rps"]))
    sweep = {}
    for label, name, rate in loads:
        kw = servers[name]
        n = max(200, min(n_req, int(rate * (4.0 if not quick else 2.0))))
        with fg.Server(device, vertex_arena=SERVED_VERTEX_ARENA, quad_arena=SERVED_QUAD_ARENA, **kw) as srv:
            idmap = np.array([srv.add_volume(d["volume"]) for d in vols], np.uint32)
            _warm(srv, idmap, vols)
            vid, iso, arr = request_trace(vols, n, rate, seed=3)
            lat, st = srv.replay(idmap[vid], iso, arr)
            bad = {int(k): int(c) for k, c in zip(*np.unique(st[st != 0], return_counts=True))}
            if bad:
                print("load %s: failed requests by status %s" % (label, bad), file=sys.stderr, flush=True)
            sweep[label] = dict(offered_rps=round(rate, 2), requests=n, failed=bad, **_lat_summary(lat, arr, n))
    out["sweep"] = sweep
    return out


def served_cpu_sample(vols, budget):
    """The oracle, all host threads, on the first requests of the saturation trace for ~budget seconds."""
    import oracle
    from framework_gb300 import fields
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    vid, iso, _ = request_trace(vols, 256, 0, seed=2)
    done, used = 0, 0.0
    for v, x in zip(vid, iso):
        t = vols[v]["volume"]
        host = fields.as_u16_numpy(t) if vols[v]["u16"] else t.cpu().numpy()
        t0 = time.perf_counter()
        oracle.extract(host, iso=float(x))
        used += time.perf_counter() - t0
        done += 1
        if used >= budget:
            break
    return done / used, cores, "first %d requests of the saturation trace (%.1f s)" % (done, used)


def run_served_reference(args, rank):
    """CPU restatement over a bounded prefix of the request trace (requests/s, all host threads)."""
    if rank != 0:
        return
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    vols = make_pool(dev)
    v, cores, sample = served_cpu_sample(vols, min(20.0, 120.0 / max(1, args.steps + args.warmup)))
    line = {
        "impl": "reference", "metric": "requests/s", "value": round(v, 3), "unit": "requests/s",
        "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": round(1e3 / v, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+u16", "data": "synthetic",
        "config": {"workload": "served64", "desc": SERVED_DESC},
        "cpu_baseline": {"value": round(v, 3), "unit": "requests/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(v, 3), "unit": "requests/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def served_e2e(vols, local, plain=False, n=256, max_batch=64, repeats=3):
    """End to end: a burst of n requests, each mesh copied into page-locked
    host buffers (a ring of reused ones, allocated before the timed burst and
    sized by an untimed pass over the same requests, as a server sizes its
    ring once) and released once its copy is done.  The copies run on a copy
    stream, so the next result's copy is queued while one is in flight.  The
    timed burst runs `repeats` times; the median rate is reported.  With
    plain=True the same burst goes to the plain per-request server."""
    import torch
    import framework_gb300 as fg
    vid, iso, _ = request_trace(vols, n, 0, seed=4)
    kw = dict(plain=True) if plain else dict(max_batch=max_batch)
    with fg.Server(local, vertex_arena=SERVED_VERTEX_ARENA, quad_arena=SERVED_QUAD_ARENA, **kw) as srv:
        idmap = [srv.add_volume(d["volume"]) for d in vols]
        vmax = qmax = 1
        for v, x in zip(vid, iso):                     # warm up: the same burst, untimed
            r = srv.submit(idmap[v], float(x))
            res = srv.wait(r, timeout=600.0)
            vmax, qmax = max(vmax, res["n_vertices"]), max(qmax, res["n_quads"])
            srv.release(r)
        nslot = 3
        hv = [torch.empty((vmax, 3), dtype=torch.float32, pin_memory=True) for _ in range(nslot)]
        hq = [torch.empty((qmax, 4), dtype=torch.int32, pin_memory=True) for _ in range(nslot)]
        busy = [None] * nslot                          # (request, copy-done event) per slot
        copy_stream = torch.cuda.Stream(device=local)

        def retire(s):
            if busy[s] is not None:
                busy[s][1].synchronize()
                srv.release(busy[s][0])
                busy[s] = None
        rates = []
        for _ in range(repeats):
            d2h = 0
            t0 = time.perf_counter()
            rids = [srv.submit(idmap[v], float(x)) for v, x in zip(vid, iso)]
            for i, r in enumerate(rids):
                res = srv.wait(r, timeout=600.0)
                s = i % nslot
                retire(s)
                if res["n_vertices"] > len(hv[s]) or res["n_quads"] > len(hq[s]):
                    hv[s] = torch.empty((res["n_vertices"], 3), dtype=torch.float32, pin_memory=True)
                    hq[s] = torch.empty((res["n_quads"], 4), dtype=torch.int32, pin_memory=True)
                nv, nq = srv.fetch_into(res, hv[s], hq[s], stream=copy_stream)
                ev = torch.cuda.Event()
                ev.record(copy_stream)
                busy[s] = (r, ev)
                d2h += 12 * nv + 16 * nq
            for s in range(nslot):
                retire(s)
            rates.append(len(rids) / (time.perf_counter() - t0))
    return {"rps": round(sorted(rates)[len(rates) // 2], 2), "runs_rps": [round(x, 1) for x in rates],
            "d2h_per_request": int(d2h / len(rids)), "requests": len(rids)}


def run_served(args, rank, world, dist=None):
    import numpy as np
    import torch
    import framework_gb300 as fg
    local = int(os.environ.get("LOCAL_RANK", "0"))   # this rank's GPU (the current device)
    vols = make_pool("cuda")
    N = sum(d["volume"].numel() for d in vols)
    nbytes = sum(d["volume"].numel() * d["volume"].element_size() for d in vols)
    clocks = ClockSampler(local)
    clocks.start()
    m = served_measure(vols, n_req=max(200, 60 * args.steps), device=local)
    clk = clocks.stop()
    # every rank serves its own request stream: whole-job capacity is the sum
    _, total_rps = combine_ranks(0.0, m["served"]["capacity_rps"], dist, "cuda")
    e2e = served_e2e(vols, local, plain=False)
    e2e_plain = served_e2e(vols, local, plain=True)
    if rank != 0:
        return None
    cpu = None
    if not args.no_cpu_baseline:
        v, cores, sample = served_cpu_sample(vols, 10.0)
        cpu = {"value": round(v, 3), "unit": "requests/s", "cores": cores, "kind": "port", "sample": sample}
    line = {
        "metric": "requests/s", "value": round(total_rps, 2), "unit": "requests/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 / m["served"]["capacity_rps"], 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+u16", "data": "synthetic",
        "config": {"workload": "served64", "desc": SERVED_DESC, "volumes": len(vols), "points": N,
                   "pool_bytes": nbytes, "mix": {k: sum(1 for d in vols if d["kind"] == k) for k in ("blobs", "noise", "gyroid")},
                   "served": m["served"], "plain": m["plain"], "sweep": m["sweep"],
                   "served_over_plain": round(m["served"]["capacity_rps"] / m["plain"]["capacity_rps"], 2),
                   "p99_ms_at_0.8_served_capacity": m["sweep"]["served@0.8served"]["p99_ms"],
                   "l2": "pool %.2f GB > L2" % (nbytes / 1e9)},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e["rps"], "unit": "requests/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": e2e["d2h_per_request"], "requests": e2e["requests"],
                "plain_value": e2e_plain["rps"], "runs": e2e["runs_rps"], "plain_runs": e2e_plain["runs_rps"],
                "note": "pool resident on the device; per request the mesh is copied into page-locked host buffers "
                        "(Server.fetch_into on a copy stream, three buffers in turn, sized by an untimed pass); "
                        "median of three bursts; plain_value: the plain "
                        "per-request server on the same burst, same copies"},
        "gpu_launches": 7 * m["served"]["stats"]["batches"],
        "clocks": clk,
    }
    return line


def run_shard(args, rank, world, dist=None):
    """One 1024^3 uint16 noise volume split in z across the ranks (strong
    scaling): each rank holds its cell planes plus halo, counts its part,
    all-gathers the (vertices, quads) totals (NCCL under torchrun, the path's
    one collective) and writes its part with global indices.  A step is
    count + exchange + emit; value = the whole volume's points / the slowest
    rank's step time.  e2e adds, per step, the upload of the rank's planes
    from page-locked host memory and the download of its part."""
    import torch
    import framework_gb300 as fg
    from framework_gb300 import fields, shard
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dims, dtype, iso, desc = WORKLOADS["noise1024"]
    nz = dims[2]
    full = fields.value_noise_u16(dims, device="cuda")
    zb, ze = shard.shard_ranges(nz - 1, world)[rank]
    p0, p1 = shard.point_planes(nz, zb, ze)
    part_in = full[p0:p1].clone()
    del full
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    N = dims[0] * dims[1] * dims[2]
    ex = fg.Extractor(local, algo="brick")
    res = shard.extract_sharded(ex, part_in, nz, zb, ze, iso=iso, dist=dist)
    V, Q = res["vertices"].shape[0], res["quads"].shape[0]
    vbuf = torch.empty((max(V, 1), 3), device="cuda")
    qbuf = torch.empty((max(Q, 1), 4), dtype=torch.int32, device="cuda")

    def step():
        nv, nq = ex.shard_count(part_in, nz, zb, ze, None, None, iso)
        totals = shard.exchange_totals(nv, nq, dist)
        voff, _ = shard.exclusive_offsets(totals, rank)
        ex.shard_emit(voff, vbuf, qbuf)
        return totals
    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        totals = step()
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms, _ = combine_ranks(ev0.elapsed_time(ev1) / args.steps, 0, dist, "cuda")
    # end to end: planes in from page-locked host memory, the part out
    host_in = torch.empty(part_in.shape, dtype=part_in.dtype, pin_memory=True)
    host_in.copy_(part_in)
    hv = torch.empty((max(V, 1), 3), dtype=torch.float32, pin_memory=True)
    hq = torch.empty((max(Q, 1), 4), dtype=torch.int32, pin_memory=True)
    e2e_steps = max(1, min(args.e2e_steps, args.steps))
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        part_in.copy_(host_in, non_blocking=True)
        step()
        hv.copy_(vbuf[:max(V, 1)], non_blocking=True)
        hq.copy_(qbuf[:max(Q, 1)], non_blocking=True)
        torch.cuda.synchronize()
    e2e_ms, _ = combine_ranks((time.perf_counter() - t0) * 1e3 / e2e_steps, 0, dist, "cuda")
    ex.close()
    if rank != 0:
        return None
    Vt, Qt = sum(t[0] for t in totals), sum(t[1] for t in totals)
    hbm, peak_kind = peaks()
    alg_bytes = 2 * N + 12 * Vt + 16 * Qt
    return {
        "metric": "GVoxels/s", "value": round(N / (ms * 1e-3) / 1e9, 3), "unit": "GVoxels/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "u16", "data": "synthetic",
        "config": {"workload": "shard1024", "desc": desc + "; one volume split in z across ranks",
                   "dims": list(dims), "iso": iso, "vertices": Vt, "quads": Qt,
                   "parallelism": "z-slab shards, all-gather of (V, Q) per rank" if world > 1 else "single GPU",
                   "l2": "input larger than L2 (no flush needed)"},
        "roofline": {"bound": "hbm", "achieved": round(alg_bytes / (ms * 1e-3) / 1e9 / max(world, 1), 1),
                     "peak": hbm, "unit": "GB/s",
                     "frac": round(alg_bytes / (ms * 1e-3) / 1e9 / max(world, 1) / hbm, 4), "traffic": None,
                     "kernel": "whole step per GPU", "peak_kind": peak_kind, "algorithmic_bytes": alg_bytes},
        "cpu_baseline": None,
        "e2e": {"value": round(N / (e2e_ms * 1e-3) / 1e9, 3), "unit": "GVoxels/s",
                "h2d_bytes_per_step": 2 * dims[0] * dims[1] * (p1 - p0), "d2h_bytes_per_step": 12 * V + 16 * Q,
                "steps": e2e_steps, "note": "per rank: its planes in, its part out (rank 0's bytes shown)"},
        "gpu_launches": 6 * args.steps,
        "clocks": clk,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="noise1024", choices=sorted(WORKLOADS) + ["batch256", "served64", "shard1024"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload only: skip the batched and served summaries")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.impl == "reference":
        if args.workload == "batch256":
            run_batch_reference(args, rank)
        elif args.workload == "served64":
            run_served_reference(args, rank)
        else:
            run_reference(args, rank)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    torch.cuda.set_device(local)
    if args.workload == "shard1024":
        line = run_shard(args, rank, world, dist)
        if line:
            print(json.dumps(line), flush=True)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return
    if args.workload == "served64":
        line = run_served(args, rank, world, dist)
        if line:
            print(json.dumps(line), flush=True)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return
    if args.workload == "batch256":
        line = run_batch(args, rank, world, dist)
        if line:
            print(json.dumps(line), flush=True)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return
    import numpy as np
    import framework_gb300 as fg
    from framework_gb300 import fields
    dims, dtype, iso, desc = WORKLOADS[args.workload]
    vol, iso = make_volume(args.workload, "cuda")
    N = vol.numel()
    ex = fg.Extractor(local, algo="brick")
    V, Q = ex.extract_device(vol, iso=iso)     # no output buffers: count only
    # pre-screen: samples equal to the isovalue (the cases where the < and <=
    # tests of the reference disagree)
    if dtype == "uint16":
        u = int(iso)
        at_iso = int((vol == (u - 65536 if u >= 32768 else u)).sum()) if float(iso).is_integer() and 0 <= iso < 65536 else 0
    else:
        at_iso = int((vol == iso).sum())
    vbuf = torch.empty((max(V, 1), 3), device="cuda")
    qbuf = torch.empty((max(Q, 1), 4), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        ex.extract_device(vol, iso=iso, vertices=vbuf, quads=qbuf)
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    emit_ms, count_ms, scan_ms, step_ms = [], [], [], []
    ev0.record(stream)
    for _ in range(args.steps):
        ex.extract_device(vol, iso=iso, vertices=vbuf, quads=qbuf)
        st = ex.stats()
        emit_ms.append(st["emit_ms"]); count_ms.append(st["count_ms"]); scan_ms.append(st["scan_ms"])
        step_ms.append(st["device_ms"])
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms, total_points = combine_ranks(ev0.elapsed_time(ev1) / args.steps, N, dist, "cuda")
    st = ex.stats()

    # end to end through the host C-ABI call (dmc_run_into): pinned host
    # volume in; out into pinned host buffers what dmc::run_dmc returns,
    # vertices and triangles (and, timed separately, the quads as well)
    host_t = torch.empty(vol.shape, dtype=vol.dtype, pin_memory=True)
    host_t.copy_(vol)
    host = fields.as_u16_numpy(host_t) if dtype == "uint16" else host_t.numpy()
    hv = torch.empty((V, 3), dtype=torch.float32, pin_memory=True).numpy()
    hq = torch.empty((Q, 4), dtype=torch.int32, pin_memory=True).numpy()
    ht = torch.empty((2 * Q, 3), dtype=torch.int32, pin_memory=True).numpy()
    e2e_steps = max(1, min(args.e2e_steps, args.steps))
    for _ in range(2):   # the first call grows the context's device buffers, the second sets up the slab streams
        ex.run_into(host, hv, None, ht, iso=iso)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        nv_e, nq_e = ex.run_into(host, hv, None, ht, iso=iso)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    assert (nv_e, nq_e) == (V, Q)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        nv_e, nq_e = ex.run_into(host, hv, hq, ht, iso=iso)
    e2e_q_s = (time.perf_counter() - t0) / e2e_steps
    assert (nv_e, nq_e) == (V, Q)
    # the same through dmc_run, whose mesh the library allocates per call:
    # from the page-locked volume, and from a pageable copy, as a caller of
    # dmc::run_dmc holds it
    t0 = time.perf_counter()
    m = ex.run(host, iso=iso, triangles=True)
    run_s = time.perf_counter() - t0
    assert len(m.vertices) == V and len(m.quads) == Q
    del m
    host_pg = np.array(host)
    t0 = time.perf_counter()
    m = ex.run(host_pg, iso=iso, triangles=True)
    run_pg_s = time.perf_counter() - t0
    assert len(m.vertices) == V and len(m.quads) == Q
    del m, host_pg

    line = None
    if rank == 0:
        hbm, peak_kind = peaks()
        elem = 2 if dtype == "uint16" else 4
        alg_bytes = elem * N + 12 * V + 16 * Q
        cells = (dims[0] - 1) * (dims[1] - 1) * (dims[2] - 1) * world
        emit_avg = sum(emit_ms) / len(emit_ms)
        count_avg = sum(count_ms) / len(count_ms)
        # the dominant kernel by device time: the emit sweep on dense surfaces
        # (C3), the count sweep where the surface is small (C2, whose emit
        # sweep reads a few MB and leaves its mesh in L2)
        dom, dom_ms = ("emit", emit_avg) if emit_avg >= count_avg else ("count", count_avg)
        achieved = alg_bytes / (dom_ms * 1e-3) / 1e9
        value = total_points / (ms * 1e-3) / 1e9
        cpu = None
        if not args.no_cpu_baseline:
            v, cores, sample = cpu_oracle_sample(host, iso)
            v1, sample1 = cpu_single_thread_sample(host, iso)
            cpu = {"value": round(v, 4), "unit": "GVoxels/s", "cores": cores, "kind": "port", "sample": sample,
                   "cpu_model": cpu_model(),
                   "single_thread": {"value": round(v1, 4), "unit": "GVoxels/s", "sample": sample1}}
        line = {
            "metric": "GVoxels/s", "value": round(value, 3), "unit": "GVoxels/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u16" if dtype == "uint16" else "f32", "data": "synthetic",
            "config": {"workload": args.workload, "desc": desc, "dims": list(dims), "iso": iso,
                       "vertices": V, "quads": Q, "active_cells": st["n_active_cells"],
                       "samples_at_iso": at_iso,
                       "gcells_per_s": round(cells / (ms * 1e-3) / 1e9, 3),
                       "ms_median": round(statistics.median(step_ms), 4),
                       "algo": "brick", "l2": "input larger than L2 (no flush needed)",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "kernel_ms": {"count": round(sum(count_ms) / len(count_ms), 4),
                                     "scan": round(sum(scan_ms) / len(scan_ms), 4),
                                     "emit": round(emit_avg, 4)}},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                         "frac": round(achieved / hbm, 4), "traffic": profile_traffic(args.workload, kernel=dom),
                         "kernel": "brick_" + dom, "peak_kind": peak_kind,
                         "algorithmic_bytes": alg_bytes,
                         "kernel_traffic": {k: profile_traffic(args.workload, kernel=k) for k in ("count", "emit")},
                         "pipeline_frac": round(alg_bytes / (ms * 1e-3) / 1e9 / hbm, 4)},
            "cpu_baseline": cpu,
            "e2e": {"value": round(N / e2e_s / 1e9, 3), "unit": "GVoxels/s", "h2d_bytes_per_step": elem * N,
                    "d2h_bytes_per_step": 12 * V + 24 * Q, "steps": e2e_steps,
                    "call": "dmc_run_into, page-locked host buffers (upload, extraction and download overlapped "
                            "in z slabs); out: vertices and triangles, as dmc::run_dmc returns them",
                    "with_quads_gvox_per_s": round(N / e2e_q_s / 1e9, 3),
                    "dmc_run_gvox_per_s": round(N / run_s / 1e9, 3),
                    "dmc_run_pageable_gvox_per_s": round(N / run_pg_s / 1e9, 3)},
            "gpu_launches": 5 * args.steps,
            "clocks": clk,
        }
    ex.close()
    if not args.no_extras:
        # the batched (256 uneven volumes) and served (64-volume pool) forms, summarised
        del vol, vbuf, qbuf
        torch.cuda.empty_cache()
        sub = argparse.Namespace(**vars(args))
        sub.no_cpu_baseline = True
        sub.steps, sub.e2e_steps = min(args.steps, 10), 1
        b = run_batch(sub, rank, world, dist)
        torch.cuda.empty_cache()
        sv = run_served(sub, rank, world, dist)
        if line is not None:
            line["batched"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "e2e", "roofline", "gpu_launches")}
            line["batched"].update({k: b["config"][k] for k in ("volumes", "points", "plain_volumes_per_s",
                                                               "batched_over_plain", "single_async_volumes_per_s",
                                                               "batched_over_single_async", "autotune", "kernel_ms")})
            line["served"] = {"value": sv["value"], "unit": sv["unit"], "e2e": sv["e2e"], "gpu_launches": sv["gpu_launches"]}
            line["served"].update({k: sv["config"][k] for k in ("volumes", "pool_bytes", "served_over_plain",
                                                                "p99_ms_at_0.8_served_capacity", "sweep")})
            line["served"]["plain_capacity_rps"] = sv["config"]["plain"]["capacity_rps"]
    if line is not None:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
