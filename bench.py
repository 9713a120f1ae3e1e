"""Benchmark of the morph hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (N=1): ``shapes1024`` — 8 seeded 1024x1024 RGBA8 key frames of 40-80
overlapping ellipses/rectangles (~1M atoms per key frame), SPLINE motion plus
the Perlin motion perturbation at 2 px amplitude, PERLIN colour fading, HSP
blob delimiter.  Setup (untimed) runs the whole
pipeline on the GPU: blobs, matching, chains, refinement.  One step renders
the full morph cycle, 240 output frames at t = i/240, into device memory;
``value`` is frames/s with everything resident in HBM (frames pipelined: a
frame's binning runs beside the previous frame's resolve).  ``e2e`` renders
the same frames through the C ABI, one waited-for ``am_render`` call per
frame, into pinned HOST memory: every frame reaches host memory inside the
timed region (the resolve stores it there directly over the CPU-GPU link).
``e2e_sequence`` does the same with ``am_render_many_host``, a whole cycle per
call.  ``time_to_cost`` reports the refinement side of the metric (plain
random-pair sweeps vs the guided and learned proposals) on the same chains.

--impl reference times the reference's CPU implementation of the render on
this machine's host cores: the oracle restatement (the reference itself is
not built on this machine), every host thread rendering its own frames.
Under torchrun (N ranks) a step renders a cycle of 240 N frames, split
round-robin across the ranks (240 frames each: weak scaling, every rank's
frames span the whole morph); frames are independent, so there is no
collective on the data path, only the max over ranks of the timed region.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/s at 1024²"
UNIT = "frames/s"
WORKLOAD = "shapes1024"
FRAMES_PER_STEP = 240
SETTINGS = dict(seed=5, blob_delimiter=1, motion=4, fading=6, density=1)


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _profiled_traffic(kernel):
    """DRAM bytes per launch of `kernel` (dram__bytes_read.sum +
    dram__bytes_write.sum) from the committed ncu summary of the render
    kernels on the same workload (its per-kernel traffic table), or None."""
    path = os.path.join(ROOT, "profiles", "render_shapes1024_full.md")
    try:
        for line in open(path):
            cells = [c.strip() for c in line.strip().strip("|").split("|")]
            if len(cells) == 2 and cells[0] == f"`{kernel}`":
                return int(float(cells[1]) * 1e6)
    except (OSError, ValueError):
        pass
    return None


class Clocks:
    """nvidia-smi sampling around the timed region: sampling starts before
    it (nvidia-smi takes a moment to start) every 20 ms with timestamps, the
    region's wall-clock bounds are marked, and the summary keeps the samples
    taken inside it (the nearest one when none falls inside)."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, path):
        self.path = path
        self.p = None
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "20"], stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.5)  # let the sampler start before the region
        except Exception:
            self.p = None
        return self

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def __exit__(self, *a):
        if self.p:
            time.sleep(0.1)
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self, gpu_index=0):
        import datetime
        try:
            rows = [r.split(", ") for r in open(self.path).read().strip().splitlines()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = [r for r in rows if len(r) >= 10 and r[1].strip() == str(gpu_index)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def when(r):
            try:
                return datetime.datetime.strptime(r[0].strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                return None
        inside = rows
        if self.t0 is not None and self.t1 is not None:
            stamped = [(when(r), r) for r in rows]
            inside = [r for w, r in stamped if w is not None and self.t0 <= w <= self.t1]
            if not inside:
                later = [(w, r) for w, r in stamped if w is not None and w >= self.t0]
                inside = [min(later, key=lambda x: x[0])[1]] if later else rows[-1:]
        sm = [float(r[2]) for r in inside]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in inside:
            for n, v in zip(names, r[6:10]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(inside[0][3]), "samples": len(inside),
                "reasons": sorted(reasons)}


def physical_gpu_index(torch, dev):
    """nvidia-smi index of torch device `dev`: its PCI bus id matched against
    nvidia-smi's list (CUDA_VISIBLE_DEVICES renumbers devices; nvidia-smi does
    not).  Falls back to the visible-device list, then to `dev`."""
    try:
        pr = torch.cuda.get_device_properties(dev)
        bus = f"{pr.pci_domain_id:08X}:{pr.pci_bus_id:02X}:{pr.pci_device_id:02X}.0"
        out = subprocess.run(["nvidia-smi", "--query-gpu=index,pci.bus_id", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=20).stdout
        for line in out.strip().splitlines():
            idx, b = [c.strip() for c in line.split(",")]
            if b.upper().endswith(bus[-12:]):
                return int(idx)
    except Exception:
        pass
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    ids = [v.strip() for v in vis.split(",") if v.strip()]
    if dev < len(ids) and ids[dev].isdigit():
        return int(ids[dev])
    return dev


def setup_morph(capi, frames, refine_sweeps, motion_noise=0.0):
    m = capi.Morph()
    m.load(frames, **SETTINGS)
    if motion_noise:
        m.set(motion_noise=motion_noise)
    st = m.run_until(capi.STATE_ATOM_MORPHING)
    if st != capi.STATE_ATOM_MORPHING:
        raise RuntimeError(f"pipeline stopped in state {st}")
    if refine_sweeps:
        m.refine(refine_sweeps)
    return m


def render_roofline(m, frames_ts, torch, stream):
    """Per-kernel live CUDA-event timing over one extra cycle, and the
    algorithmic bytes of the dominant kernel.  The cycle runs with frames one
    after the other (render_pipeline 0), so each kernel's span is its own
    duration rather than its share of an overlap."""
    m.tune(render_pipeline=0)
    m.profile(True)
    buf = torch.empty((m.height, m.width, 4), dtype=torch.uint8, device="cuda")
    for t in frames_ts:
        m.render_device(float(t), buf.data_ptr())
    stream.synchronize()
    prof = m.profile_read()
    m.profile(False)
    m.tune(render_pipeline=1)
    return prof


def render_records(m, frames_ts, samples=4):
    """Binned 16-byte records per frame, averaged over `samples` frames of
    the cycle: one per atom and distinct 32 x 32 tile its positive-weight
    bilinear corners fall in (from the atoms' exact positions)."""
    total = 0
    picks = [frames_ts[(i * len(frames_ts)) // samples] for i in range(samples)]
    for t in picks:
        xy = m.positions(float(t)).astype(np.int64)
        xy = xy[xy[:, 0] >= 0]
        px, py, xf, yf = xy[:, 0] >> 8, xy[:, 1] >> 8, xy[:, 0] & 255, xy[:, 1] & 255
        n = np.ones(len(xy), np.int64)
        cx = (px % 32 == 31) & (xf > 0)   # a right corner in the next tile
        cy = (py % 32 == 31) & (yf > 0)   # a lower corner in the next tile
        n += cx.astype(np.int64) + cy.astype(np.int64) + (cx & cy).astype(np.int64)
        total += int(n.sum())
    return total // samples


def max_over_ranks(ms, world, device="cuda"):
    """Slowest rank's timed region: the whole job's throughput is measured
    against it (ranks render their own share of the frames, so this is the only
    collective of a multi-GPU run)."""
    if world == 1:
        return float(ms)
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_value(frames_per_rank, world, ms):
    """Whole-job frames/s: frames all ranks rendered over the slowest rank's time."""
    return frames_per_rank * world / (ms / 1e3)


def bench_ours(args, rank, world):
    import torch
    from atomorph_gb300 import capi, synth

    dev = 0 if world == 1 else int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(dev)
    gpu_index = physical_gpu_index(torch, dev)
    frames = synth.workload(WORKLOAD)
    atoms_per_frame = int(np.mean([synth.opaque_count(f) for f in frames]))
    m = setup_morph(capi, frames, refine_sweeps=args.refine_sweeps, motion_noise=args.motion_noise)
    N, K = m.atoms, len(frames)
    stream = torch.cuda.ExternalStream(m.stream)
    from atomorph_gb300 import shard
    ts = [m.get_time(i, FRAMES_PER_STEP * world) for i in shard.frame_indices(rank, world, FRAMES_PER_STEP)]
    out = torch.empty((FRAMES_PER_STEP, m.height, m.width, 4), dtype=torch.uint8, device="cuda")
    fb = m.height * m.width * 4

    def step():
        base = out.data_ptr()
        for i, t in enumerate(ts):
            m.render_device(float(t), base + i * fb)

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches0 = capi.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with Clocks(os.path.join(args.clocks_dir, f"clocks_rank{rank}.csv")) as clk:
        torch.cuda.synchronize()
        clk.mark_start()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        stream.synchronize()
        torch.cuda.synchronize()
        clk.mark_end()
    ms = e0.elapsed_time(e1)
    launches = capi.launch_count() - launches0
    ms = max_over_ranks(ms, world)
    value = job_value(FRAMES_PER_STEP * args.steps, world, ms)

    # e2e: same frames through the C ABI into pinned host memory
    host = torch.empty((8, m.height, m.width, 4), dtype=torch.uint8).pin_memory()
    hp = host.data_ptr()
    for i in range(min(16, len(ts))):
        m.lib.am_render(m.h, float(ts[i]), hp + (i % 8) * fb, 0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for i, t in enumerate(ts):
            rc = m.lib.am_render(m.h, float(t), hp + (i % 8) * fb, 0)
            assert rc == 0
    e2e_s = time.perf_counter() - t0
    e2e = FRAMES_PER_STEP * args.steps * world / e2e_s

    # a whole cycle per call into pinned host memory (am_render_many_host):
    # frames pipelined and stored by the GPU directly, one wait per call
    import ctypes as C
    seq_host = torch.empty((FRAMES_PER_STEP, m.height, m.width, 4), dtype=torch.uint8).pin_memory()
    ts_arr = np.ascontiguousarray(np.array(ts, np.float64))
    tp = ts_arr.ctypes.data_as(C.POINTER(C.c_double))
    assert m.lib.am_render_many_host(m.h, tp, len(ts), seq_host.data_ptr()) == 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        assert m.lib.am_render_many_host(m.h, tp, len(ts), seq_host.data_ptr()) == 0
    seq_s = time.perf_counter() - t0
    e2e_seq = FRAMES_PER_STEP * args.steps * world / seq_s

    # roofline of the dominant kernel from a profiled cycle
    prof = render_roofline(m, ts, torch, stream)
    per_frame = {k: v for k, v in prof.items() if v[1] > 0}
    dom = max(per_frame.items(), key=lambda kv: kv[1][0])
    hbm, peak_kind = _peaks()
    # Algorithmic bytes per frame (spline path): per active atom the four
    # control points (32 B) + two colours (8 B) + lag/slope (8 B) + chain rank
    # (4 B) + original index (4 B) = 56 B read once, plus the motion noise
    # pair (8 B) when the perturbation is on, plus 4 B per output pixel.
    atom_bytes = 56 + (8 if args.motion_noise else 0)
    frame_bytes = N * atom_bytes + m.width * m.height * 4
    frame_ms_profiled = sum(v[0] for v in per_frame.values() if True) / FRAMES_PER_STEP
    # in the timed cycle frames overlap (a frame's binning runs beside the
    # previous frame's resolve), so the whole-frame figure uses the timed
    # milliseconds per frame; kernel_ms_sum is the one-after-the-other sum
    frame_ms = ms / (FRAMES_PER_STEP * args.steps)
    dom_name, (dom_ms, dom_n) = dom[0], dom[1]
    dom_avg_ms = dom_ms / dom_n
    # Algorithmic bytes per launch of each frame kernel, split as the frame's
    # are counted: the binning reads the atoms' inputs once, the resolve
    # writes 4 B per output pixel.  The 16-byte records the binning writes
    # and the resolve reads are intermediate: each kernel's figure with them
    # is given beside ("with_records", records counted from the atoms' tile
    # crossings as the live frames bin them).
    recs = render_records(m, ts)
    kernel_bytes = {
        "k_frame_bin": N * atom_bytes,
        "k_frame_resolve": m.width * m.height * 4,
    }
    with_records = {"k_frame_bin": N * atom_bytes + recs * 16, "k_frame_resolve": recs * 16 + m.width * m.height * 4}

    def kernel_roof(name):
        n_l = per_frame[name][1]
        avg = per_frame[name][0] / n_l
        kb = kernel_bytes.get(name, frame_bytes)
        out = {"algorithmic_bytes_per_launch": int(kb), "avg_launch_ms": round(avg, 5),
               "achieved": round(kb / (avg / 1e3) / 1e9, 1), "frac": round(kb / (avg / 1e3) / 1e9 / hbm, 4),
               "traffic": _profiled_traffic(name)}
        if name in with_records:
            wr = with_records[name]
            out["with_records"] = {"bytes": int(wr), "achieved": round(wr / (avg / 1e3) / 1e9, 1),
                                   "frac": round(wr / (avg / 1e3) / 1e9 / hbm, 4)}
        return out

    dk = kernel_roof(dom_name)
    roof = {"kernel": dom_name, "bound": "hbm", "achieved": dk["achieved"], "peak": hbm, "unit": "GB/s",
            "frac": dk["frac"], "peak_kind": peak_kind, "traffic": dk["traffic"],
            "traffic_source": "profiles/render_shapes1024_full.md (ncu, cold cache, bytes per launch)",
            "algorithmic_bytes_per_launch": dk["algorithmic_bytes_per_launch"], "avg_launch_ms": dk["avg_launch_ms"],
            "record_bytes": f"16 B per binned record, {recs} records per frame (intermediate; see per_kernel)",
            "frame": {"algorithmic_bytes": int(frame_bytes), "ms": round(frame_ms, 5),
                      "kernel_ms_sum": round(frame_ms_profiled, 5),
                      "achieved_gbs": round(frame_bytes / (frame_ms / 1e3) / 1e9, 1),
                      "frac": round(frame_bytes / (frame_ms / 1e3) / 1e9 / hbm, 4)},
            "per_kernel": {k: kernel_roof(k) for k in ("k_frame_bin", "k_frame_resolve") if k in per_frame},
            "kernels_ms_per_frame": {k: round(v[0] / FRAMES_PER_STEP, 5) for k, v in per_frame.items()}}

    flu = None
    if rank == 0 and args.fluid_frames:
        flu = fluid_bench(m, torch, stream, args)
    ttc = None
    if rank == 0 and args.time_to_cost:
        ttc = time_to_cost(capi, frames, args)
    bat = None
    if rank == 0 and args.batch_jobs:
        bat = batch_bench(capi, args)
    c4 = None
    if rank == 0 and args.c4:
        c4 = pair_proposal(capi, args)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(m, frames, ts, args)

    res = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8/int32 fixed-point (exact integer means)",
        "data": "synthetic seeded key frames (no public dataset exists for this path)",
        "config": {"workload": WORKLOAD, "key_frames": K, "resolution": [m.width, m.height],
                   "atoms_per_key_frame": atoms_per_frame, "chain_atoms": N, "chains": m.chains,
                   "frames_per_step": FRAMES_PER_STEP, "motion": "spline", "fading": "perlin",
                   "motion_noise_px": args.motion_noise,
                   "refine_sweeps_before_render": args.refine_sweeps,
                   "l2": "per-step working set > L2 (240 output frames, 960 MB, written each step)",
                   "parallelism": (f"frames split x{world}: a cycle of {FRAMES_PER_STEP * world} frames, "
                                   f"{FRAMES_PER_STEP} per rank round-robin") if world > 1 else "1 GPU"},
        "e2e": {"value": round(e2e, 2), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": FRAMES_PER_STEP * fb},
        "e2e_sequence": {"value": round(e2e_seq, 2), "unit": UNIT, "h2d_bytes_per_step": 0,
                         "d2h_bytes_per_step": FRAMES_PER_STEP * fb,
                         "call": "am_render_many_host, 240 frames per call into pinned host memory"},
        "gpu_launches": int(launches),
        "roofline": roof,
        "clocks": clk.summary(gpu_index),
    }
    if flu is not None:
        res["fluid"] = flu
    if ttc is not None:
        res["time_to_cost"] = ttc
    if bat is not None:
        res["batch"] = bat
    if c4 is not None:
        res["learned_pairs_c4"] = c4
    if cpu is not None:
        res["cpu_baseline"] = cpu
    return res


def fluid_bench(m, torch, stream, args):
    """Fluid-on frames (the draw_fluid path the reference takes when fluid
    steps are set, morph.cpp:1417-1418) on the same chains: every frame
    manages the particles (step_fluid), runs `--fluid-steps` solver steps on
    a 512 x 512 grid (sparseness 492/1024: 1024 * s + 20 = 512 nodes per
    axis) and draws them.  The simulation is
    stateful, so frames are rendered in cycle order; timed with CUDA events
    on the render stream.  Per-part times come from one further profiled run
    of frames."""
    sparseness = 492.0 / 1024.0
    m.set(fluid=args.fluid_steps, fluid_sparseness=sparseness)
    n_frames = FRAMES_PER_STEP
    out = torch.empty((m.height, m.width, 4), dtype=torch.uint8, device="cuda")
    ts = [m.get_time(i, n_frames) for i in range(n_frames)]
    cursor = [0]

    def frames(k):
        for _ in range(k):
            m.render_device(float(ts[cursor[0] % n_frames]), out.data_ptr())
            cursor[0] += 1

    frames(max(args.warmup, 3))
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    frames(args.fluid_frames)
    e1.record(stream)
    stream.synchronize()
    ms = e0.elapsed_time(e1)
    m.profile(True)
    m.profile_read()
    frames(min(args.fluid_frames, 8))
    stream.synchronize()
    prof = m.profile_read()
    m.profile(False)
    m.set(fluid=0)
    hbm, peak_kind = _peaks()
    P = m.atoms
    gx = gy = int(round(1024 * sparseness)) + 20
    step_bytes = P * 96 + gx * gy * 104  # particle fields read 16 + written 8 (FP32); 13 node fields x2
    st_ms, st_n = prof.get("fluid_step", (0.0, 0))
    res = {"workload": WORKLOAD + " with fluid", "grid": [gx, gy], "particles": int(P),
           "steps_per_frame": args.fluid_steps, "frames": args.fluid_frames,
           "frames_per_s": round(args.fluid_frames / (ms / 1e3), 2),
           "ms_per_frame": round(ms / args.fluid_frames, 4),
           "ms_per_frame_parts": {k: round(v[0] / max(1, min(args.fluid_frames, 8)), 4) for k, v in prof.items()
                                  if k.startswith("fluid") and v[1] > 0}}
    if st_n:
        achieved = step_bytes / (st_ms / st_n / 1e3) / 1e9
        res["step_roofline"] = {"bound": "hbm", "algorithmic_bytes_per_step": int(step_bytes),
                                "avg_step_ms": round(st_ms / st_n, 5), "achieved": round(achieved, 1),
                                "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 4),
                                "peak_kind": peak_kind}
    return res


def _twin(capi, frames, w, pts, order):
    """A fresh handle with the same key frames and settings holding the given
    chains (sweep counter 0, as the original's was when they were exported)."""
    t = capi.Morph()
    t.load(frames, **SETTINGS)
    t.import_chains(w, pts, order)
    return t


def time_to_cost(capi, frames, args):
    """Refinement half of the metric on the same workload.  The plain
    random-pair refinement runs until the last `plain_window` sweeps gain
    less than `plain_conv` of the cost (or `plain_max_s` seconds): that cost
    is its converged cost C_plain.  Then each proposal kind starts from the
    same initial chains (a fresh twin handle, same seed and sweep counter) and
    runs until its cost is <= 1.005 C_plain.  All forms refine in blocks of
    `block` sweeps per am_refine call (each call also publishes the chains
    for rendering).  The learned form records its first guided sweeps, trains
    its network on them on the GPU where the recording left them
    (am_train_recorded), and continues gated; recording and training are
    inside its wall time."""
    out = {}
    B = args.block
    m = setup_morph(capi, frames, refine_sweeps=0)
    w, pts0, order = m.export_chains()
    c0 = m.cost()
    t0 = time.perf_counter()
    trace = [(0, 0.0, c0)]
    sweeps, c = 0, c0
    while True:
        g = m.refine(B, capi.PROPOSAL_RANDOM)
        sweeps += B
        c -= int(g.sum())
        trace.append((sweeps, time.perf_counter() - t0, c))
        back = next((tr for tr in reversed(trace) if tr[0] <= sweeps - args.plain_window), None)
        if back is not None and back[2] - c < args.plain_conv * c:
            break
        if trace[-1][1] > args.plain_max_s:
            break
    m.close()
    c_plain = trace[-1][2]
    target = 1.005 * c_plain
    hit = next(tr for tr in trace if tr[2] <= target)
    out["plain"] = {"converged_cost": int(c_plain), "converged_sweeps": sweeps,
                    "converged_s": round(trace[-1][1], 3), "sweeps_to_target": hit[0],
                    "s_to_target": round(hit[1], 4),
                    "ms_per_sweep": round(1e3 * trace[-1][1] / max(sweeps, 1), 4)}
    out["initial_cost"] = int(c0)
    out["target_cost"] = int(target)
    out["block"] = B
    for kind, name in ((capi.PROPOSAL_LOCAL, "local"), (capi.PROPOSAL_LEARNED, "learned")):
        t = _twin(capi, frames, w, pts0, order)
        info = {}
        t0 = time.perf_counter()
        sweeps, c = 0, c0
        if kind == capi.PROPOSAL_LEARNED:
            t.tune(learned_keep=args.learned_keep)
            t.record_swaps(args.learned_samples)
            recording = True
        while c > target and time.perf_counter() - t0 < args.proposal_max_s:
            g = t.refine(B, kind)
            sweeps += B
            c -= int(g.sum())
            if kind == capi.PROPOSAL_LEARNED and recording and t.recorded_count() >= args.learned_samples // 2:
                t1 = time.perf_counter()
                n_rec = min(t.recorded_count(), args.learned_samples)
                loss = t.train_recorded(epochs=args.learned_epochs, lr=2e-3)  # on the device-resident log
                t.record_swaps(0)
                recording = False
                info.update(trained_at_sweep=sweeps, samples=int(n_rec),
                            train_s=round(time.perf_counter() - t1, 4), loss=round(float(loss), 5))
        info.update(sweeps_to_target=sweeps, s_to_target=round(time.perf_counter() - t0, 4), cost=int(c),
                    reached=bool(c <= target))
        out[name] = info
        t.close()
    for name in ("local", "learned"):
        if out[name].get("reached"):
            out[f"speedup_{name}_vs_plain"] = round(out["plain"]["s_to_target"] / max(out[name]["s_to_target"], 1e-9), 2)
    return out


def _to_target(t, kind, target, B, max_s):
    """Refines handle t with `kind` in blocks of B sweeps until its exact cost
    is <= target (or max_s seconds); returns (sweeps, seconds, cost)."""
    c = t.cost()
    sweeps = 0
    t0 = time.perf_counter()
    while c > target and time.perf_counter() - t0 < max_s:
        g = t.refine(B, kind)
        sweeps += B
        c -= int(g.sum())
    return sweeps, time.perf_counter() - t0, c


def pair_proposal(capi, args):
    """The learned pair proposal on the C4 configuration.  Training: plain
    sweeps of a seeded 256x256 job (shapes256, job 1, about 42k atoms) log
    the outcome of every proposal (am_record_outcomes) until `--c4-samples`
    are logged, and the network trains on them where they lie
    (am_train_recorded).  Evaluation: a 512x512 job (shapes512, about 200k
    atoms): plain refinement to its converged cost C (a 2000-sweep window
    gaining < 2e-5), then every form from the same initial chains until its
    cost is <= 1.005 C: plain, guided, and the pair proposal with the network
    trained at 256x256 (training outside its time; its calls alternate with
    plain sweeps by measured gain per second).  scored_block: one block of
    scored sweeps alone from the same chains against the same number of plain
    sweeps (cost reached, milliseconds per sweep)."""
    from atomorph_gb300 import synth
    out = {"train_workload": "shapes256 (job 1)", "eval_workload": "shapes512"}
    tr = setup_morph(capi, synth.workload("shapes256", 1), 0)
    out["train_atoms"] = tr.atoms
    tr.record_outcomes(args.c4_samples, 1)
    t0 = time.perf_counter()
    sweeps = 0
    while tr.recorded_count() < args.c4_samples:
        tr.refine(50, capi.PROPOSAL_RANDOM)
        sweeps += 50
    out["log_sweeps"] = sweeps
    out["log_s"] = round(time.perf_counter() - t0, 3)
    f, y = tr.recorded_swaps(min(tr.recorded_count(), 1_000_000))
    out["accept_rate_first_1M"] = round(float(y.mean()), 4)
    t0 = time.perf_counter()
    loss = tr.train_recorded(epochs=args.c4_epochs, lr=2e-3)
    out["train_s"] = round(time.perf_counter() - t0, 3)
    out["samples"] = int(min(tr.recorded_count(), args.c4_samples))
    out["loss"] = round(float(loss), 5)
    weights = tr.proposal_weights()
    tr.close()
    frames = synth.workload("shapes512")
    m = setup_morph(capi, frames, 0)
    w, pts0, order = m.export_chains()
    out["eval_atoms"] = m.atoms
    c0 = m.cost()
    trace = [(0, 0.0, c0)]
    sweeps, c = 0, c0
    t0 = time.perf_counter()
    while True:
        g = m.refine(args.block, capi.PROPOSAL_RANDOM)
        sweeps += args.block
        c -= int(g.sum())
        trace.append((sweeps, time.perf_counter() - t0, c))
        back = next((tr_ for tr_ in reversed(trace) if tr_[0] <= sweeps - args.plain_window), None)
        if (back is not None and back[2] - c < args.plain_conv * c) or trace[-1][1] > args.plain_max_s:
            break
    m.close()
    target = 1.005 * c
    hit = next(tr_ for tr_ in trace if tr_[2] <= target)
    out["plain"] = {"converged_cost": int(c), "converged_sweeps": sweeps, "sweeps_to_target": hit[0],
                    "s_to_target": round(hit[1], 4)}
    out["initial_cost"] = int(c0)
    out["target_cost"] = int(target)
    for kind, name in ((capi.PROPOSAL_LOCAL, "guided"), (capi.PROPOSAL_SCORED, "pair_proposal")):
        t = _twin(capi, frames, w, pts0, order)
        if kind == capi.PROPOSAL_SCORED:
            t.proposal_weights(weights)
        sw, secs, cost = _to_target(t, kind, target, args.block, args.proposal_max_s)
        out[name] = {"sweeps_to_target": sw, "s_to_target": round(secs, 4), "cost": int(cost),
                     "reached": bool(cost <= target)}
        t.close()
    blk = {}
    for kind, name in ((capi.PROPOSAL_SCORED, "scored"), (capi.PROPOSAL_RANDOM, "plain")):
        t = _twin(capi, frames, w, pts0, order)
        if kind == capi.PROPOSAL_SCORED:
            t.proposal_weights(weights)
        t1 = time.perf_counter()
        g = t.refine(200, kind)
        blk[name] = {"cost": int(c0 - int(g.sum())), "ms_per_sweep": round(1e3 * (time.perf_counter() - t1) / 200, 4)}
        t.close()
    out["scored_block"] = dict(blk, sweeps=200)
    for name in ("guided", "pair_proposal"):
        if out[name]["reached"]:
            out[f"speedup_{name}_vs_plain"] = round(out["plain"]["s_to_target"] / max(out[name]["s_to_target"], 1e-9), 2)
    return out


def batch_bench(capi, args):
    """Batching workload: 32 jobs (atoms log-uniform 2k-200k, 3-8 key frames,
    128/256/512 canvases).  Each job refines `batch_sweeps` plain sweeps,
    once job by job (one am_refine per job) and once as one batch (one
    persistent launch in a replayed CUDA graph, autotuned); both start from
    the same chains with the same sweep counters, so every job's cost must
    come out identical.  Each form runs twice; the second run is timed.
    schedule: from the same initial chains, the plain/guided split the
    schedule autotuner picks for the same budget, run batched (plain sweeps
    and guided sweeps each one persistent launch per call), against the
    summed cost 200 plain sweeps reach.  Atom counts: per key frame (opaque
    pixels, C3's 2k-200k) and per chain layout (widths summed: the larger
    blob of each matched group, so up to about twice a key frame's).
    render: `batch_frames` frames per job, job by job vs batched."""
    from atomorph_gb300 import synth
    n, S = args.batch_jobs, args.batch_sweeps
    solo, twin, init = [], [], []
    t0 = time.perf_counter()
    for j in range(n):
        frames = synth.workload("batch", j)
        a = capi.Morph()
        a.load(frames, seed=j + 1, blob_delimiter=0, motion=capi.SPLINE)
        if a.run_until(capi.STATE_ATOM_MORPHING) != capi.STATE_ATOM_MORPHING:
            raise RuntimeError(f"batch job {j}: pipeline stopped early")
        b = capi.Morph()
        b.load(frames, seed=j + 1, blob_delimiter=0, motion=capi.SPLINE)
        ch = a.export_chains()
        b.import_chains(*ch)
        solo.append(a)
        twin.append(b)
        init.append((frames, j, ch))
    setup_s = time.perf_counter() - t0
    atoms = [a.atoms for a in solo]
    kf_atoms = [synth.opaque_count(f) for fr, _, _ in init for f in fr]
    keys = [a.export_chains()[2].shape[0] for a in solo]
    seq_s = []
    for _ in range(2):
        t0 = time.perf_counter()
        for a in solo:
            a.refine(S, capi.PROPOSAL_RANDOM)
        seq_s.append(time.perf_counter() - t0)
        if len(seq_s) == 1:
            cost_plain = sum(a.cost() for a in solo)
    batch = capi.Batch(twin)
    t0 = time.perf_counter()
    tuning = batch.tune(3)
    tune_s = time.perf_counter() - t0
    bat_s = []
    for _ in range(2):
        t0 = time.perf_counter()
        batch.refine(S)
        bat_s.append(time.perf_counter() - t0)
    equal = all(a.cost() == b.cost() for a, b in zip(solo, twin))
    third = []
    for frames, j, ch in init:
        c = capi.Morph()
        c.load(frames, seed=j + 1, blob_delimiter=0, motion=capi.SPLINE)
        c.import_chains(*ch)
        third.append(c)
    cost0 = sum(c.cost() for c in third)
    sb = capi.Batch(third)
    sb.set_tuning(**{k: v for k, v in tuning.items()})
    t0 = time.perf_counter()
    n_plain = sb.tune_schedule(S)
    stune_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    sb.refine_schedule(S)
    sched_s = time.perf_counter() - t0
    cost_sched = sum(c.cost() for c in third)
    sb.close()
    # the same schedule job by job (plain sweeps, then guided from the first)
    fourth = []
    for frames, j, ch in init:
        d = capi.Morph()
        d.load(frames, seed=j + 1, blob_delimiter=0, motion=capi.SPLINE)
        d.import_chains(*ch)
        d.tune(guided_switch=0)
        fourth.append(d)
    t0 = time.perf_counter()
    for d in fourth:
        if n_plain:
            d.refine(int(n_plain), capi.PROPOSAL_RANDOM)
        d.refine(int(S - n_plain), capi.PROPOSAL_LOCAL)
    sched_seq_s = time.perf_counter() - t0
    sched_equal = all(c.cost() == d.cost() for c, d in zip(third, fourth))
    for c in third + fourth:
        c.close()
    # frames: F per job at t = i / F from the refined chains (identical in
    # both sets), job by job (each job's own pipelined am_render into device
    # memory, then one device synchronisation) and batched (am_batch_render:
    # per time one binning, one resolve and one plan launch for all jobs);
    # the same into pageable host memory (am_render per frame vs one batched
    # call).  Each form runs twice; the second run is timed.
    import torch
    F = args.batch_frames
    ts = [i / F for i in range(F)]
    dev_solo = [torch.empty((F, a.height, a.width, 4), dtype=torch.uint8, device="cuda") for a in solo]
    dev_twin = [torch.empty_like(d) for d in dev_solo]
    rs_s, rb_s, hs_s, hb_s = [], [], [], []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for a, d in zip(solo, dev_solo):
            step = a.width * a.height * 4
            for i, t in enumerate(ts):
                a.render_device(t, d.data_ptr() + i * step)
        torch.cuda.synchronize()
        rs_s.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        batch.render_device(ts, [d.data_ptr() for d in dev_twin])
        rb_s.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        host_solo = [np.stack([a.render(t) for t in ts]) for a in solo]
        hs_s.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        host_twin = batch.render(ts)
        hb_s.append(time.perf_counter() - t0)
    same_dev = [bool(torch.equal(x, y)) for x, y in zip(dev_solo, dev_twin)]
    same_host = [bool(np.array_equal(x, y)) for x, y in zip(host_solo, host_twin)]
    same_dh = [bool(np.array_equal(x.cpu().numpy(), y)) for x, y in zip(dev_solo, host_solo)]
    frames_equal = all(same_dev) and all(same_host) and all(same_dh)
    pixels = sum(a.width * a.height for a in solo) * F
    render = {"frames_per_job": F, "frames": n * F, "pixels": int(pixels),
              "sequential_s": round(rs_s[1], 4), "batched_s": round(rb_s[1], 4),
              "frames_per_s_sequential": round(n * F / rs_s[1], 1), "frames_per_s_batched": round(n * F / rb_s[1], 1),
              "speedup": round(rs_s[1] / rb_s[1], 2),
              "host_sequential_s": round(hs_s[1], 4), "host_batched_s": round(hb_s[1], 4),
              "host_speedup": round(hs_s[1] / hb_s[1], 2),
              "per_job_frames_identical": bool(frames_equal)}
    if not frames_equal:
        render["jobs_differing"] = {"device": [j for j, v in enumerate(same_dev) if not v],
                                    "host": [j for j, v in enumerate(same_host) if not v],
                                    "device_vs_host": [j for j, v in enumerate(same_dh) if not v]}
    del dev_solo, dev_twin, host_solo, host_twin
    out = {"workload": f"batch ({n} jobs)", "atoms_per_key_frame_min": min(kf_atoms),
           "atoms_per_key_frame_max": max(kf_atoms), "chain_atoms_min": min(atoms), "chain_atoms_max": max(atoms),
           "atoms_total": int(sum(atoms)), "key_frames": sorted(set(keys)), "sweeps_per_job": S,
           "setup_s": round(setup_s, 2), "sequential_s": round(seq_s[1], 4), "batched_s": round(bat_s[1], 4),
           "first_batched_call_s": round(bat_s[0], 4), "tune_s": round(tune_s, 3), "tuning": tuning,
           "jobs_per_s_sequential": round(n / seq_s[1], 2), "jobs_per_s_batched": round(n / bat_s[1], 2),
           "speedup": round(seq_s[1] / bat_s[1], 2), "per_job_cost_identical": bool(equal),
           "schedule": {"plain_sweeps": int(n_plain), "guided_sweeps": int(S - n_plain), "tune_s": round(stune_s, 3),
                        "batched_s": round(sched_s, 4), "jobs_per_s": round(n / sched_s, 2),
                        "sequential_s": round(sched_seq_s, 4), "jobs_per_s_sequential": round(n / sched_seq_s, 2),
                        "per_job_cost_identical": bool(sched_equal),
                        "initial_cost_sum": int(cost0), "cost_sum": int(cost_sched),
                        "cost_sum_after_plain_sweeps": int(cost_plain),
                        "vs_plain": round(cost_sched / max(cost_plain, 1), 4)},
           "render": render,
           "jobs_per_s_refine_and_render_sequential": round(n / (seq_s[1] + rs_s[1]), 2),
           "jobs_per_s_refine_and_render_batched": round(n / (bat_s[1] + rb_s[1]), 2)}
    batch.close()
    for m in solo + twin:
        m.close()
    return out


def cpu_baseline(m, frames, ts, args):
    """The oracle restatement of the reference render, timed on one host
    thread on a bounded sample of the same frames and chains."""
    from oracle import oracle as orc
    O = orc.Oracle()
    w, pts, order = m.export_chains()
    st = _oracle_state(O, m, frames, w, pts, order)
    st["motion_noise"] = args.motion_noise
    sample = [ts[i] for i in (37, 150)][: args.cpu_frames]
    t0 = time.perf_counter()
    O.render_many(st, sample, threads=1)
    dt = time.perf_counter() - t0
    return {"value": round(len(sample) / dt, 5), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{len(sample)} frames of {WORKLOAD} (t={', '.join(f'{t:.4f}' for t in sample)}), same chains"}


def _oracle_state(O, m, frames, w, pts, order):
    from oracle import oracle as orc
    colors, present = orc.stored_frames(frames, SETTINGS["blob_delimiter"], O)
    xs, ys = [], []
    for f in frames:
        y, x = np.nonzero(f[..., 3])
        xs += [int(x.min()), int(x.max())]
        ys += [int(y.min()), int(y.max())]
    return dict(K=len(frames), width=m.width, height=m.height, bbox=np.array([min(xs), min(ys), max(xs), max(ys)]),
                seed=SETTINGS["seed"], motion=SETTINGS["motion"], fading=SETTINGS["fading"],
                delimiter=SETTINGS["blob_delimiter"], density=SETTINGS["density"], colors=colors, present=present,
                widths=w, pts=pts, blob_order=order, frame_keys=np.arange(len(frames), dtype=np.uint64))


def bench_reference(args, rank, world):
    """CPU reference arm: chains built on the CPU by the oracle (components,
    blob matching, chain construction, a few reference sweeps), then every
    step renders one frame per host thread with the oracle renderer."""
    if rank != 0:
        return None
    from atomorph_gb300 import synth
    from oracle import oracle as orc
    O = orc.Oracle()
    frames = synth.workload(WORKLOAD)
    K = len(frames)
    st = cpu_pipeline(O, frames)
    st["motion_noise"] = args.motion_noise
    threads = os.cpu_count() or 1
    ts = [i / FRAMES_PER_STEP for i in range(FRAMES_PER_STEP)]
    per_step = threads
    cursor = [0]

    def step():
        sample = [ts[(cursor[0] + j * 17) % FRAMES_PER_STEP] for j in range(per_step)]
        cursor[0] += 1
        O.render_many(st, sample, threads=threads)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    value = per_step * args.steps / dt
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 5), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 (reference arithmetic)",
        "data": "synthetic seeded key frames",
        "config": {"workload": WORKLOAD, "key_frames": K, "resolution": [1024, 1024],
                   "chain_atoms": int(np.sum(st["widths"])), "frames_per_step": per_step,
                   "motion": "spline", "fading": "perlin", "motion_noise_px": args.motion_noise,
                   "parallelism": f"{threads} host threads, one frame each"},
        "cpu_baseline": {"value": round(value, 5), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{per_step} frames per step of {WORKLOAD}, one per host thread"},
        "e2e": {"value": round(value, 5), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def cpu_pipeline(O, frames):
    """CPU restatement of the reference pipeline up to chains (components,
    blob matching, chain construction; oracle/oracle.cpp)."""
    from oracle import oracle as orc
    return orc.pipeline(O, frames, delimiter=SETTINGS["blob_delimiter"], density=SETTINGS["density"],
                        seed=SETTINGS["seed"], motion=SETTINGS["motion"], fading=SETTINGS["fading"])


def profile_case(args):
    """Every kernel of the morph path, a few launches each, on one seeded
    workload: the program the per-kernel ncu captures under profiles/ run.
    After the pipeline (components, blob matching, chain construction):
    `--refine-sweeps` plain sweeps (as the benchmark refines before it
    renders), 4 guided sweeps, 2 recorded sweeps, one training epoch, 4
    gated (learned) sweeps, the allocation-free cost, `--frames` atom frames,
    2 fluid frames with 2 solver steps each on a (0.5 W + 20)^2 grid, and one
    batched refinement and two batched frames of 4 small jobs.  Settings as
    the benchmark's."""
    import ctypes as C

    import torch
    from atomorph_gb300 import capi, synth

    keys = synth.workload(args.workload)
    m = capi.Morph()
    m.load(keys, **SETTINGS)
    if args.motion_noise:
        m.set(motion_noise=args.motion_noise)
    if m.run_until(capi.STATE_ATOM_MORPHING) != capi.STATE_ATOM_MORPHING:
        raise RuntimeError("pipeline stopped early")
    m.refine(max(args.refine_sweeps, 1), capi.PROPOSAL_RANDOM)
    m.tune(guided_switch=0)
    m.refine(4, capi.PROPOSAL_LOCAL)
    m.tune(learned_adaptive=0)
    m.record_swaps(1 << 22)  # recording sweeps run the learned form's gate with every region kept
    m.refine(2, capi.PROPOSAL_LEARNED)
    f, y = m.recorded_swaps(1 << 22)
    m.record_swaps(0)
    if not len(y):
        raise RuntimeError("no recorded samples")
    m.train_proposal(f, y, epochs=1, lr=2e-3)
    m.refine(4, capi.PROPOSAL_LEARNED)
    v = C.c_uint64()
    rc = m.lib.am_get_cost_noalloc(m.h, C.byref(v))
    if rc:
        raise RuntimeError(f"am_get_cost_noalloc: {rc}")
    out = torch.empty((m.height, m.width, 4), dtype=torch.uint8, device="cuda")
    for i in range(args.frames):
        m.render_device(m.get_time(i * 7 + 1, 240), out.data_ptr())
    m.set(fluid=2, fluid_sparseness=0.5)
    for i in range(2):
        m.render_device(m.get_time(i, 240), out.data_ptr())
    m.set(fluid=0)
    torch.cuda.synchronize()
    jobs = []
    for j in range(4):
        a = capi.Morph()
        a.load(synth.workload("batch", j), seed=j + 1, blob_delimiter=0, motion=capi.SPLINE)
        if a.run_until(capi.STATE_ATOM_MORPHING) != capi.STATE_ATOM_MORPHING:
            raise RuntimeError(f"batch job {j}: pipeline stopped early")
        jobs.append(a)
    b = capi.Batch(jobs)
    b.refine(4)
    b.render([0.1, 0.6])
    b.close()
    for a in jobs:
        a.close()
    res = {"profile_case": args.workload, "atoms": m.atoms, "cost": int(v.value), "samples": int(len(y))}
    m.close()
    return res


def profile_heavy(args):
    """A frame with a heavy tile (more than 8192 binned records): batch job
    19 (398,786 atoms, 512^2, 7 key frames) at t = 0.1875, where one tile
    holds 181,428 records, after 200 plain sweeps.  The first render resolves
    the tile with one CTA (k_frame_resolve); the plan notes it, and the next
    renders resolve it in 32 row bands (k_frame_resolve_heavy).  Serialised
    frames (render_pipeline 0).  The program of the heavy-tile ncu capture."""
    import torch
    from atomorph_gb300 import capi, synth

    j, t = 19, 0.1875
    m = capi.Morph()
    m.load(synth.workload("batch", j), seed=j + 1, blob_delimiter=0, motion=capi.SPLINE)
    if m.run_until(capi.STATE_ATOM_MORPHING) != capi.STATE_ATOM_MORPHING:
        raise RuntimeError("pipeline stopped early")
    m.refine(200, capi.PROPOSAL_RANDOM)
    m.tune(render_pipeline=0)
    out = torch.empty((m.height, m.width, 4), dtype=torch.uint8, device="cuda")
    for _ in range(args.frames):
        m.render_device(t, out.data_ptr())
    torch.cuda.synchronize()
    tiles, helpers = m.heavy_tiles()
    res = {"profile_heavy": f"batch job {j} at t={t}", "atoms": m.atoms, "heavy_tiles": tiles, "helpers": helpers}
    m.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--refine-sweeps", type=int, default=100)
    ap.add_argument("--time-to-cost", type=int, default=1)
    ap.add_argument("--block", type=int, default=20)
    ap.add_argument("--plain-window", type=int, default=2000)
    ap.add_argument("--plain-conv", type=float, default=2e-5)
    ap.add_argument("--plain-max-s", type=float, default=60.0)
    ap.add_argument("--proposal-max-s", type=float, default=30.0)
    ap.add_argument("--learned-keep", type=float, default=0.25)
    ap.add_argument("--learned-samples", type=int, default=1_000_000)
    ap.add_argument("--learned-epochs", type=int, default=1)
    ap.add_argument("--cpu-frames", type=int, default=2)
    ap.add_argument("--c4", type=int, default=1, help="run the learned pair proposal's C4 measurement")
    ap.add_argument("--c4-samples", type=int, default=20_000_000)
    ap.add_argument("--c4-epochs", type=int, default=1)
    ap.add_argument("--batch-jobs", type=int, default=32)
    ap.add_argument("--batch-sweeps", type=int, default=200)
    ap.add_argument("--batch-frames", type=int, default=16, help="frames per job in the batched render")
    ap.add_argument("--fluid-frames", type=int, default=24)
    ap.add_argument("--fluid-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--clocks-dir", default=".", help="where the nvidia-smi clock samples of the timed region go")
    ap.add_argument("--motion-noise", type=float, default=2.0,
                    help="Perlin motion perturbation amplitude in px (0 = spline paths alone)")
    ap.add_argument("--profile-case", action="store_true",
                    help="run every kernel of the path a few times on --workload (for ncu captures) and exit")
    ap.add_argument("--workload", default=WORKLOAD, help="workload of --profile-case")
    ap.add_argument("--frames", type=int, default=3, help="atom frames of --profile-case / --profile-heavy")
    ap.add_argument("--profile-heavy", action="store_true",
                    help="render a frame with a heavy tile --frames times (for ncu captures) and exit")
    args = ap.parse_args()
    if args.profile_case:
        print(json.dumps(profile_case(args)))
        return
    if args.profile_heavy:
        print(json.dumps(profile_heavy(args)))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
        res = bench_reference(args, rank, world)
    else:
        res = bench_ours(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res))
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
