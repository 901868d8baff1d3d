#!/usr/bin/env python
"""Benchmark of the so3g ProjectionEngine hot path on GB300.

Workload (default "cfg2"): CAR TQU NonTiled map 3 x 2000 x 2000 float64 at
1 arcmin, 1000 detectors (hexagonal focal plane, radius 1.5 deg) x
1,000,000 samples at 200 Hz of a constant-elevation scan (el 50 deg, az
180 +- 10 deg at 1 deg/s), signal float32 N(0,1) plus 1/f noise (knee
1 Hz).  Seeded synthetic data (numpy default_rng(0) for the focal plane,
a seeded CUDA generator for the TOD).

One step = to_map + from_map over all samples (the metric's "to_map/from_map
TOD samples/s").  value = samples per second of the step, inputs resident
in HBM; e2e = the same through the public API with host (pinned) buffers,
host<->device copies inside the timed region.  The 4 GB TOD is larger than
L2, so no L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N > 1) every rank runs an independent replica of the
workload on its own GPU (the path needs no exchange); the step time is the
max over ranks and value counts the samples of all ranks.
"""
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

CONFIGS = {
    "cfg1": dict(n_det=64, n_time=100_000, radius=1.0, shape=(600, 600), noise=False),
    "cfg2": dict(n_det=1000, n_time=1_000_000, radius=1.5, shape=(2000, 2000), noise=True),
    # HEALPix TQU nside 1024 RING (--tiled: NEST, nside_tile 16, every tile
    # present); el 45, az 180 +- 30 deg at 2 deg/s drifting 15 deg/hour.
    "cfg3": dict(kind="hp", n_det=2000, n_time=2_000_000, radius=1.5, nside=1024,
                 nside_tile=16, el=45., throw=30., v_az=2., drift=15., noise=False),
    # Differentiable from_map: ZEA bilinear TQU 3 x 3000 x 3000 at 0.5 arcmin,
    # a Gaussian field with power ~ l^-2; one step = from_map forward +
    # to_map backward through torch.autograd.
    "cfg5": dict(kind="zea_grad", n_det=4000, n_time=2_000_000, radius=1.5,
                 shape=(3000, 3000), res_arcmin=0.5, noise=False),
    # 16 observations of uneven size into one CAR 3 x 4000 x 4000 map.
    "cfg4": dict(n_obs=16, n_det=(500, 2000), n_time=(200_000, 2_000_000), el=(40., 60.),
                 az_spread=90., radius=1.5, shape=(4000, 4000), res_arcmin=1.8, noise=False),
}
METRIC = "to_map/from_map TOD samples/s (CAR TQU) mixed vs FP64 GPU path, % HBM peak"
POINTING = {"exact": 0, "certified": 1, "mixed": 2}
PRECISION = {
    "mixed": "float32 pointing with certified pixel indices (double-float, then float64, "
             "fallback), float32 spin factors and products, float64 map accumulation",
    "certified": "pointing certified equal to float64 (double-float with float64 fallback), "
                 "float32 products, float64 map accumulation",
    "exact": "float64 pointing, float32 products, float64 map accumulation",
}
ARCMIN = np.pi / 180 / 60


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="cfg2", choices=list(CONFIGS))
    ap.add_argument("--n-det", type=int, default=None)
    ap.add_argument("--n-time", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64-path", action="store_true")
    ap.add_argument("--no-precomp", action="store_true",
                    help="leave out the precomputed-pointing leg of the default line")
    ap.add_argument("--no-legs", action="store_true",
                    help="leave out the HEALPix, differentiable and batched legs")
    ap.add_argument("--ops", default="to_map,from_map",
                    help="operations timed in a step (profiling runs pick one)")
    ap.add_argument("--batch-scale", type=float, default=1.0,
                    help="cfg4: scale every observation's sample count")
    ap.add_argument("--tiled", action="store_true",
                    help="cfg3: the Tiled NEST variant; cfg1/cfg2: 100x100 tiles")
    ap.add_argument("--pointing", default="mixed", choices=["mixed", "certified", "exact"],
                    help="pointing mode of the timed steps")
    ap.add_argument("--precomp", action="store_true",
                    help="time the Precomp engine on the workload's precomputed pointing")
    return ap.parse_args()


def config(args):
    c = dict(CONFIGS[args.config])
    c.setdefault("kind", "car")
    if args.n_det:
        c["n_det"] = args.n_det
    if args.n_time:
        c["n_time"] = args.n_time
    if args.tiled and c["kind"] in ("hp", "car"):
        c["tiled"] = True
    return c


def describe(c):
    """(metric, workload name, map shape) of a configuration."""
    n = "%d det x %d samples" % (c["n_det"], c["n_time"])
    if c["kind"] == "hp":
        npix = 12 * c["nside"] ** 2
        if c.get("tiled"):
            w = "HEALPix TQU Tiled NEST nside %d (nside_tile %d) float64 map, %s" % (
                c["nside"], c["nside_tile"], n)
        else:
            w = "HEALPix TQU NonTiled RING nside %d float64 map, %s" % (c["nside"], n)
        return ("to_map/from_map TOD samples/s (HEALPix TQU)", w, [3, npix])
    shape = list(c["shape"])
    if c["kind"] == "zea_grad":
        return ("differentiable from_map forward+backward TOD samples/s (ZEA bilinear TQU)",
                "ZEA bilinear TQU NonTiled %dx%d float64 map, %s" % (shape[0], shape[1], n),
                [3] + shape)
    tiling = "Tiled (100x100 tiles, all present)" if c.get("tiled") else "NonTiled"
    return (METRIC, "CAR TQU %s %dx%d float64 map, %s" % (tiling, shape[0], shape[1], n),
            [3] + shape)


def npix_of(c):
    return 12 * c["nside"] ** 2 if c["kind"] == "hp" else c["shape"][0] * c["shape"][1]


def max_over_ranks(ms, device=None):
    """The slowest rank's step time (ms): every rank runs an independent
    replica, so the job's step ends when the last replica's does."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(samples_per_rank, world, ms):
    """Whole-job samples/s: every rank's samples over the slowest step."""
    return samples_per_rank * world / (ms * 1e-3)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def host_inputs(c, seed=0):
    """Boresight (native frame), detectors, responses and the geometry."""
    from so3g_gb300 import synth
    from so3g_gb300.proj.wcs import ProjectionistHealpix
    rng = np.random.default_rng(seed)
    dets, resp, gamma = synth.focal_plane(rng, c["n_det"], c["radius"])
    el = c.get("el", 50.)
    Q, t = synth.scan(c["n_time"], rate=200., el=el, az0=180., throw=c.get("throw", 10.),
                      v_az=c.get("v_az", 1.), drift_deg_per_hour=c.get("drift", 0.))
    kind = c.get("kind", "car")
    if kind == "hp":
        if c.get("tiled"):
            nt = 12 * c["nside_tile"] ** 2
            p = ProjectionistHealpix.for_healpix(c["nside"], nside_tile=c["nside_tile"],
                                                 active_tiles=list(range(nt)), ordering="NEST")
        else:
            p = ProjectionistHealpix.for_healpix(c["nside"], ordering="RING")
    elif kind == "zea_grad":
        p = synth.car_projectionist(c["shape"], c["res_arcmin"] * ARCMIN, el=el, az0=180.,
                                    proj="ZEA", interpol="bilinear")
    else:
        p = synth.car_projectionist(c["shape"], c.get("res_arcmin", 1.) * ARCMIN, el=el,
                                    az0=180., proj=c.get("proj", "CAR"),
                                    tile_shape=(100, 100) if c.get("tiled") else None)
    q = synth.native(p, Q)
    return p, q, dets, resp


def gaussian_field(torch, shape, dev, seed=0):
    """(3, ny, nx) float64 Gaussian random field with power ~ l^-2."""
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    ny, nx = shape
    w = torch.randn((3, ny, nx), generator=g, device=dev, dtype=torch.float64)
    ky = torch.fft.fftfreq(ny, device=dev, dtype=torch.float64)[:, None]
    kx = torch.fft.rfftfreq(nx, device=dev, dtype=torch.float64)[None, :]
    ell = torch.sqrt(ky * ky + kx * kx)
    amp = 1.0 / torch.clamp(ell, min=1.0 / max(ny, nx))
    f = torch.fft.irfft2(torch.fft.rfft2(w) * amp, s=(ny, nx))
    return (f / f.std()).contiguous()


def zero_map(m):
    for t in (m if isinstance(m, list) else [m]):
        if t is not None:
            t.zero_()


def make_signal(torch, c, dev, seed=0):
    """float32 N(0,1) TOD (+ 1/f noise, knee 1 Hz, alpha -2) on the GPU."""
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    sig = torch.randn((c["n_det"], c["n_time"]), generator=g, device=dev, dtype=torch.float32)
    if c["noise"]:
        f = torch.fft.rfftfreq(c["n_time"], d=1 / 200., device=dev)
        amp = torch.sqrt(1 + (1.0 / torch.clamp(f, min=1e-12)) ** 2)
        amp[0] = 0.
        for a in range(0, c["n_det"], 32):
            b = min(c["n_det"], a + 32)
            w = torch.randn((b - a, c["n_time"]), generator=g, device=dev, dtype=torch.float32)
            sig[a:b] += torch.fft.irfft(torch.fft.rfft(w) * amp, n=c["n_time"]).float()
    return sig


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 50 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi's start-up (NVML initialisation) can hold the GPU's
            # work queue for ~100 ms: the timed region starts after its first
            # reading, not during its start-up.
            deadline = time.time() + 5.
            while not self.lines and time.time() < deadline and self.proc.poll() is None:
                time.sleep(0.01)
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
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


# DRAM bytes per sample (dram__bytes_read.sum + dram__bytes_write.sum / samples)
# of one ncu capture of the to_map and from_map kernels, CAR TQU 3x2000x2000,
# 200 det x 1M samples, per pointing mode (profiles/to_map_from_map_*_car_
# tqu_200det_1M.md; mixed: the chunked main kernels k_scatter_ix4 and
# k_from_map_ix4).  The traffic is the signal (4 B read, from_map also 4 B
# written) and the boresight per detector, so it scales with the samples.
MEASURED_TRAFFIC_PER_SAMPLE = {
    "certified": {"to_map": (834.33e6 + 3.78e6) / 2e8,
                  "from_map": (835.40e6 + 747.14e6) / 2e8},
    "mixed": {"to_map": (807.045e6 + 13.405e6) / 2e8,
              "from_map": (806.769e6 + 790.061e6) / 2e8},
}
# Float64-pipe lane operations per sample of the float64 path's to_map
# (ncu sm__inst_executed_pipe_fp64.sum x 32 / samples, 200 detectors x 1M)
# and the float64 FMA rate measured on a GB300 (1.6 lane-ops/clock/SM).
FP64_OPS_PER_SAMPLE_TO_MAP = 1.018354e9 * 32 / 2e8
FP64_LANE_OPS_PER_S = 5.0e11
# The same for the Precomp kernels (ncu, 100 detectors x 1M samples; from_map:
# k_pc_from_map4, the per-call map split's 0.17 GB left out).
MEASURED_TRAFFIC_PRECOMP = {"to_map": (2.400927e9 + 3.107e6) / 1e8,
                            "from_map": (2.401793e9 + 391.814e6) / 1e8}


def algorithmic_bytes(c, op):
    """Compulsory bytes per (det, sample) of an operation (map of
    3 x npix float64)."""
    n_det, n_time = c["n_det"], c["n_time"]
    N = n_det * n_time
    npix = npix_of(c)
    bore = 32. / n_det
    dets = 16. / n_time
    if op == "to_map":
        return 4. + bore + dets + 16. * 3 * npix / N
    if op == "from_map":
        return 8. + bore + dets + 8. * 3 * npix / N   # signal read + write
    if op == "to_weight_map":
        return bore + dets + 16. * 6 * npix / N
    if op == "from_map_fwd_bwd":
        # from_map (signal out) + to_map of the signal gradient
        return algorithmic_bytes(c, "from_map") - 4. + algorithmic_bytes(c, "to_map")
    raise ValueError(op)


# ---------------------------------------------------------------------------
# Our implementation.

def run_ours(args, c, rank, world, lean=False):
    """Times args.steps steps of the workload on this rank's GPU; lean:
    the timed steps only (no certified / float64 / accuracy / weight-map /
    end-to-end side measurements)."""
    import torch
    import so3g_gb300
    from so3g_gb300 import _abi

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    lib = _abi.lib()
    p, q, dets, resp = host_inputs(c)
    eng = p.get_ProjEng("TQU")
    q_d = torch.from_numpy(q).to(dev)
    dets_d = torch.from_numpy(dets).to(dev)
    resp_d = torch.from_numpy(resp).to(dev)
    sig = make_signal(torch, c, dev, seed=rank)
    m = eng.zeros(3, device=dev)
    w = eng.zeros((3, 3), device=dev)
    out = torch.zeros_like(sig)
    N = c["n_det"] * c["n_time"]
    ops = args.ops.split(",")
    stream = torch.cuda.current_stream()
    if c["kind"] == "zea_grad":
        from so3g_gb300 import autograd
        field = gaussian_field(torch, c["shape"], dev, seed=rank)
        ops = ["from_map_fwd_bwd"]

    def step(accum, ev=None):
        t = {}
        if "from_map_fwd_bwd" in ops:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            mm = field.detach().requires_grad_(True)
            e0.record(stream)
            s_ = autograd.from_map(eng, mm, q_d, dets_d, resp_d)
            s_.backward(sig)
            e1.record(stream)
            t["from_map_fwd_bwd"] = (e0, e1)
        if "to_map" in ops:
            zero_map(m)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.to_map(m, q_d, dets_d, resp_d, sig, None, None, accum=accum)
            e1.record(stream)
            t["to_map"] = (e0, e1)
        if "from_map" in ops:
            out.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.from_map(m, q_d, dets_d, resp_d, out)
            e1.record(stream)
            t["from_map"] = (e0, e1)
        return t

    def timed(accum, steps, warmup, pointing=_abi.POINTING_CERTIFIED):
        eng.pointing = pointing
        for _ in range(warmup):
            step(accum)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        n0 = lib.so3g_launch_count()
        e_start = torch.cuda.Event(enable_timing=True)
        e_end = torch.cuda.Event(enable_timing=True)
        per = {op: [] for op in ops}
        with ClockSampler(dev.index) as clk:
            torch.cuda.nvtx.range_push("timed")
            e_start.record(stream)
            for _ in range(steps):
                t = step(accum)
                for op, ev in t.items():
                    per[op].append(ev)
            e_end.record(stream)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_pop()
        if world > 1:
            torch.distributed.barrier()
        launches = lib.so3g_launch_count() - n0
        total_ms = e_start.elapsed_time(e_end)
        op_ms = {op: float(np.mean([a.elapsed_time(b) for a, b in v])) for op, v in per.items()}
        return total_ms / steps, op_ms, launches, clk.summary()

    mode = POINTING[args.pointing]
    ms, op_ms, launches, clocks = timed(_abi.ACCUM_WARP_RUNS, args.steps, args.warmup,
                                        pointing=mode)
    ms = max_over_ranks(ms, dev)
    res = {"ms_per_step": ms, "op_ms": op_ms, "launches": launches, "clocks": clocks}
    if lean:
        del sig, out
        return res, N
    if world == 1 and c["kind"] != "zea_grad" and mode != _abi.POINTING_CERTIFIED:
        # The bit-exact certified mode, for comparison.
        msc, opc, _, _ = timed(_abi.ACCUM_WARP_RUNS, max(1, args.steps // 2), 1,
                               pointing=_abi.POINTING_CERTIFIED)
        res["certified"] = {"ms_per_step": msc, "op_ms": opc}
    if not args.no_fp64_path and world == 1 and c["kind"] == "car":
        # The plain float64 GPU path: exact float64 pointing, one float64
        # atomic per term.
        ms64, op64, _, _ = timed(_abi.ACCUM_ATOMIC, max(1, args.steps // 2), 1,
                                 pointing=_abi.POINTING_EXACT)
        res["fp64_path"] = {"ms_per_step": ms64, "op_ms": op64}
    if world == 1 and c["kind"] != "zea_grad" and mode != _abi.POINTING_EXACT:
        # Accuracy of the timed mode against the float64 path on this
        # workload: to_map maps, and from_map signals of the same map.
        eng.pointing = _abi.POINTING_EXACT
        m_ex = eng.to_map(eng.zeros(3, device=dev), q_d, dets_d, resp_d, sig, None, None)
        s_ex = eng.from_map(m_ex, q_d, dets_d, resp_d, None)
        eng.pointing = mode
        m_md = eng.to_map(eng.zeros(3, device=dev), q_d, dets_d, resp_d, sig, None, None)
        s_md = eng.from_map(m_ex, q_d, dets_d, resp_d, None)

        def rel(a, b):
            if isinstance(a, list):
                a = torch.cat([t.reshape(-1) for t in a])
                b = torch.cat([t.reshape(-1) for t in b])
            return float((a.double() - b.double()).abs().max() / a.double().abs().max())
        res["accuracy"] = {"to_map_max_rel_err": rel(m_ex, m_md),
                           "from_map_max_rel_err": rel(s_ex, s_md),
                           "reference": "float64 GPU path (exact pointing)"}
        del m_ex, s_ex, m_md, s_md
    eng.pointing = mode
    # to_weight_map, timed on its own (not part of the step).
    if world == 1:
        for _ in range(2):
            zero_map(w)
            eng.to_weight_map(w, q_d, dets_d, resp_d, None, None)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.to_weight_map(w, q_d, dets_d, resp_d, None, None)
        e1.record(stream)
        torch.cuda.synchronize()
        res["to_weight_map_ms"] = e0.elapsed_time(e1)
    if not args.no_e2e and world == 1 and c["kind"] == "car" and not c.get("tiled"):
        res["e2e"] = run_e2e(args, c, eng, q, dets, resp, sig, dev)
    del sig, out
    return res, N


# Page-locked host <-> device copy rates of a GB300 machine (torch copies of a
# 4 GiB buffer, one to eight concurrent streams alike): 209-211 GB/s to the
# device, 192-193 GB/s back; 171 GB/s each way when both run at once.
HOST_COPY_GBS = {"h2d": 210.0, "d2h": 193.0}


def run_e2e(args, c, eng, q, dets, resp, sig_dev, dev):
    """Same step through the public API with pinned host buffers."""
    import torch
    sig_h = torch.empty(sig_dev.shape, dtype=torch.float32, pin_memory=True)
    sig_h.copy_(sig_dev)
    q_h = torch.from_numpy(q).pin_memory()
    d_h = torch.from_numpy(dets).pin_memory()
    r_h = torch.from_numpy(resp).pin_memory()
    ny, nx = c["shape"]
    m_h = torch.zeros((3, ny, nx), dtype=torch.float64).pin_memory()

    parts = {"to_map": [], "from_map": []}

    def step():
        # to_map of the host signal into the host map, then from_map of that
        # map into a new host signal (signal=None, as a map-maker's P m).
        m_h.zero_()
        t0 = time.perf_counter()
        eng.to_map(m_h, q_h, d_h, r_h, sig_h, None, None)
        t1 = time.perf_counter()
        out = eng.from_map(m_h, q_h, d_h, r_h, None)
        t2 = time.perf_counter()
        assert len(out) == sig_h.shape[0]
        parts["to_map"].append((t1 - t0) * 1e3)
        parts["from_map"].append((t2 - t1) * 1e3)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    # Every step is timed on its own.  The value is the mean step (all the
    # timed steps' wall time over their count): the host link of these
    # shared hosts stalls now and then for 30-200 ms (plain torch copies
    # show the same), and those stalls are part of what a caller sees.  The
    # median step, without them, is reported beside it.
    steps = max(3, args.steps)
    for v in parts.values():
        v.clear()
    per_step = []
    for _ in range(steps):
        t0 = time.perf_counter()
        step()
        torch.cuda.synchronize()
        per_step.append(time.perf_counter() - t0)
    dt = float(np.mean(per_step))
    N = c["n_det"] * c["n_time"]
    nb_sig = sig_h.numel() * 4
    nb_map = m_h.numel() * 8
    nb_point = q_h.numel() * 8 + d_h.numel() * 8 + r_h.numel() * 4
    # to_map: signal, map and pointing in, map out; from_map: map and
    # pointing in, the new signal out.
    h2d = nb_sig + nb_map + nb_point + nb_map + nb_point
    d2h = nb_map + nb_sig
    from so3g_gb300 import projeng
    # The host link bounds this step: to_map's upload has to finish before
    # from_map can read the map it made, so the two directions run one
    # after the other at the copy engines' rate.
    link_ms = (h2d / HOST_COPY_GBS["h2d"] + d2h / HOST_COPY_GBS["d2h"]) / 1e6
    return {"value": N / dt, "unit": "samples/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "ms_per_step": dt * 1e3,
            "ms_per_step_median": float(np.median(per_step)) * 1e3,
            "ms_steps": [round(x * 1e3, 2) for x in per_step],
            "estimator": "mean of %d individually timed steps" % steps,
            "host_link": {"bound": "host<->device copies, one direction after the other",
                          "copy_gbs": HOST_COPY_GBS, "bound_ms": link_ms,
                          "frac_median_step": link_ms / (float(np.median(per_step)) * 1e3),
                          "frac_mean_step": link_ms / (dt * 1e3)},
            "op_ms": {k: float(np.median(v)) for k, v in parts.items()},
            "step": "to_map(host map, page-locked host signal) + from_map(host map, "
                    "signal=None) -> new host signal",
            "host_signal": "policy %s: to_map input %s" % (
                projeng.host_signal_policy(),
                "used in place" if projeng._host_direct(sig_h, False) else "streamed")}


# ---------------------------------------------------------------------------
# Precomputed pointing: ProjEng_Precomp on the workload's pointing matrix.

def precomp_leg(c, steps, warmup):
    """ProjEng_Precomp to_map + from_map on the workload's precomputed
    pointing (pixel indices and spin factors from pointing_matrix, computed
    once and timed on its own): the form a map-maker iterating over the same
    observation uses.  Returns the timings and the HBM roofline."""
    import torch
    import so3g_gb300
    from so3g_gb300 import _abi
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    lib = _abi.lib()
    p, q, dets, resp = host_inputs(c)
    eng = p.get_ProjEng("TQU")
    q_d, dets_d, resp_d = (torch.from_numpy(x).to(dev) for x in (q, dets, resp))
    stream = torch.cuda.current_stream()
    eng.pointing_matrix(q_d, dets_d, resp_d)    # warm-up
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    pix, spin = eng.pointing_matrix(q_d, dets_d, resp_d)
    e1.record(stream)
    torch.cuda.synchronize()
    pm_ms = e0.elapsed_time(e1)
    del q_d
    sig = make_signal(torch, c, dev)
    pc = so3g_gb300.ProjEng_Precomp_NonTiled()
    m = torch.zeros((3,) + tuple(c["shape"]), dtype=torch.float64, device=dev)
    out = torch.zeros_like(sig)
    N = c["n_det"] * c["n_time"]

    def step(ev):
        m.zero_()
        ev[0].record(stream)
        pc.to_map(m, pix, spin, sig)
        ev[1].record(stream)
        out.zero_()
        ev[2].record(stream)
        pc.from_map(m, pix, spin, out)
        ev[3].record(stream)

    for _ in range(warmup):
        step([torch.cuda.Event(enable_timing=True) for _ in range(4)])
    torch.cuda.synchronize()
    n0 = lib.so3g_launch_count()
    evs = []
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        torch.cuda.nvtx.range_push("precomp_timed")
        e0.record(stream)
        for _ in range(steps):
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            step(ev)
            evs.append(ev)
        e1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    launches = lib.so3g_launch_count() - n0
    ms = e0.elapsed_time(e1) / steps
    tm = float(np.mean([a.elapsed_time(b) for a, b, _, _ in evs]))
    fm = float(np.mean([a.elapsed_time(b) for _, _, a, b in evs]))
    npix = c["shape"][0] * c["shape"][1]
    # Compulsory bytes per sample: pixel (2 int32) + spin (3 float32) +
    # signal (4, read; from_map also writes it) + the map once.
    b_tm = 8. + 12. + 4. + 16. * 3 * npix / N
    b_fm = 8. + 12. + 8. + 8. * 3 * npix / N
    hbm, kind = peaks()
    ach_tm = b_tm * N / (tm * 1e-3) / 1e9
    ach_fm = b_fm * N / (fm * 1e-3) / 1e9
    del pix, spin, sig, out, m
    return {"value": N / (ms * 1e-3), "ms_per_step": ms, "op_ms": {"to_map": tm, "from_map": fm},
            "pointing_matrix_ms": pm_ms,
            "roofline": {"bound": "hbm", "kernel": "precomp from_map", "achieved": ach_fm,
                         "peak": hbm, "unit": "GB/s", "frac": ach_fm / hbm,
                         "traffic": MEASURED_TRAFFIC_PRECOMP["from_map"] * N,
                         "bytes_per_sample": b_fm, "peak_kind": kind,
                         "to_map": {"achieved": ach_tm, "frac": ach_tm / hbm,
                                    "traffic": MEASURED_TRAFFIC_PRECOMP["to_map"] * N,
                                    "bytes_per_sample": b_tm}},
            "clocks": clk.summary(), "gpu_launches": int(launches)}


def run_precomp(args, c):
    r = precomp_leg(c, args.steps, args.warmup)
    N = c["n_det"] * c["n_time"]
    metric, workload, map_shape = describe(c)
    line = {"metric": "Precomp to_map/from_map TOD samples/s (CAR TQU, precomputed pointing)",
            "value": r["value"], "unit": "samples/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload + ", pointing precomputed (ProjEng_Precomp)",
                       "n_det": c["n_det"], "n_time": c["n_time"], "map": map_shape,
                       "step": "Precomp to_map + from_map",
                       "l2": "inputs larger than L2 (pointing + TOD %.1f GB)" % (N * 24 / 1e9),
                       "parallelism": "single GPU"},
            "op_ms": r["op_ms"], "pointing_matrix_ms": r["pointing_matrix_ms"],
            "roofline": r["roofline"], "clocks": r["clocks"], "gpu_launches": r["gpu_launches"]}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# Batched map-making input: many observations into one map.

def batch_inputs(c, scale=1.0, seed=0):
    """Projectionist and per-observation host inputs (boresight in the
    map's native frame, detectors, responses) of the batched workload."""
    from so3g_gb300 import synth
    rng = np.random.default_rng(seed)
    ny, nx = c["shape"]
    p = synth.car_projectionist((ny, nx), c["res_arcmin"] * ARCMIN, el=50., az0=180.)
    obs = []
    for i in range(c["n_obs"]):
        nd = int(rng.integers(c["n_det"][0], c["n_det"][1] + 1))
        nt = max(1, int(int(rng.integers(c["n_time"][0], c["n_time"][1] + 1)) * scale))
        el = float(rng.uniform(*c["el"]))
        az0 = 180. + float(rng.uniform(-0.5, 0.5)) * c["az_spread"]
        dets, resp, _ = synth.focal_plane(rng, nd, c["radius"])
        Q, _ = synth.scan(nt, rate=200., el=el, az0=az0, throw=10., v_az=1.)
        obs.append((synth.native(p, Q), dets, resp))
    return p, obs


def run_batch(args, c):
    """One step = to_map + to_weight_map of every observation into one
    map (zeroed first), as one CUDA graph of two persistent batched
    launches with autotuned launch shapes; compared against one plain
    to_map + to_weight_map call per observation."""
    import torch
    from so3g_gb300 import _abi
    from so3g_gb300.batch import Observation, ObservationBatch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    lib = _abi.lib()
    p, hobs = batch_inputs(c, args.batch_scale)
    eng = p.get_ProjEng("TQU")
    eng.pointing = POINTING[args.pointing]
    g = torch.Generator(device=dev)
    g.manual_seed(0)
    obs = []
    for q, dets, resp in hobs:
        sig = torch.randn((dets.shape[0], q.shape[0]), generator=g, device=dev,
                          dtype=torch.float32)
        obs.append(Observation(torch.from_numpy(q).to(dev), torch.from_numpy(dets).to(dev),
                               torch.from_numpy(resp).to(dev), sig))
    N = sum(o.signal.numel() for o in obs)
    b = ObservationBatch(eng, obs)
    tune = {}
    for weight in (False, True):
        piece, blocks = b.tune(weight=weight, pieces=(8192, 32768),
                               blocks_per_sm=(0, -1), reps=1, store=False)
        tune["to_weight_map" if weight else "to_map"] = {
            "piece": piece, "blocks": blocks, "log": b.tune_log}
    ny, nx = c["shape"]
    m = torch.zeros((3, ny, nx), dtype=torch.float64, device=dev)
    w = torch.zeros((3, 3, ny, nx), dtype=torch.float64, device=dev)
    t_m, t_w = tune["to_map"], tune["to_weight_map"]
    graph = b.graph(m, w, map_shape=(t_m["piece"], t_m["blocks"]),
                    weight_shape=(t_w["piece"], t_w["blocks"]))
    stream = torch.cuda.current_stream()

    def step():
        m.zero_()
        w.zero_()
        graph.replay()

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(dev.index) as clk:
            e0.record(stream)
            for _ in range(steps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, clk.summary()

    ms, clocks = timed(step, args.steps, args.warmup)
    graph.check()
    m_batch = m.clone()

    def sequential():
        m.zero_()
        w.zero_()
        for o in obs:
            eng.to_map(m, o.boresight, o.dets, o.response, o.signal, None, None)
            eng.to_weight_map(w, o.boresight, o.dets, o.response, None, None)

    n0 = lib.so3g_launch_count()
    ms_seq, _ = timed(sequential, max(1, args.steps // 2), 1)
    seq_launches = (lib.so3g_launch_count() - n0) // (max(1, args.steps // 2) + 1)
    err = float((m - m_batch).abs().max() / m_batch.abs().max())

    # to_map batch alone, for the roofline.
    def to_map_only():
        b.to_map(m, piece=t_m["piece"], blocks=t_m["blocks"])
    ms_tm, _ = timed(to_map_only, 2, 1)
    npix = ny * nx
    bytes_tm = sum(4. * o.signal.numel() + 32. * o.boresight.shape[0] + 16. * o.dets.shape[0]
                   for o in obs) + 16. * 3 * npix
    hbm, kind = peaks()
    achieved = bytes_tm / (ms_tm * 1e-3) / 1e9
    sizes = [[int(o.dets.shape[0]), int(o.boresight.shape[0])] for o in obs]
    cfg = {"workload": "16 observations (det 500-2000, samples 200k-2M) into one CAR TQU "
                       "3x%dx%d float64 map" % (ny, nx),
           "n_obs": len(obs), "samples": N, "sizes": sizes, "batch_scale": args.batch_scale,
           "step": "to_map + to_weight_map, one CUDA graph with the tuned launches",
           "pointing": args.pointing,
           "l2": "inputs larger than L2 (TOD %.1f GB)" % (N * 4 / 1e9),
           "parallelism": "single GPU"}
    line = {"metric": "batched to_map + to_weight_map TOD samples/s (CAR TQU, 16 obs)",
            "value": N / (ms * 1e-3), "unit": "samples/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": cfg, "tuned": {k: {"piece": v["piece"], "blocks": v["blocks"]}
                                     for k, v in tune.items()},
            "tune_log": {k: v["log"] for k, v in tune.items()},
            "sequential": {"value": N / (ms_seq * 1e-3), "ms_per_step": ms_seq,
                           "launches_per_step": int(seq_launches),
                           "batched_speedup": ms_seq / ms,
                           "max_rel_map_diff": err},
            "roofline": {"bound": "hbm", "kernel": "to_map batch", "achieved": achieved,
                         "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "traffic": None,
                         "peak_kind": kind, "to_map_ms": ms_tm},
            "clocks": clocks, "gpu_launches": graph.launches * args.steps}
    return line


# ---------------------------------------------------------------------------
# The other workloads, as legs of the default line.

def _free_gpu():
    import gc
    import torch
    gc.collect()
    torch.cuda.empty_cache()


def workload_leg(args, name, steps=3, warmup=3):
    """The mixed-pointing step of workload `name` (cfg3: HEALPix to_map +
    from_map; cfg5: differentiable from_map forward + backward) at full
    size, with its HBM roofline."""
    a = argparse.Namespace(**vars(args))
    a.config, a.steps, a.warmup, a.tiled, a.pointing = name, steps, warmup, False, "mixed"
    a.ops = "to_map,from_map"
    c = config(a)
    _free_gpu()
    res, N = run_ours(a, c, 0, 1, lean=True)
    _free_gpu()
    metric, workload, map_shape = describe(c)
    hbm, kind = peaks()
    op = "from_map_fwd_bwd" if c["kind"] == "zea_grad" else "to_map"
    B = algorithmic_bytes(c, op)
    ach = B * N / (res["op_ms"][op] * 1e-3) / 1e9
    return {"metric": metric, "workload": workload, "value": N / (res["ms_per_step"] * 1e-3),
            "unit": "samples/s", "steps": steps, "warmup": warmup,
            "ms_per_step": res["ms_per_step"], "op_ms": res["op_ms"],
            "roofline": {"bound": "hbm", "kernel": op, "achieved": ach, "peak": hbm,
                         "unit": "GB/s", "frac": ach / hbm, "traffic": None,
                         "bytes_per_sample": B, "peak_kind": kind},
            "clocks": res["clocks"], "gpu_launches": int(res["launches"])}


def batch_leg(args, steps=3, warmup=3):
    """cfg4: 16 observations into one map, the tuned graph against 16
    sequential plain calls."""
    a = argparse.Namespace(**vars(args))
    a.steps, a.warmup, a.pointing, a.batch_scale = steps, warmup, "mixed", 1.0
    _free_gpu()
    line = run_batch(a, dict(CONFIGS["cfg4"]))
    _free_gpu()
    for k in ("tune_log", "n_gpus", "vs_baseline", "data", "dtype", "scaling",
              "higher_is_better"):
        line.pop(k, None)
    return line


# ---------------------------------------------------------------------------
# CPU: the oracle (the reference's algorithm restated in C++ with OpenMP).

def cpu_signal(c, seed=0):
    """float32 N(0,1) TOD (+ 1/f noise, knee 1 Hz, alpha -2) on the host
    (torch's CPU generator and FFT, all host threads)."""
    import torch
    g = torch.Generator()
    g.manual_seed(seed)
    sig = torch.randn((c["n_det"], c["n_time"]), generator=g, dtype=torch.float32)
    if c.get("noise"):
        f = torch.fft.rfftfreq(c["n_time"], d=1 / 200.)
        amp = torch.sqrt(1 + (1.0 / torch.clamp(f, min=1e-12)) ** 2)
        amp[0] = 0.
        for a in range(0, c["n_det"], 64):
            b = min(c["n_det"], a + 64)
            w = torch.randn((b - a, c["n_time"]), generator=g, dtype=torch.float32)
            sig[a:b] += torch.fft.irfft(torch.fft.rfft(w) * amp, n=c["n_time"]).float()
    return sig.numpy()


def _simple_threads(orc, pz, q, dets, n_domain, chunk=50):
    """The reference's 'simple' thread assignment (pixel_ranges with
    n_domain stripes, src/Projection.cxx:1440-1541) as [parallel bunch,
    serial bunch] of per-thread, per-detector interval lists, built
    detector chunk by chunk (the labels of the whole workload would take
    4 bytes per sample)."""
    n_det = len(dets)
    par = [[None] * n_det for _ in range(n_domain)]
    ser = [[None] * n_det]
    for a in range(0, n_det, chunk):
        b = min(n_det, a + chunk)
        lab = orc.labels(pz, q, np.ascontiguousarray(dets[a:b]), 0, n_domain)
        th = _labels_to_threads(lab, n_domain)
        for k in range(n_domain):
            par[k][a:b] = th[0][k]
        ser[0][a:b] = th[1][0]
    return [par, ser]


class CpuWorkload:
    """The oracle (the reference's ProjectionEngine arithmetic restated in
    C++ with OpenMP) on the whole workload, on all host cores."""

    def __init__(self, c, threads=None):
        from oracle import Oracle
        self.orc = Oracle()
        self.threads = threads or os.cpu_count() or 1
        self.orc.set_threads(self.threads)
        s = dict(c)
        s["tiled"] = False        # the oracle runs the untiled map
        self.c = s
        p, self.q, self.dets, self.resp = host_inputs(s)
        self.pz = p.get_ProjEng("TQU")._pz()
        self.sig = cpu_signal(s)
        self.npix = npix_of(c)
        self.out = np.zeros((s["n_det"], s["n_time"]), np.float32)
        self.m = np.zeros(3 * self.npix)
        t0 = time.perf_counter()
        self.ranges = self.orc.schedule(
            _simple_threads(self.orc, self.pz, self.q, self.dets, self.threads),
            len(self.dets))
        self.assign_s = time.perf_counter() - t0

    def step(self, simple=True):
        """to_map (with the 'simple' thread assignment, or thread_intervals
        = None: one thread, the reference's default) + from_map (OpenMP over
        detectors); returns the seconds of each."""
        self.m[:] = 0
        t0 = time.perf_counter()
        self.orc.to_map(self.pz, self.q, self.dets, self.resp, self.sig, None, self.m,
                        threads=self.ranges if simple else None)
        t1 = time.perf_counter()
        self.out[:] = 0
        self.orc.from_map(self.pz, self.q, self.dets, self.resp, self.m, self.out)
        t2 = time.perf_counter()
        return t1 - t0, t2 - t1

    @property
    def samples(self):
        return self.c["n_det"] * self.c["n_time"]

    def describe(self):
        return ("the whole workload (%d det x %d samples) per step; to_map with the "
                "reference's 'simple' thread assignment over %d threads (assignment %.1f s, "
                "made once, not timed), from_map over %d threads" % (
                    self.c["n_det"], self.c["n_time"], self.threads, self.assign_s,
                    self.threads))


class _R:
    """Minimal Ranges view for oracle.schedule()."""

    def __init__(self, iv):
        self.iv = iv
        self.count = 0

    def ranges(self):
        return np.asarray(self.iv, dtype=np.int32).reshape(-1, 2)


def _labels_to_threads(lab, n_domain):
    """Per-sample stripe labels -> [parallel bunch, serial bunch] of
    per-thread, per-detector interval lists (pixel_ranges'
    construction, src/Projection.cxx:1507-1523)."""
    n_det, n_time = lab.shape
    par = [[[] for _ in range(n_det)] for _ in range(n_domain)]
    ser = [[[] for _ in range(n_det)]]
    for d in range(n_det):
        row = lab[d]
        edges = np.flatnonzero(np.diff(row)) + 1
        starts = np.concatenate([[0], edges])
        ends = np.concatenate([edges, [n_time]])
        for a, b in zip(starts, ends):
            L = row[a]
            if L < 0:
                continue
            (par[L] if L < n_domain else ser[0])[d].append((a, b))
    return [[[_R(iv) for iv in th] for th in par], [[_R(iv) for iv in th] for th in ser]]


def run_reference(args, c, cfg, metric, world):
    """The reference arm: the oracle on the whole workload, W warm-up
    steps, then K timed steps; the median step gives the value."""
    w = CpuWorkload(c)
    for _ in range(args.warmup):
        w.step()
    per = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        a, b = w.step()
        per.append((time.perf_counter() - t0, a, b))
    total = time.perf_counter() - t_all
    ms = float(np.median([x[0] for x in per])) * 1e3
    value = w.samples / (ms * 1e-3)
    line = {"metric": metric, "value": value, "unit": "samples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg, "impl": "reference",
            "op_ms": {"to_map": float(np.median([x[1] for x in per])) * 1e3,
                      "from_map": float(np.median([x[2] for x in per])) * 1e3},
            "ms_per_step_mean": total / max(1, args.steps) * 1e3,
            "estimator": "median of %d steps after %d warm-up steps" % (args.steps, args.warmup),
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": w.threads,
                             "kind": "port", "sample": w.describe()},
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def cpu_baseline(c):
    """One step of the oracle on the whole workload with the 'simple'
    thread assignment, and one with thread_intervals = None (to_map on one
    thread, as the reference runs it by default)."""
    w = CpuWorkload(c)
    w.step()                                   # warm-up (page faults, caches)
    a, b = w.step()
    a1, b1 = w.step(simple=False)
    return {"value": w.samples / (a + b), "unit": "samples/s", "cores": w.threads,
            "kind": "port", "sample": w.describe() + "; one step after one warm-up step",
            "op_s": {"to_map": a, "from_map": b},
            "value_default_threads": w.samples / (a1 + b1),
            "default_threads": "to_map with thread_intervals=None (one thread, the "
                               "reference's default): %.1f s; from_map over %d threads" % (
                                   a1, w.threads)}


# ---------------------------------------------------------------------------

def main():
    args = parse()
    if args.config == "cfg4" and args.impl == "ours":
        print(json.dumps(run_batch(args, dict(CONFIGS["cfg4"]))))
        return
    c = config(args)
    if args.precomp and args.impl == "ours":
        return run_precomp(args, c)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    metric, workload, map_shape = describe(c)
    step_name = ("from_map forward + to_map backward (torch.autograd)"
                 if c["kind"] == "zea_grad" else args.ops.replace(",", " + "))
    cfg = {"workload": workload, "n_det": c["n_det"], "n_time": c["n_time"],
           "map": map_shape, "step": step_name,
           "l2": ("inputs larger than L2 (TOD %.1f GB)" % (c["n_det"] * c["n_time"] * 4 / 1e9)
                  if c["n_det"] * c["n_time"] * 4 > 129e6 else
                  "TOD of %.1f MB fits in L2 (no flush between steps)" % (
                      c["n_det"] * c["n_time"] * 4 / 1e6)),
           "precision": (PRECISION[args.pointing] if c["kind"] in ("car", "hp") or
                         args.pointing != "mixed" else
                         "double-float pointing with the reference's bilinear taps (certified, "
                         "float64 fallback), float32 spin factors, weights and products, "
                         "float64 map accumulation"),
           "pointing": args.pointing,
           "parallelism": "replicas" if world > 1 else "single GPU"}

    if args.impl == "reference":
        if rank != 0:
            return
        return run_reference(args, c, cfg, metric, world)

    res, N = run_ours(args, c, rank, world)
    if rank != 0:
        return
    hbm, kind = peaks()
    ms = res["ms_per_step"]
    value = replica_throughput(N, world, ms)
    op = "to_map" if "to_map" in res["op_ms"] else list(res["op_ms"])[0]
    B = algorithmic_bytes(c, op)
    achieved = B * N / (res["op_ms"][op] * 1e-3) / 1e9
    line = {"metric": metric, "value": value, "unit": "samples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg,
            "op_ms": res["op_ms"],
            "roofline": {"bound": "hbm", "kernel": op, "achieved": achieved, "peak": hbm,
                         "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": (MEASURED_TRAFFIC_PER_SAMPLE[args.pointing][op] * N
                                     if c["kind"] == "car" and not c.get("tiled") and op in
                                     MEASURED_TRAFFIC_PER_SAMPLE.get(args.pointing, {})
                                     else None),
                         "bytes_per_sample": B, "peak_kind": kind},
            "clocks": res["clocks"], "gpu_launches": int(res["launches"])}
    if "certified" in res:
        f = res["certified"]
        line["certified"] = {"value": N / (f["ms_per_step"] * 1e-3), "op_ms": f["op_ms"]}
    if "accuracy" in res:
        line["accuracy"] = res["accuracy"]
    if "fp64_path" in res:
        f = res["fp64_path"]
        line["fp64_path"] = {"value": N / (f["ms_per_step"] * 1e-3), "op_ms": f["op_ms"],
                             "mixed_over_fp64": f["ms_per_step"] / ms}
        if "to_map" in f["op_ms"]:
            # Its bound: the float64 pipe (ncu: 163 float64-pipe lane
            # operations per sample in to_map; the float64 FMA rate measured
            # on a GB300: 5.0e11 lane-ops/s).
            ach = FP64_OPS_PER_SAMPLE_TO_MAP * N / (f["op_ms"]["to_map"] * 1e-3)
            line["fp64_path"]["roofline"] = {
                "bound": "fp64 pipe", "kernel": "to_map", "achieved": ach,
                "peak": FP64_LANE_OPS_PER_S, "unit": "lane-ops/s",
                "frac": ach / FP64_LANE_OPS_PER_S}
    if "to_weight_map_ms" in res:
        line["to_weight_map"] = {"ms": res["to_weight_map_ms"],
                                 "samples_per_s": N / (res["to_weight_map_ms"] * 1e-3)}
    if "e2e" in res:
        line["e2e"] = res["e2e"]
    if world == 1 and c["kind"] == "car" and not c.get("tiled") and not args.no_precomp:
        # The same workload with its pointing precomputed once
        # (ProjEng_Precomp): the HBM-bound form of the path.
        r = precomp_leg(c, args.steps, args.warmup)
        line["precomp"] = {"value": r["value"], "unit": "samples/s",
                           "ms_per_step": r["ms_per_step"], "op_ms": r["op_ms"],
                           "pointing_matrix_ms": r["pointing_matrix_ms"],
                           "roofline": r["roofline"], "gpu_launches": r["gpu_launches"],
                           "step": "Precomp to_map + from_map on pointing_matrix output "
                                   "(pixel indices bit-exact, spin factors as the "
                                   "certified path)"}
    if world == 1 and args.config == "cfg2" and not args.no_legs:
        # The other benchmark workloads at full size, mixed pointing.
        line["legs"] = {"hp": workload_leg(args, "cfg3"), "grad": workload_leg(args, "cfg5"),
                        "batch": batch_leg(args)}
    if world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(c)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
