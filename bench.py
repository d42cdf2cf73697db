#!/usr/bin/env python3
"""Benchmark of the TM_CCOEFF_NORMED path on one GB300.

Workload: Match on a 1920x1080 RGBA UI-like frame with a 96x32 button
template (the reference's 4-channel Match configuration), synthetic data
generated from fixed seeds.  One step = one Match call.  Metric:
template*Mpx/s = (templates x parent pixels / 1e6) / seconds.

  value  device-resident: frame and template already in HBM, the call
         queued on a stream, CUDA-event timed per step, L2 flushed
         (256 MB write) between steps outside the timed spans
  e2e    the same call through the host-buffer C ABI entry point
         (cvm_match): frame and template copied from pinned host memory,
         the 24-byte result copied back, timed on the host clock
  --impl reference  times the reference algorithm on the host cores
         (the C restatement of the reference's Go path in oracle/, the
         reference's own toolchain being absent) with every host thread,
         capped at the reference's 16-worker limit.

Prints one JSON line (rank 0).  With torchrun and N>1, each rank runs an
independent replica on its own GPU ("replicas only": the path has no
exchange step) and value sums the ranks' throughput over the max time.
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
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# ----------------------------------------------------------- synthetic scenes


def pink_noise(rng, h, w, mean=128.0, sigma=40.0):
    """1/f^2-power noise (amplitude ~ 1/f) scaled to mean/sigma."""
    white = rng.standard_normal((h, w)).astype(np.float32)
    F = np.fft.rfft2(white)
    fy = np.fft.fftfreq(h)[:, None]
    fx = np.fft.rfftfreq(w)[None, :]
    f = np.sqrt(fx * fx + fy * fy)
    f[0, 0] = 1.0
    F /= f
    F[0, 0] = 0
    img = np.fft.irfft2(F, s=(h, w)).astype(np.float32)
    img = (img - img.mean()) / (img.std() + 1e-9)
    return img * sigma + mean


def add_rects(rng, img, count, smin, smax, channels):
    h, w = img.shape[:2]
    for _ in range(count):
        rw, rh = rng.integers(smin, smax + 1, 2)
        x, y = rng.integers(0, max(1, w - rw)), rng.integers(0, max(1, h - rh))
        col = rng.integers(0, 256, channels)
        img[y:y + rh, x:x + rw] = col if channels > 1 else col[0]
    return img


def to_u8(a):
    return np.clip(np.rint(a), 0, 255).astype(np.uint8)


def scene_gray_640x480(seed=1):
    """640x480 RGBA: 1/f^2 noise + 20 rectangles + N(0,2); 64x48 crop."""
    rng = np.random.default_rng(seed)
    base = pink_noise(rng, 480, 640)
    img = np.repeat(base[..., None], 3, axis=2)
    img += rng.standard_normal((480, 640, 3)).astype(np.float32) * 20  # colour variation
    img = add_rects(rng, img, 20, 8, 120, 3)
    img += rng.standard_normal(img.shape).astype(np.float32) * 2
    rgba = np.empty((480, 640, 4), np.uint8)
    rgba[..., :3] = to_u8(img)
    rgba[..., 3] = 255
    x, y = int(rng.integers(0, 640 - 64)), int(rng.integers(0, 480 - 48))
    return rgba, rgba[y:y + 48, x:x + 64].copy(), (x, y)


def scene_ui_1920x1080(seed=2):
    """1920x1080 UI-like RGBA: flat panels, gradients, 1-px glyph strokes,
    three near-duplicate 96x32 buttons; the template is one button with an
    a*x+b intensity shift."""
    rng = np.random.default_rng(seed)
    H, W = 1080, 1920
    img = np.empty((H, W, 3), np.float32)
    img[:] = rng.integers(180, 240, 3)
    for _ in range(40):  # panels
        rw, rh = rng.integers(60, 600), rng.integers(40, 400)
        x, y = rng.integers(0, W - rw), rng.integers(0, H - rh)
        img[y:y + rh, x:x + rw] = rng.integers(0, 256, 3)
    for _ in range(12):  # linear gradients
        rw, rh = rng.integers(100, 500), rng.integers(30, 200)
        x, y = rng.integers(0, W - rw), rng.integers(0, H - rh)
        c0, c1 = rng.integers(0, 256, 3).astype(np.float32), rng.integers(0, 256, 3).astype(np.float32)
        t = np.linspace(0, 1, rw, dtype=np.float32)[None, :, None]
        img[y:y + rh, x:x + rw] = c0 * (1 - t) + c1 * t
    for _ in range(3000):  # 1-px glyph strokes
        x, y = rng.integers(0, W - 12), rng.integers(0, H - 12)
        L = rng.integers(3, 12)
        col = rng.integers(0, 80, 3)
        if rng.random() < 0.5:
            img[y, x:x + L] = col
        else:
            img[y:y + L, x] = col
    # the button and two near duplicates (<= 4 pixels differ)
    btn = np.empty((32, 96, 3), np.float32)
    btn[:] = rng.integers(40, 200, 3)
    btn[0, :] = btn[-1, :] = btn[:, 0] = btn[:, -1] = 20
    for _ in range(25):
        x, y = rng.integers(8, 88), rng.integers(8, 24)
        btn[y, x:x + rng.integers(2, 6)] = 250
    spots = [(300, 200), (1200, 640), (1600, 90)]
    for i, (x, y) in enumerate(spots):
        b = btn.copy()
        if i > 0:
            for _ in range(4):
                b[rng.integers(2, 30), rng.integers(2, 94)] = rng.integers(0, 256, 3)
        img[y:y + 32, x:x + 96] = b
    rgba = np.empty((H, W, 4), np.uint8)
    rgba[..., :3] = to_u8(img)
    rgba[..., 3] = 255
    a, b0 = rng.uniform(0.9, 1.1), rng.uniform(-10, 10)
    tpl = np.empty((32, 96, 4), np.uint8)
    tpl[..., :3] = to_u8(btn * a + b0)
    tpl[..., 3] = 255
    return rgba, tpl, spots[0]


def scene_gray_3840x2160(seed=3):
    """3840x2160 gray: 1/f^2 noise + rectangles + N(0,3); a 256x256 crop
    with N(0,4) added."""
    rng = np.random.default_rng(seed)
    img = pink_noise(rng, 2160, 3840)
    img = add_rects(rng, img, 60, 16, 400, 1)
    img += rng.standard_normal(img.shape).astype(np.float32) * 3
    g = to_u8(img)
    x, y = int(rng.integers(0, 3840 - 256)), int(rng.integers(0, 2160 - 256))
    tpl = to_u8(g[y:y + 256, x:x + 256].astype(np.float32) + rng.standard_normal((256, 256)) * 4)
    return g, tpl, (x, y)


def scene_fleet_2560x1440(seed=4, count=256):
    """2560x1440 RGBA frame and `count` templates, sizes U[16,192]xU[16,128];
    70% crops with an a*x+b shift, 30% from an independent seed."""
    rng = np.random.default_rng(seed)
    base = pink_noise(rng, 1440, 2560)
    img = np.repeat(base[..., None], 3, axis=2)
    img += rng.standard_normal(img.shape).astype(np.float32) * 25
    img = add_rects(rng, img, 80, 8, 300, 3)
    img += rng.standard_normal(img.shape).astype(np.float32) * 2
    frame = np.empty((1440, 2560, 4), np.uint8)
    frame[..., :3] = to_u8(img)
    frame[..., 3] = 255
    other = np.random.default_rng(seed + 1000)
    tpls, where = [], []
    for i in range(count):
        w, h = int(rng.integers(16, 193)), int(rng.integers(16, 129))
        t = np.empty((h, w, 4), np.uint8)
        t[..., 3] = 255
        if rng.random() < 0.7:
            x, y = int(rng.integers(0, 2560 - w)), int(rng.integers(0, 1440 - h))
            a, b = rng.uniform(0.9, 1.1), rng.uniform(-10, 10)
            t[..., :3] = to_u8(frame[y:y + h, x:x + w, :3].astype(np.float32) * a + b)
            where.append((x, y))
        else:
            t[..., :3] = other.integers(0, 256, (h, w, 3), dtype=np.uint8)
            where.append(None)
        tpls.append(t)
    return frame, tpls, where


def scene_stream_1920x1080(seed=5, frames=16, ncolor=64, ngray=8):
    """A 1920x1080 RGBA frame sequence: a 1/f^2 noise + rectangles scene,
    each frame the previous one with 5% of the rectangles moved and the
    sigma=2 noise redrawn; 64 colour templates of 24x24..128x96 (70% crops
    with an a*x+b shift, 30% from an independent seed) and 8 gray crops."""
    rng = np.random.default_rng(seed)
    H, W = 1080, 1920
    base = pink_noise(rng, H, W)
    bg = np.repeat(base[..., None], 3, axis=2) + rng.standard_normal((H, W, 3)).astype(np.float32) * 20
    rects = []
    for _ in range(60):
        rw, rh = (int(v) for v in rng.integers(8, 200, 2))
        rects.append([int(rng.integers(0, W - rw)), int(rng.integers(0, H - rh)), rw, rh, rng.integers(0, 256, 3)])
    out = []
    for _ in range(frames):
        for i in rng.choice(len(rects), max(1, len(rects) // 20), replace=False):
            r = rects[i]
            r[0] = int(np.clip(r[0] + rng.integers(-40, 41), 0, W - r[2]))
            r[1] = int(np.clip(r[1] + rng.integers(-40, 41), 0, H - r[3]))
        img = bg.copy()
        for x, y, rw, rh, col in rects:
            img[y:y + rh, x:x + rw] = col
        img += rng.standard_normal(img.shape).astype(np.float32) * 2
        f = np.empty((H, W, 4), np.uint8)
        f[..., :3] = to_u8(img)
        f[..., 3] = 255
        out.append(f)
    other = np.random.default_rng(seed + 1000)
    color = []
    for _ in range(ncolor):
        w, h = int(rng.integers(24, 129)), int(rng.integers(24, 97))
        t = np.empty((h, w, 4), np.uint8)
        t[..., 3] = 255
        if rng.random() < 0.7:
            x, y = int(rng.integers(0, W - w)), int(rng.integers(0, H - h))
            a, b = rng.uniform(0.9, 1.1), rng.uniform(-10, 10)
            t[..., :3] = to_u8(out[0][y:y + h, x:x + w, :3].astype(np.float32) * a + b)
        else:
            t[..., :3] = other.integers(0, 256, (h, w, 3), dtype=np.uint8)
        color.append(t)
    gray = []
    for _ in range(ngray):
        w, h = int(rng.integers(24, 129)), int(rng.integers(24, 97))
        x, y = int(rng.integers(0, W - w)), int(rng.integers(0, H - h))
        gray.append(np.ascontiguousarray(out[0][y:y + h, x:x + w]))
    return out, color, gray


# ------------------------------------------------------------------ helpers


def slowest_rank_ms(ms: float, ws: int, device) -> float:
    """The largest of the ranks' times (replicas run independently; the job
    is as slow as its slowest rank)."""
    if ws <= 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, ms: float, ws: int) -> float:
    """Whole-job units per second: every rank processes units_per_rank in
    the slowest rank's time."""
    return ws * units_per_rank / (ms / 1e3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # start timing only once samples are flowing
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0:
                time.sleep(0.01)
        except OSError:
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
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


WORKLOAD = {"workload": "Match RGBA 1920x1080, template 96x32 (UI-like synthetic, a*x+b shifted button)",
            "parent": [1920, 1080], "template": [96, 32], "channels": "RGBA (cn=3 after the alpha scan)",
            "templates": 1, "l2": "flushed (256 MB write) between timed steps"}
MPX = 1920 * 1080 / 1e6


# --------------------------------------------------------- reference arm


FORM = {"exact": 0, "fast": 1}  # CVM_FORM_EXACT, CVM_FORM_FAST


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import oracle
    frame, tpl, _ = scene_ui_1920x1080()
    threads = min(16, os.cpu_count() or 1)
    for _ in range(max(1, args.warmup)):
        oracle.match_u8(frame, tpl, 3, threads=threads, want_map=False)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.match_u8(frame, tpl, 3, threads=threads, want_map=False)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.mean(times))
    v = MPX / (ms / 1e3)
    line = {"metric": "template*Mpx/s", "value": v, "unit": "template*Mpx/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": WORKLOAD, "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "template*Mpx/s", "cores": threads, "kind": "port",
                             "sample": "one full Match per step (cvmatch's scalar Go path restated in C, "
                                       "oracle/cvm_oracle.c; Go is not installed on this host)"},
            "e2e": {"value": v, "unit": "template*Mpx/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# --------------------------------------------------------------- GPU arm


def cpu_baseline_sample(frame, tpl, budget_s=12.0):
    """The oracle timed single-threaded on a bounded sample of the workload."""
    import oracle
    oracle.match_u8(frame, tpl, 3, threads=1, want_map=False)
    times = []
    t_end = time.perf_counter() + budget_s
    while time.perf_counter() < t_end and len(times) < 50:
        t0 = time.perf_counter()
        oracle.match_u8(frame, tpl, 3, threads=1, want_map=False)
        times.append(time.perf_counter() - t0)
    s = float(np.mean(times))
    return {"value": MPX / s, "unit": "template*Mpx/s", "cores": 1, "kind": "port",
            "sample": f"{len(times)} full Match calls on the same frame, 1 thread "
                      "(C restatement of the reference's scalar Go path)"}


def run_gpu(args):
    import ctypes as C
    import torch
    import cvmatch_gb300 as cvm

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    L = cvm.lib()
    cvm.SetForm(FORM[args.form])
    frame, tpl, _ = scene_ui_1920x1080()
    d_frame = torch.from_numpy(frame).to(dev)
    d_tpl = torch.from_numpy(tpl).to(dev)
    d_out = torch.zeros(6, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step_dev():
        rc = L.cvm_match_device(d_frame.data_ptr(), frame.strides[0], 1920, 1080, d_tpl.data_ptr(),
                                tpl.strides[0], 96, 32, None, d_out.data_ptr(), sh)
        if rc:
            buf = C.create_string_buffer(512)
            L.cvm_last_error(buf, 512)
            raise RuntimeError(buf.value.decode())

    hp = L.cvm_host_alloc(frame.nbytes)
    hframe = np.ctypeslib.as_array((C.c_uint8 * frame.nbytes).from_address(hp)).reshape(frame.shape)
    hframe[:] = frame
    res = cvm._CResult()

    def measure(form):
        """Device-resident ms per step (CUDA events, L2 flushed), the e2e ms
        through cvm_match with the pinned host frame, launches per step and
        the clock record, in one arithmetic form."""
        cvm.SetForm(FORM[form])
        for _ in range(max(3, args.warmup)):
            step_dev()
        torch.cuda.synchronize()
        l0 = L.cvm_launch_count()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            for i in range(args.steps):
                flush.zero_()
                starts[i].record(stream)
                step_dev()
                ends[i].record(stream)
            torch.cuda.synchronize()
        launches = (L.cvm_launch_count() - l0) // args.steps
        ms = slowest_rank_ms(float(np.mean([s.elapsed_time(e) for s, e in zip(starts, ends)])), ws, dev)
        # e2e through the host-buffer entry point, pinned host frame
        for _ in range(3):
            L.cvm_match(hp, frame.strides[0], 1920, 1080, tpl.ctypes.data, tpl.strides[0], 96, 32, C.byref(res))
        e2e_t = []
        for i in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rc = L.cvm_match(hp, frame.strides[0], 1920, 1080, tpl.ctypes.data, tpl.strides[0], 96, 32, C.byref(res))
            e2e_t.append(time.perf_counter() - t0)
            assert rc == 0
        e2e_ms = slowest_rank_ms(1e3 * float(np.mean(e2e_t)), ws, dev)
        out = d_out.cpu().numpy()
        got = (float(out[:1].view(np.float32)[0]), int(out[1]), int(out[2]),
               float(out[3:4].view(np.float32)[0]), int(out[4]), int(out[5]))
        assert got == res.tuple(), (got, res.tuple())  # device-resident and host-buffer calls agree
        return ms, e2e_ms, launches, clk, got

    # the reported form first, then the other one; the roofline pass below
    # runs the reported form again
    other = "fast" if args.form == "exact" else "exact"
    ms, e2e_ms, launches, clk, got = measure(args.form)
    o_ms, o_e2e, _, _, _ = measure(other)
    cvm.SetForm(FORM[args.form])
    value = replica_throughput(MPX, ms, ws)
    L.cvm_host_free(hp)

    line = None
    if rank == 0:
        peak, peak_kind = measured_peaks()
        roof = roofline(L, step_dev, torch, stream, peak, peak_kind, args.form)
        if args.timeline:
            for nm, a, b in timeline(L, step_dev, torch):
                sys.stderr.write(f"timeline {nm:24s} {a:8.1f} {b:8.1f} us\n")
        line = {"metric": "template*Mpx/s", "value": value, "unit": "template*Mpx/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": dict(WORKLOAD, parallelism="replicas" if ws > 1 else "single"), "form": args.form,
                "e2e": {"value": replica_throughput(MPX, e2e_ms, ws), "unit": "template*Mpx/s",
                        "h2d_bytes_per_step": int(frame.nbytes + tpl.nbytes), "d2h_bytes_per_step": 24},
                "gpu_launches": int(launches), "clocks": clk.summary(), "roofline": roof,
                "result": list(got),
                # the same workload in the other arithmetic form, measured in this run
                "forms": {other: {"value": replica_throughput(MPX, o_ms, ws), "ms_per_step": o_ms,
                                  "e2e": replica_throughput(MPX, o_e2e, ws), "e2e_ms_per_step": o_e2e},
                          args.form: {"value": value, "ms_per_step": ms,
                                      "e2e": replica_throughput(MPX, e2e_ms, ws), "e2e_ms_per_step": e2e_ms}}}
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_sample(frame, tpl)
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def fft_flops(n):
    """Flops of one n-point transform of the reference's radix-4 engine
    (radix4.go:106-149): 34 per radix-4 butterfly (three 6-flop complex
    multiplies, eight complex adds), 4 per radix-2 head butterfly."""
    lg = n.bit_length() - 1
    f, h = 0, 1
    if lg & 1:
        f += 4 * (n // 2)
        h = 2
    while 4 * h <= n:
        f += 34 * (n // 4)
        h *= 4
    return f


def match_models(L, form="exact"):
    """Algorithmic bytes and flops per launch of each kernel on the
    benchmark workload (cn = 3 after the alpha scan; RGBA input): the HBM
    bytes each kernel must read and write by design (frame, spectra,
    window sums, per-result lanes) and the radix-4 engine's flops.  The
    fast form's fused column kernel reads every channel's row spectra and
    template spectra and writes one summed spectrum; its inverse rows read
    that one channel and one den float per result."""
    import ctypes as C
    tw, th, iw, ih, cn = 96, 32, 1920, 1080, 3
    rw, rh = iw - tw + 1, ih - th + 1
    out = (C.c_int32 * 6)()
    L.cvm_plan(tw, th, rw, rh, out)
    dftW, dftH, bW, bH, dh2, ntiles = list(out)
    hw = dftW // 2 + 1
    ntx, nty = -(-rw // bW), -(-rh // bH)
    fast = form == "fast"
    m = {k: [0.0, 0.0] for k in ("k_prep", "k_fwd_rows", "k_cols_fwd_mul_inv", "k_cols_fwd_sum_inv", "k_inv_rows",
                                 "k_hsum", "k_vstats")}
    cinv = 1 if fast else cn  # channels through the inverse transforms
    for t in range(ntiles):
        tx, ty = t % ntx, t // ntx
        x0, y0 = tx * bW, ty * bH
        bw, bh = min(bW, rw - x0), min(bH, rh - y0)
        H = dh2 if (dh2 and ty == nty - 1) else dftH
        loadW, loadH = bw + tw - 1, bh + th - 1
        rows = min(loadH, H)
        loaded = min(H, (loadH + 1) & ~1)
        rows_out = min(H, (bh + 1) & ~1)
        m["k_fwd_rows"][0] += loadW * rows * 4 + cn * loaded * hw * 8
        m["k_fwd_rows"][1] += cn * (loaded // 2) * (fft_flops(dftW) + 6 * hw)
        m["k_cols_fwd_mul_inv"][0] += cn * (loaded * hw * 8 + H * hw * 8 + rows_out * hw * 8)
        m["k_cols_fwd_mul_inv"][1] += cn * hw * (2 * fft_flops(H) + 6 * H)
        m["k_cols_fwd_sum_inv"][0] += cn * (loaded * hw * 8 + H * hw * 8) + rows_out * hw * 8
        m["k_cols_fwd_sum_inv"][1] += hw * ((cn + 1) * fft_flops(H) + 8 * cn * H)
        m["k_inv_rows"][0] += cinv * rows_out * hw * 8
        m["k_inv_rows"][1] += cinv * (rows_out // 2) * (fft_flops(dftW) + 2 * dftW) + bw * bh * 8
    hp = -(-rw // 32) * 32
    lane = 4 if fast else 8                                 # den alone, or the (t, den) lane, per result
    m["k_prep"][0] = iw * ih * 4
    m["k_inv_rows"][0] += rw * rh * lane
    m["k_hsum"][0] = iw * ih * 4 + ih * hp * 16             # frame in, 4 window sums per (row, x) out
    bands = -(-rh // 16)
    m["k_vstats"][0] = bands * (16 + th) * rw * 16 + rw * rh * lane
    return m


def measured_traffic(form="exact"):
    """DRAM bytes per launch per kernel from the committed ncu summary of
    this workload in this form (profiles/match_rgba_1920x1080_dram_traffic.txt,
    profiles/match_rgba_1920x1080_fast_dram_traffic.txt), or {}."""
    path = os.path.join(ROOT, "profiles", "match_rgba_1920x1080_fast_dram_traffic.txt" if form == "fast"
                        else "match_rgba_1920x1080_dram_traffic.txt")
    out = {}
    if os.path.exists(path):
        for line in open(path):
            f = line.split("#", 1)[0].split()
            if len(f) == 2:
                out[f[0]] = int(f[1])
    return out


def profile_kernels(L, step_dev, torch, reps=20):
    """Per-kernel totals over `reps` steps from the library's event
    instrumentation (events recorded on the stream each kernel is launched
    on): [(name, total ms, launches)]."""
    import ctypes as C
    L.cvm_profile_enable.argtypes = [C.c_int]
    L.cvm_profile_enable.restype = None
    L.cvm_profile_read.argtypes = [C.c_int, C.c_char_p, C.c_size_t, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
    L.cvm_profile_enable(1)
    for _ in range(reps):
        step_dev()
    torch.cuda.synchronize()
    L.cvm_profile_enable(0)
    rows = []
    name = C.create_string_buffer(64)
    ms_, cnt = C.c_double(), C.c_uint64()
    i = 0
    while L.cvm_profile_read(i, name, 64, C.byref(ms_), C.byref(cnt)) == 0:
        rows.append((name.value.decode(), ms_.value, int(cnt.value)))
        i += 1
    return rows


def timeline(L, step_dev, torch, steps=3):
    """Per-launch spans (kernel, start, end; ms after the first launch) of
    the last of `steps` profiled steps, across the library's streams."""
    import ctypes as C
    L.cvm_profile_span.argtypes = [C.c_int, C.c_char_p, C.c_size_t, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.cvm_profile_enable(1)
    for _ in range(steps):
        step_dev()
    torch.cuda.synchronize()
    L.cvm_profile_enable(0)
    spans, i = [], 0
    name = C.create_string_buffer(64)
    t0, t1 = C.c_double(), C.c_double()
    while L.cvm_profile_span(i, name, 64, C.byref(t0), C.byref(t1)) == 0:
        spans.append((name.value.decode(), t0.value, t1.value))
        i += 1
    per = len(spans) // steps
    last = spans[-per:] if per else []
    base = min((a for _, a, _ in last), default=0.0)
    return [(nm, round(1e3 * (a - base), 1), round(1e3 * (b - base), 1)) for nm, a, b in last]


def roofline(L, step_dev, torch, stream, peak, peak_kind, form="exact"):
    """The dominant kernel's algorithmic bytes over its duration, timed live
    by the library's event instrumentation."""
    rows = profile_kernels(L, step_dev, torch)
    models = match_models(L, form)
    total = sum(r[1] for r in rows)
    kernels = {}
    for nm, ms, n in rows:
        per = ms / max(n, 1)
        by, fl = models.get(nm, (None, None))
        kernels[nm] = {"ms_per_launch": per, "launches": n, "share": ms / total if total else None,
                       "alg_bytes": by, "gbs": (by / (per / 1e3) / 1e9) if by else None,
                       "gflops": (fl / (per / 1e3) / 1e9) if fl else None}
    top = max(((nm, v) for nm, v in kernels.items() if v["alg_bytes"]), key=lambda kv: kv[1]["share"])
    nm, v = top
    traffic = measured_traffic(form).get(nm)
    return {"bound": "hbm", "kernel": nm, "achieved": v["gbs"], "peak": peak, "unit": "GB/s",
            "frac": v["gbs"] / peak, "peak_source": peak_kind, "traffic": traffic, "share": v["share"],
            "alg_bytes_per_launch": v["alg_bytes"], "kernels": kernels}


def run_stream(args):
    """A stream of 1920x1080 RGBA frames against 64 colour templates and
    8 gray matchers on each frame's gray conversion, through cvm_stream (the
    per-frame pipeline replayed as a CUDA graph, two frames in flight, host
    frames copied in and results copied out).  Reports frames/s, template
    Mpx/s (72 templates x 2.07 Mpx per frame) and the per-frame device
    latency p50/p99 (upload start to results back, one frame queued
    ahead), beside the same frames through Fleet.FindAll one call at a time."""
    import ctypes as C
    import torch
    import cvmatch_gb300 as cvm
    frames, color, gray = scene_stream_1920x1080()
    H, W = frames[0].shape[:2]
    cf = cvm.NewFleet(*[cvm.NewMatcher(t) for t in color])
    gf = cvm.NewFleet(*[cvm.NewGrayMatcher(t) for t in gray])
    cf.SetForm(FORM[args.form])
    gf.SetForm(FORM[args.form])
    st = cvm.NewStream(cf, gf, W, H)
    graphed, per_frame_launches = st.info()
    nfr = args.frames
    K = len(frames)
    for i in range(max(3, args.warmup)):
        st.push(frames[i % K])
        st.pull()
    torch.cuda.synchronize()
    lat = []
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for i in range(nfr):
            st.push(frames[i % K])
            if i >= 1:
                lat.append(st.pull()[2])
        lat.append(st.pull()[2])
        wall = time.perf_counter() - t0
    fps = nfr / wall
    mpx = (len(color) + len(gray)) * W * H / 1e6
    # the same frames one FindAll at a time (host buffers, no graph, no overlap)
    g_frames = [cvm.rgba_to_gray(f) for f in frames[:4]]
    for i in range(3):
        cf.FindAll(frames[i % 4]), gf.FindAll(g_frames[i % 4])
    t1 = time.perf_counter()
    nb = min(100, nfr)
    for i in range(nb):
        cf.FindAll(frames[i % 4])
        gf.FindAll(cvm.rgba_to_gray(frames[i % 4]))
    fps_plain = nb / (time.perf_counter() - t1)
    line = {"metric": "template*Mpx/s", "value": fps * mpx, "unit": "template*Mpx/s", "n_gpus": 1,
            "steps": nfr, "warmup": args.warmup, "ms_per_step": 1e3 / fps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "Fleet stream: 1920x1080 RGBA frames, 64 colour templates 24x24..128x96 + 8 gray "
                                   "matchers on the gray conversion; each frame moves 5% of the rectangles and redraws "
                                   f"sigma=2 noise ({K} precomputed frames cycled)",
                       "frames": nfr, "templates": len(color) + len(gray), "parent": [W, H], "form": args.form},
            "frames_per_s": fps, "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
            "graphed": graphed, "gpu_launches": per_frame_launches,
            "findall_per_frame_fps": fps_plain, "clocks": clk.summary(),
            "e2e": {"value": fps * mpx, "unit": "template*Mpx/s", "h2d_bytes_per_step": int(frames[0].nbytes),
                    "d2h_bytes_per_step": int((len(color) + len(gray)) * 24)}, "secondary": True}
    print(json.dumps(line))
    return 0


def run_gpu_secondary(args):
    """Secondary workloads (not the default line): 'fleet' = Fleet.FindAll
    of 256 templates on a 2560x1440 RGBA frame, 'gray' = MatchGray
    640x480 / 64x48, 'map' = MatchMap gray 3840x2160 / 256x256."""
    import ctypes as C
    import torch
    import cvmatch_gb300 as cvm
    import oracle

    dev = torch.device("cuda", 0)
    L = cvm.lib()
    cvm.SetForm(FORM[args.form])
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    if args.workload == "fleet":
        frame, tpls, _ = scene_fleet_2560x1440(count=args.templates)
        ms = [cvm.NewMatcher(t) for t in tpls]
        fleet = cvm.NewFleet(*ms)
        fleet.SetForm(FORM[args.form])
        n = len(ms)
        H, W = frame.shape[:2]
        mpx = n * W * H / 1e6
        d_frame = torch.from_numpy(frame).to(dev)
        d_out = torch.zeros(6 * n, dtype=torch.int32, device=dev)

        def step_dev():
            fleet.find_all_device(d_frame.data_ptr(), frame.strides[0], W, H, d_out.data_ptr(), sh)

        hp = L.cvm_host_alloc(frame.nbytes)
        hframe = np.ctypeslib.as_array((C.c_uint8 * frame.nbytes).from_address(hp)).reshape(frame.shape)
        hframe[:] = frame
        outs = (cvm._CResult * n)()

        def step_e2e():
            rc = L.cvm_fleet_find_all(fleet._h, hp, frame.strides[0], W, H, outs)
            assert rc == 0

        h2d, d2h = frame.nbytes, 24 * n
        cfg = {"workload": f"Fleet.FindAll, {n} RGBA templates 16..192 x 16..128 on a 2560x1440 RGBA frame",
               "templates": n, "parent": [W, H], "form": args.form}

        def cpu_sample():
            k = 4
            t0 = time.perf_counter()
            oracle.fleet_find_all(tpls[:k], frame, threads=1)
            dt = time.perf_counter() - t0
            return {"value": k * W * H / 1e6 / dt, "unit": "template*Mpx/s", "cores": 1, "kind": "port",
                    "sample": f"the first {k} templates of the fleet, 1 thread"}
    elif args.workload == "gray":
        frame, tpl, _ = scene_gray_640x480()
        g, gt = oracle.rgba_to_gray(frame), oracle.rgba_to_gray(tpl)
        H, W = g.shape
        th, tw = gt.shape
        mpx = W * H / 1e6
        d_img = torch.from_numpy(g).to(dev)
        d_tpl = torch.from_numpy(gt).to(dev)
        d_out = torch.zeros(6, dtype=torch.int32, device=dev)
        L.cvm_match_u8_device.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_int,
                                          C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]

        def step_dev():
            assert L.cvm_match_u8_device(d_img.data_ptr(), W, W, H, d_tpl.data_ptr(), tw, tw, th, 1, 1, None,
                                         d_out.data_ptr(), sh) == 0

        res = cvm._CResult()

        def step_e2e():
            assert L.cvm_match_gray_rgba(frame.ctypes.data, frame.strides[0], frame.shape[1], frame.shape[0],
                                         tpl.ctypes.data, tpl.strides[0], tpl.shape[1], tpl.shape[0],
                                         C.byref(res)) == 0

        h2d, d2h = frame.nbytes + tpl.nbytes, 24
        cfg = {"workload": "MatchGray 640x480 (from RGBA), template 64x48", "parent": [W, H], "templates": 1,
               "form": args.form}

        def cpu_sample():
            t0 = time.perf_counter()
            reps = 0
            while time.perf_counter() - t0 < 5:
                oracle.match_u8(g, gt, 1, threads=1, want_map=False)
                reps += 1
            return {"value": reps * mpx / (time.perf_counter() - t0), "unit": "template*Mpx/s", "cores": 1,
                    "kind": "port", "sample": f"{reps} MatchGray calls, 1 thread"}
    else:  # map
        g, tpl, _ = scene_gray_3840x2160()
        H, W = g.shape
        th, tw = tpl.shape
        mpx = W * H / 1e6
        rw, rh = W - tw + 1, H - th + 1
        d_img = torch.from_numpy(g).to(dev)
        d_tpl = torch.from_numpy(tpl).to(dev)
        d_map = torch.empty((rh, rw), dtype=torch.float32, device=dev)
        d_out = torch.zeros(6, dtype=torch.int32, device=dev)
        L.cvm_match_u8_device.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_int,
                                          C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]

        def step_dev():
            assert L.cvm_match_u8_device(d_img.data_ptr(), W, W, H, d_tpl.data_ptr(), tw, tw, th, 1, 1,
                                         d_map.data_ptr(), d_out.data_ptr(), sh) == 0

        hmap = np.empty((rh, rw), np.float32)
        res = cvm._CResult()
        L.cvm_match_u8.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_int, C.c_int,
                                   C.c_int, C.c_int, C.c_void_p, C.POINTER(cvm._CResult)]

        def step_e2e():
            assert L.cvm_match_u8(g.ctypes.data, W, W, H, tpl.ctypes.data, tw, tw, th, 1, 1, hmap.ctypes.data,
                                  C.byref(res)) == 0

        h2d, d2h = g.nbytes + tpl.nbytes, hmap.nbytes + 24
        cfg = {"workload": "MatchMap gray 3840x2160, template 256x256, full float32 map returned",
               "parent": [W, H], "templates": 1, "form": args.form}

        def cpu_sample():
            t0 = time.perf_counter()
            oracle.match_u8(g, tpl, 1, threads=1, want_map=True)
            return {"value": mpx / (time.perf_counter() - t0), "unit": "template*Mpx/s", "cores": 1, "kind": "port",
                    "sample": "one MatchMap call, 1 thread"}

    for _ in range(max(3, args.warmup)):
        step_dev()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    l0 = L.cvm_launch_count()
    for i in range(args.steps):
        flush.zero_()
        starts[i].record(stream)
        step_dev()
        ends[i].record(stream)
    torch.cuda.synchronize()
    launches = (L.cvm_launch_count() - l0) // args.steps
    ms = float(np.mean([a.elapsed_time(b) for a, b in zip(starts, ends)]))
    for _ in range(2):
        step_e2e()
    et = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step_e2e()
        et.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * float(np.mean(et))
    line = {"metric": "template*Mpx/s", "value": mpx / (ms / 1e3), "unit": "template*Mpx/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
            "e2e": {"value": mpx / (e2e_ms / 1e3), "unit": "template*Mpx/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms},
            "gpu_launches": int(launches), "secondary": True}
    rows = profile_kernels(L, step_dev, torch, reps=3)
    tot = sum(r[1] for r in rows) or 1.0
    line["kernels"] = {nm: {"ms_per_launch": t / max(n, 1), "launches": n, "share": t / tot} for nm, t, n in rows}
    if args.timeline:
        for nm, a, b in timeline(L, step_dev, torch):
            sys.stderr.write(f"timeline {nm:24s} {a:8.1f} {b:8.1f} us\n")
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample()
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--frames", type=int, default=1000, help="frames for --workload stream")
    ap.add_argument("--workload", default="match", choices=["match", "fleet", "gray", "map", "stream"],
                    help="match (default, the reported line) or a secondary configuration")
    ap.add_argument("--templates", type=int, default=256, help="fleet size for --workload fleet")
    ap.add_argument("--form", default="fast", choices=["exact", "fast"],
                    help="arithmetic: fast (default; within 1e-5 of the FP64 definition) or exact (the "
                         "reference's float32 bits; cvm_set_form / cvm_fleet_set_form)")
    ap.add_argument("--timeline", action="store_true", help="print one profiled step's launch spans to stderr")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "stream":
        return run_stream(args)
    if args.workload != "match":
        return run_gpu_secondary(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
