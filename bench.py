#!/usr/bin/env python3
"""Benchmark of the TM_CCOEFF_NORMED path on one GB300.

Default workload (the reported line): Fleet.FindAll of 256 RGBA templates
(sizes uniform 16..192 x 16..128; 70% shifted crops of the frame, 30% from
an independent seed) on one 2560x1440 RGBA frame -- the largest single-GPU
configuration of the metric (the reference's Fleet batching, fleet.go).
Synthetic data from fixed seeds.  One step = one FindAll.  Metric:
template*Mpx/s = (templates x parent pixels / 1e6) / seconds.  Secondary
workloads: --workload match (Match RGBA 1920x1080 / 96x32), gray
(MatchGray 640x480 / 64x48, the RGBA->gray conversions included), map
(MatchMap gray 3840x2160 / 256x256, full map returned), stream (1080p frame
stream, 64 colour + 8 gray templates per frame).

  value     device-resident: inputs already in HBM, the call queued on a
            stream, CUDA-event timed per step, L2 flushed (256 MB write)
            between steps outside the timed spans
  e2e       the same call through the public host-buffer API with the
            caller's ordinary (pageable) host memory, as the Python mirror
            and a cgo shim pass it: input copies and the results' read-back
            inside the timed span, host clock; e2e.pinned is the same with
            the frame in page-locked memory (cvm_host_alloc)
  roofline  the reference algorithm's flops on the reference's own plan
            (the count of the metric's configuration table: two real 2-D
            FFTs of 2.5 N log2 N per tile and channel, 6 per spectrum
            element for the conjugate product, 2 cn + 12 per result for the
            normalisation) over the step time, against the FP32 peak (SMs x
            128 lanes x 2 flops x the maximum SM clock); the dominant
            kernel's share, time and flops beside it, and HBM against the
            compulsory bytes (inputs, 24 B per template, the map if returned)
  --impl reference  the reference algorithm on the host cores (the C
            restatement of the reference's Go path in oracle/; the
            reference's own toolchain is absent) with every host thread,
            capped at the reference's 16-worker limit, on the same workload
            (a bounded sample of its member tails for the fleet)

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
    """Samples SM clocks and throttle reasons with nvidia-smi (query only)
    while running; each sample carries its host time, so the record can be
    split into the timed region and the rest of the window."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index: int, period_ms: int = 20):
        self.index = index
        self.period_ms = period_ms
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
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
            self.lines.append((time.time(), line.strip()))

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0=None, t1=None):
        """Median SM clock and the throttle reasons seen over every sample
        taken under load; `samples_timed` counts those inside [t0, t1] (the
        timed region), when given, and `sm_mhz_timed` is their median."""
        sm, smax, reasons, timed = [], None, set(), []
        for entry in self.lines:
            ts, ln = entry if isinstance(entry, tuple) else (None, entry)
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                v, mx = float(parts[0]), float(parts[1])
            except ValueError:
                continue
            sm.append(v)
            smax = mx
            if t0 is not None and ts is not None and t0 <= ts <= t1:
                timed.append(v)
            for nm, flag in zip(self.NAMES, parts[4:8]):
                if flag.lower() == "active":
                    reasons.add(nm)
        out = {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
               "reasons": sorted(reasons), "samples": len(sm)}
        if t0 is not None:
            # the samples taken inside the timed region itself, and their median
            out["samples_timed"] = len(timed)
            out["sm_mhz_timed"] = float(np.median(timed)) if timed else None
        return out


def measured_peaks():
    """(HBM GB/s, source): the measured copy bandwidth of the GB300s,
    else the stated fallback."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def fp32_peak_tflops(sms: int):
    """FP32 peak of the device: SMs x 128 FP32 lanes x 2 flops (one FMA) x
    the maximum SM clock (MEASURED_PEAKS.json's sm_max_mhz, else the
    GB300's 2070 MHz)."""
    mhz, src = 2070.0, "GB300 maximum SM clock"
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        if d.get("sm_max_mhz"):
            mhz, src = float(d["sm_max_mhz"]), "MEASURED_PEAKS.json sm_max_mhz"
    return sms * 128 * 2 * mhz * 1e6 / 1e12, f"derived: {sms} SMs x 128 FP32 lanes x 2 flops x {mhz:.0f} MHz ({src})"


FORM = {"exact": 0, "fast": 1, "mixed": 2}  # CVM_FORM_EXACT, CVM_FORM_FAST, CVM_FORM_MIXED


# ------------------------------------------------ the algorithmic work model


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


def rfft2_flops(w, h):
    """One real 2-D FFT of w x h points: 2.5 N log2 N, split into its row
    part (2.5 N log2 w) and column part (2.5 N log2 h)."""
    n = w * h
    return 2.5 * n * np.log2(w), 2.5 * n * np.log2(h)


def tile_heights(rw, rh, plan):
    """Per tile of newGoPlan's grid its transform height (dh2 on the shrunk
    last band, impl.go:573-582)."""
    dftW, dftH, bW, bH, dh2 = plan[:5]
    ntx, nty = -(-rw // bW), -(-rh // bH)
    return [dh2 if (dh2 and ty == nty - 1) else dftH for ty in range(nty) for _ in range(ntx)]


def solo_flops(L, tw, th, iw, ih, cn):
    """The reference algorithm's flops for one match on its own plan, per
    library kernel that does that part of the work: two real 2-D
    FFTs per tile and channel (forward, inverse), 6 per spectrum element
    for the conjugate product, 2 cn + 12 per result for normOne.  The
    template's own spectrum is not counted (cached by Matcher/Fleet)."""
    import ctypes as C
    rw, rh = iw - tw + 1, ih - th + 1
    out = (C.c_int32 * 6)()
    L.cvm_plan(tw, th, rw, rh, out)
    plan = list(out)
    dftW = plan[0]
    hw = dftW // 2 + 1
    fr = fc = cm = ir = 0.0
    for H in tile_heights(rw, rh, plan):
        r, c = rfft2_flops(dftW, H)
        fr += cn * r                        # forward rows of the frame tile
        fc += cn * c                        # forward columns
        cm += cn * (c + 6 * H * hw)         # conjugate product + inverse columns
        ir += cn * r                        # inverse rows
    ir += rw * rh * (2 * cn + 12)           # normOne + extrema in the inverse rows' epilogue
    return {"fwd_rows": fr, "fwd_cols": fc, "mul_inv_cols": cm, "inv_rows": ir}


def fleet_flops(buckets, members, tpl_shapes, pw, ph, cns):
    """The same count for Fleet.FindAll: each bucket's frame tiles once
    (phase 1, fleet.go:240-263), each member's tails on its bucket's plan
    (phase 2, fleet.go:265-328).  buckets: per bucket (tw, th, dftW, dftH,
    blockW, blockH, dh2, tiles, members); members: per bucket its member
    indices."""
    fr = fc = cm = ir = 0.0
    for (btw, bth, dftW, dftH, bW, bH, dh2, tiles, nmem), mem in zip(buckets, members):
        rwF, rhF = pw - btw + 1, ph - bth + 1
        hs = tile_heights(rwF, rhF, (dftW, dftH, bW, bH, dh2))
        hw = dftW // 2 + 1
        cn_max = max(cns[i] for i in mem) if mem else 3
        for H in hs:
            r, c = rfft2_flops(dftW, H)
            fr += cn_max * r
            fc += cn_max * c
        for i in mem:
            w, h = tpl_shapes[i]
            for H in hs:
                r, c = rfft2_flops(dftW, H)
                cm += cns[i] * (c + 6 * H * hw)
                ir += cns[i] * r
            ir += (pw - w + 1) * (ph - h + 1) * (2 * cns[i] + 12)
    return {"fwd_rows": fr, "fwd_cols": fc, "mul_inv_cols": cm, "inv_rows": ir}


# which live-profiled kernels do which part of the counted work
KERNEL_PART = {"k_fwd_rows": "fwd_rows", "k_fwd_rows_tma": "fwd_rows", "k_cols_fwd": "fwd_cols", "k_cols_fwd_mul_inv": "fwd_cols+mul_inv_cols",
               "k_cols_fwd_sum_inv": "fwd_cols+mul_inv_cols", "k_cols_mul_inv": "mul_inv_cols",
               "k_cols_sum_inv": "mul_inv_cols", "k_inv_rows": "inv_rows", "k_inv_rows_tc": "inv_rows"}


def kernel_flops(parts, name):
    key = KERNEL_PART.get(name)
    if not key:
        return None
    return sum(parts[k] for k in key.split("+"))


def match_models(L, form="exact"):
    """Algorithmic bytes and flops per launch of each kernel on the
    1920x1080 colour match (cn = 3 after the alpha scan; RGBA input): the
    HBM bytes each kernel must read and write by design (frame, spectra,
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


def measured_traffic(workload="match", form="exact"):
    """DRAM bytes per launch per kernel from the committed ncu summary of a
    workload in a form (profiles/<workload>_dram_traffic.txt), or {}."""
    names = {("match", "fast"): "match_rgba_1920x1080_fast_dram_traffic.txt",
             ("match", "exact"): "match_rgba_1920x1080_dram_traffic.txt",
             ("fleet", "fast"): "fleet_2560x1440_fast_dram_traffic.txt",
             ("fleet", "exact"): "fleet_2560x1440_dram_traffic.txt"}
    if workload in ("fast", "exact"):  # measured_traffic(form) of the colour match
        workload, form = "match", workload
    nm = names.get((workload, form))
    out = {}
    if nm and os.path.exists(os.path.join(ROOT, "profiles", nm)):
        for line in open(os.path.join(ROOT, "profiles", nm)):
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


def roofline(L, W, torch, ms, form, sms, reps):
    """FP32 roofline of the step on the counted algorithmic flops, the
    dominant kernel (largest live share) with its own flops and time, and
    HBM against the compulsory bytes."""
    peak, peak_src = fp32_peak_tflops(sms)
    hbm, hbm_kind = measured_peaks()
    parts = W.flops()
    total = sum(parts.values())
    achieved = total / (ms / 1e3) / 1e12
    # Each launch's own duration: a fleet's overlapped waves run one wave's
    # inverse rows beside the next wave's columns, so events around a launch
    # would also count the time it shares the GPU; the per-kernel pass runs
    # the waves in sequence (the step's `ms` above is the overlapped one).
    fleet = getattr(W, "fleet", None)
    if fleet is not None and hasattr(fleet, "SetOverlap"):
        fleet.SetOverlap(False)
    for _ in range(3):  # a form switch drops cached spectra: rebuild them outside the profile
        W.step_dev()
    torch.cuda.synchronize()
    rows = profile_kernels(L, W.step_dev, torch, reps=reps)
    if fleet is not None and hasattr(fleet, "SetOverlap"):
        fleet.SetOverlap(getattr(W, "overlap", True))
    tot_ms = sum(r[1] for r in rows) or 1.0
    kernels = {}
    for nm, t, n in rows:
        f = kernel_flops(parts, nm)
        per_step = t / reps
        kernels[nm] = {"ms_per_step": per_step, "launches_per_step": n / reps, "share": t / tot_ms,
                       "alg_flops_per_step": f, "tflops": (f / (per_step / 1e3) / 1e12) if f else None}
    top = max(kernels.items(), key=lambda kv: kv[1]["share"]) if kernels else (None, {})
    nm, kv = top
    traffic = measured_traffic(W.key, form).get(nm) if nm else None
    out = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
           **({"kernels_timed": "waves in sequence (each launch's own duration)"} if fleet is not None else {}),
           "traffic": traffic, "peak_source": peak_src, "alg_flops_per_step": total,
           "basis": "reference algorithm on the reference's plan: 2 real 2-D FFTs (2.5 N log2 N) per tile and "
                    "channel, 6 flops per spectrum element for the conjugate product, 2 cn + 12 per result; "
                    "the template spectra (cached per geometry) not counted",
           "kernel": {"name": nm, "share": kv.get("share"), "ms_per_step": kv.get("ms_per_step"),
                      "launches_per_step": kv.get("launches_per_step"),
                      "alg_flops_per_step": kv.get("alg_flops_per_step"), "tflops": kv.get("tflops"),
                      "frac": (kv["tflops"] / peak) if kv.get("tflops") else None,
                      "traffic_per_launch": traffic},
           "hbm": {"alg_bytes_per_step": W.alg_bytes, "gbs": W.alg_bytes / (ms / 1e3) / 1e9, "peak": hbm,
                   "peak_source": hbm_kind, "frac": W.alg_bytes / (ms / 1e3) / 1e9 / hbm},
           "kernels": kernels}
    return out


# ---------------------------------------------------------------- workloads


def _workload_config(key, ws, args):
    par = "replicas" if ws > 1 else "single"
    l2 = "flushed (256 MB write) between timed steps"
    if key == "fleet":
        return {"workload": f"Fleet.FindAll, {args.templates} RGBA templates 16..192 x 16..128 (70% a*x+b shifted "
                            "crops, 30% absent) on a 2560x1440 RGBA frame", "parent": [2560, 1440],
                "templates": args.templates, "channels": "RGBA (cn=3 after the alpha scans)", "l2": l2,
                "parallelism": par, **({"stats": "inverse-rows epilogue"} if getattr(args, "stats", "kernel")
                                       == "epilogue" else {}),
                **({"overlap": "off"} if getattr(args, "overlap", "on") == "off" else {}),
                **({"wave": args.wave} if getattr(args, "wave", 0) else {})}
    if key == "match":
        return {"workload": "Match RGBA 1920x1080, template 96x32 (UI-like synthetic, a*x+b shifted button)",
                "parent": [1920, 1080], "template": [96, 32], "channels": "RGBA (cn=3 after the alpha scan)",
                "templates": 1, "l2": l2, "parallelism": par}
    if key == "gray":
        return {"workload": "MatchGray 640x480 from RGBA (both conversions on every call), template 64x48",
                "parent": [640, 480], "template": [64, 48], "templates": 1, "l2": l2, "parallelism": par}
    if key == "map":
        return {"workload": "MatchMap gray 3840x2160, template 256x256, full float32 map returned",
                "parent": [3840, 2160], "template": [256, 256], "templates": 1, "l2": l2, "parallelism": par}
    raise ValueError(key)


def _units(key, args):
    return {"fleet": args.templates * 2560 * 1440 / 1e6, "match": 1920 * 1080 / 1e6, "gray": 640 * 480 / 1e6,
            "map": 3840 * 2160 / 1e6}[key]


def _alpha_cn(t):
    return 3 if (t[..., 3] == t.reshape(-1, 4)[0, 3]).all() else 4


class _Base:
    key = ""

    def __init__(self, cvm, torch, dev, stream):
        self.cvm, self.torch, self.dev = cvm, torch, dev
        self.L = cvm.lib()
        self.stream = stream
        self.sh = stream.cuda_stream
        self._pinned = []

    def pinned_copy(self, a):
        import ctypes as C
        hp = self.L.cvm_host_alloc(a.nbytes)
        assert hp, "cvm_host_alloc failed"
        self._pinned.append(hp)
        h = np.ctypeslib.as_array((C.c_uint8 * a.nbytes).from_address(hp)).view(a.dtype).reshape(a.shape)
        h[...] = a
        return h

    def close(self):
        for p in self._pinned:
            self.L.cvm_host_free(p)
        self._pinned = []

    def set_form(self, form):
        self.cvm.SetForm(FORM[form])


class FleetWorkload(_Base):
    key = "fleet"

    def __init__(self, cvm, torch, dev, stream, count=256):
        import ctypes as C
        super().__init__(cvm, torch, dev, stream)
        self.frame, self.tpls, self.where = scene_fleet_2560x1440(count=count)
        self.fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in self.tpls])
        self.n = len(self.tpls)
        self.H, self.W = self.frame.shape[:2]
        self.d_frame = torch.from_numpy(self.frame).to(dev)
        self.d_out = torch.zeros(6 * self.n, dtype=torch.int32, device=dev)
        self.hframe = self.pinned_copy(self.frame)
        self.outs = (cvm._CResult * self.n)()
        self.h2d, self.d2h = self.frame.nbytes, 24 * self.n
        self.alg_bytes = self.frame.nbytes + 24 * self.n
        self._C = C

    def set_form(self, form):
        self.fleet.SetForm(FORM[form])

    def step_dev(self):
        self.fleet.find_all_device(self.d_frame.data_ptr(), self.frame.strides[0], self.W, self.H,
                                   self.d_out.data_ptr(), self.sh)

    def _host(self, img):
        rc = self.L.cvm_fleet_find_all(self.fleet._h, img.ctypes.data, img.strides[0], self.W, self.H, self.outs)
        assert rc == 0

    def step_e2e(self):
        self._host(self.frame)       # the caller's pageable memory

    def step_e2e_pinned(self):
        self._host(self.hframe)

    def dev_result(self):
        o = self.d_out.cpu().numpy().reshape(self.n, 6)
        return [(float(r[:1].view(np.float32)[0]), int(r[1]), int(r[2]), float(r[3:4].view(np.float32)[0]),
                 int(r[4]), int(r[5])) for r in o]

    def host_result(self):
        return [o.tuple() for o in self.outs]

    def flops(self):
        pconst = bool((self.frame[..., 3] == self.frame[0, 0, 3]).all())
        cns = [(_alpha_cn(t) if pconst else 4) for t in self.tpls]
        shapes = [(t.shape[1], t.shape[0]) for t in self.tpls]
        bk = self.fleet.buckets(self.W, self.H)
        mem = [self.fleet.bucket_members(b) for b in range(len(bk))]
        return fleet_flops(bk, mem, shapes, self.W, self.H, cns)


class MatchWorkload(_Base):
    key = "match"

    def __init__(self, cvm, torch, dev, stream):
        import ctypes as C
        super().__init__(cvm, torch, dev, stream)
        self.frame, self.tpl, _ = scene_ui_1920x1080()
        self.d_frame = torch.from_numpy(self.frame).to(dev)
        self.d_tpl = torch.from_numpy(self.tpl).to(dev)
        self.d_out = torch.zeros(6, dtype=torch.int32, device=dev)
        self.hframe = self.pinned_copy(self.frame)
        self.res = cvm._CResult()
        self.h2d, self.d2h = self.frame.nbytes + self.tpl.nbytes, 24
        self.alg_bytes = self.frame.nbytes + 24
        self._C = C

    def step_dev(self):
        rc = self.L.cvm_match_device(self.d_frame.data_ptr(), self.frame.strides[0], 1920, 1080,
                                     self.d_tpl.data_ptr(), self.tpl.strides[0], 96, 32, None,
                                     self.d_out.data_ptr(), self.sh)
        assert rc == 0

    def _host(self, img):
        C = self._C
        rc = self.L.cvm_match(img.ctypes.data, img.strides[0], 1920, 1080, self.tpl.ctypes.data,
                              self.tpl.strides[0], 96, 32, C.byref(self.res))
        assert rc == 0

    def step_e2e(self):
        self._host(self.frame)

    def step_e2e_pinned(self):
        self._host(self.hframe)

    def dev_result(self):
        o = self.d_out.cpu().numpy()
        return (float(o[:1].view(np.float32)[0]), int(o[1]), int(o[2]), float(o[3:4].view(np.float32)[0]),
                int(o[4]), int(o[5]))

    def host_result(self):
        return self.res.tuple()

    def flops(self):
        return solo_flops(self.L, 96, 32, 1920, 1080, 3)


class GrayWorkload(_Base):
    """MatchGray on RGBA inputs: both gray conversions are part of every
    call (toGray, cvmatch.go:201-217), on the device as on the host."""
    key = "gray"

    def __init__(self, cvm, torch, dev, stream):
        import ctypes as C
        super().__init__(cvm, torch, dev, stream)
        self.frame, self.tpl, _ = scene_gray_640x480()
        self.d_frame = torch.from_numpy(self.frame).to(dev)
        self.d_tpl = torch.from_numpy(self.tpl).to(dev)
        self.d_g = torch.empty((480, 640), dtype=torch.uint8, device=dev)
        self.d_gt = torch.empty((48, 64), dtype=torch.uint8, device=dev)
        self.d_out = torch.zeros(6, dtype=torch.int32, device=dev)
        self.hframe = self.pinned_copy(self.frame)
        self.res = cvm._CResult()
        self.h2d, self.d2h = self.frame.nbytes + self.tpl.nbytes, 24
        self.alg_bytes = self.frame.nbytes + 24
        self._C = C

    def step_dev(self):
        L = self.L
        assert L.cvm_rgba_to_gray_device(self.d_frame.data_ptr(), 640 * 4, 640, 480, self.d_g.data_ptr(), 640,
                                         self.sh) == 0
        assert L.cvm_rgba_to_gray_device(self.d_tpl.data_ptr(), 64 * 4, 64, 48, self.d_gt.data_ptr(), 64,
                                         self.sh) == 0
        assert L.cvm_match_u8_device(self.d_g.data_ptr(), 640, 640, 480, self.d_gt.data_ptr(), 64, 64, 48, 1, 1,
                                     None, self.d_out.data_ptr(), self.sh) == 0

    def _host(self, img):
        C = self._C
        assert self.L.cvm_match_gray_rgba(img.ctypes.data, img.strides[0], 640, 480, self.tpl.ctypes.data,
                                          self.tpl.strides[0], 64, 48, C.byref(self.res)) == 0

    def step_e2e(self):
        self._host(self.frame)

    def step_e2e_pinned(self):
        self._host(self.hframe)

    dev_result = MatchWorkload.dev_result
    host_result = MatchWorkload.host_result

    def flops(self):
        return solo_flops(self.L, 64, 48, 640, 480, 1)


class MapWorkload(_Base):
    key = "map"

    def __init__(self, cvm, torch, dev, stream):
        import ctypes as C
        super().__init__(cvm, torch, dev, stream)
        self.g, self.tpl, _ = scene_gray_3840x2160()
        self.rw, self.rh = 3840 - 256 + 1, 2160 - 256 + 1
        self.d_img = torch.from_numpy(self.g).to(dev)
        self.d_tpl = torch.from_numpy(self.tpl).to(dev)
        self.d_map = torch.empty((self.rh, self.rw), dtype=torch.float32, device=dev)
        self.d_out = torch.zeros(6, dtype=torch.int32, device=dev)
        self.hmap = np.empty((self.rh, self.rw), np.float32)
        self.himg = self.pinned_copy(self.g)
        self.hmap_pinned = self.pinned_copy(self.hmap)
        self.res = cvm._CResult()
        self.h2d, self.d2h = self.g.nbytes + self.tpl.nbytes, self.hmap.nbytes + 24
        self.alg_bytes = self.g.nbytes + self.hmap.nbytes + 24
        self._C = C

    def step_dev(self):
        assert self.L.cvm_match_u8_device(self.d_img.data_ptr(), 3840, 3840, 2160, self.d_tpl.data_ptr(), 256, 256,
                                          256, 1, 1, self.d_map.data_ptr(), self.d_out.data_ptr(), self.sh) == 0

    def _host(self, img, hmap):
        C = self._C
        assert self.L.cvm_match_u8(img.ctypes.data, 3840, 3840, 2160, self.tpl.ctypes.data, 256, 256, 256, 1, 1,
                                   hmap.ctypes.data, C.byref(self.res)) == 0

    def step_e2e(self):
        self._host(self.g, self.hmap)

    def step_e2e_pinned(self):
        self._host(self.himg, self.hmap_pinned)

    dev_result = MatchWorkload.dev_result
    host_result = MatchWorkload.host_result

    def flops(self):
        return solo_flops(self.L, 256, 256, 3840, 2160, 1)


WORKLOADS = {"fleet": FleetWorkload, "match": MatchWorkload, "gray": GrayWorkload, "map": MapWorkload}


# --------------------------------------------------------- reference arm


def _ref_fleet_sample(frame, tpls, k, threads, rng_seed=0):
    """Fleet.FindAll of the whole fleet timed on a bounded sample: the frame
    spectra of every bucket (phase 1) and the member tails (phase 2) of k
    members spread over the size range; the whole frame's time is phase 1 +
    (n / k) x phase 2 (every member's tail costs the same: it runs every
    tile of its bucket's plan, fleet.go:265-328, and the reference claims
    members <= 16 at a time, one worker each).  The member spectra
    (buildGeom's per-geometry cache, fleet.go:366-375) are in neither
    phase."""
    import oracle
    n = len(tpls)
    order = sorted(range(n), key=lambda i: (tpls[i].shape[0] * tpls[i].shape[1], i))
    pick = sorted({order[round(j * (n - 1) / max(k - 1, 1))] for j in range(k)})
    _, _, (p1, p2) = oracle.fleet_find_all_sel(tpls, frame, pick, threads=threads)
    return p1 + (n / len(pick)) * p2, len(pick)


def _reference_step(key, args, data, threads):
    """One step of the reference algorithm on the host cores; returns its
    (estimated, for the fleet sample) seconds."""
    import oracle
    if key == "fleet":
        frame, tpls = data
        s, _ = _ref_fleet_sample(frame, tpls, args.ref_sample, threads)
        return s
    t0 = time.perf_counter()
    if key == "match":
        frame, tpl = data
        oracle.match_u8(frame, tpl, 3, threads=threads, want_map=False)
    elif key == "gray":
        frame, tpl = data
        oracle.match_u8(oracle.rgba_to_gray(frame), oracle.rgba_to_gray(tpl), 1, threads=threads, want_map=False)
    else:
        g, tpl = data
        oracle.match_u8(g, tpl, 1, threads=threads, want_map=True)
    return time.perf_counter() - t0


def _reference_data(key, args):
    if key == "fleet":
        frame, tpls, _ = scene_fleet_2560x1440(count=args.templates)
        return frame, tpls
    if key == "match":
        frame, tpl, _ = scene_ui_1920x1080()
        return frame, tpl
    if key == "gray":
        frame, tpl, _ = scene_gray_640x480()
        return frame, tpl
    g, tpl, _ = scene_gray_3840x2160()
    return g, tpl


def _reference_sample_text(key, args, threads):
    base = ("cvmatch's scalar Go path restated in C (oracle/cvm_oracle.c; Go is not installed on this host), "
            f"{threads} threads")
    if key == "fleet":
        return (f"per step, the whole fleet's frame spectra (phase 1) and the member tails of {args.ref_sample} of "
                f"its {args.templates} members spread over the size range (phase 2), scaled to the whole fleet as "
                f"phase 1 + ({args.templates}/{args.ref_sample}) x phase 2; " + base)
    return "one full call per step; " + base


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    if args.workload == "stream":
        return run_stream_reference(args)
    key = args.workload
    threads = min(16, os.cpu_count() or 1)
    data = _reference_data(key, args)
    for _ in range(max(1, args.warmup)):
        _reference_step(key, args, data, threads)
    secs = [_reference_step(key, args, data, threads) for _ in range(args.steps)]
    ms = 1e3 * float(np.mean(secs))
    units = _units(key, args)
    v = units / (ms / 1e3)
    line = {"metric": "template*Mpx/s", "value": v, "unit": "template*Mpx/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": _workload_config(key, ws, args),
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "template*Mpx/s", "cores": threads, "kind": "port",
                             "sample": _reference_sample_text(key, args, threads)},
            "e2e": {"value": v, "unit": "template*Mpx/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def cpu_baseline(key, args, budget_s=12.0):
    """The reference algorithm on one host thread, on a bounded sample of
    the workload (about budget_s seconds)."""
    data = _reference_data(key, args)
    if key == "fleet":
        frame, tpls = data
        s, k = _ref_fleet_sample(frame, tpls, 2, 1)
        return {"value": _units(key, args) / s, "unit": "template*Mpx/s", "cores": 1, "kind": "port",
                "sample": f"one FindAll's frame spectra and the tails of {k} of its {len(tpls)} members, 1 thread, "
                          f"scaled to the whole fleet as phase 1 + ({len(tpls)}/{k}) x phase 2 (C restatement of "
                          "the reference's scalar Go path)"}
    times = []
    t_end = time.perf_counter() + budget_s
    while time.perf_counter() < t_end and len(times) < 50:
        times.append(_reference_step(key, args, data, 1))
    s = float(np.mean(times))
    return {"value": _units(key, args) / s, "unit": "template*Mpx/s", "cores": 1, "kind": "port",
            "sample": f"{len(times)} full calls on the same inputs, 1 thread (C restatement of the reference's "
                      "scalar Go path)"}


# --------------------------------------------------------------- GPU arm


def _nvtx(torch):
    """torch.cuda.nvtx, or a no-op stand-in where this torch build has no NVTX."""
    try:
        torch.cuda.nvtx.range_push("probe")
        torch.cuda.nvtx.range_pop()
        return torch.cuda.nvtx
    except Exception:  # noqa: BLE001
        class _Off:
            @staticmethod
            def range_push(_):
                pass

            @staticmethod
            def range_pop():
                pass
        return _Off


def measure(W, form, args, ws, dev, torch, local):
    """Device-resident ms per step (CUDA events on the launching stream, L2
    flushed between steps), the e2e ms through the public host-buffer API
    (pageable and page-locked frames), launches per step, and the clock
    record (sampled through the timed steps, then for the rest of a >= 1 s
    window of the same steps), in one arithmetic form."""
    L = W.L
    W.set_form(form)
    flush = W.flush
    for _ in range(max(3, args.warmup)):
        W.step_dev()
    torch.cuda.synchronize()
    l0 = L.cvm_launch_count()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.time()
        nvtx = _nvtx(torch)
        nvtx.range_push("timed_" + form)  # a profiler's launch list can select the timed steps by this range
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(W.stream)
            W.step_dev()
            ends[i].record(W.stream)
        torch.cuda.synchronize()
        nvtx.range_pop()
        t1 = time.time()
        launches = (L.cvm_launch_count() - l0) // args.steps
        # keep the clocks sampled under the same load for at least 1 s
        while time.time() - t0 < 1.0:
            flush.zero_()
            W.step_dev()
            torch.cuda.synchronize()
    ms = slowest_rank_ms(float(np.mean([s.elapsed_time(e) for s, e in zip(starts, ends)])), ws, dev)
    got = W.dev_result()

    def host_ms(fn):
        for _ in range(2):
            fn()
        t = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            a = time.perf_counter()
            fn()
            t.append(time.perf_counter() - a)
        return slowest_rank_ms(1e3 * float(np.mean(t)), ws, dev)

    e2e_ms = host_ms(W.step_e2e)
    assert W.host_result() == got, "host-buffer and device-resident calls disagree"
    e2e_pinned_ms = host_ms(W.step_e2e_pinned)
    assert W.host_result() == got
    return {"ms": ms, "e2e_ms": e2e_ms, "e2e_pinned_ms": e2e_pinned_ms, "launches": int(launches),
            "clocks": clk.summary(t0, t1), "result": got}


def run_gpu(args):
    import torch
    import cvmatch_gb300 as cvm

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    cvm.SetAutotune(args.autotune == "on")
    key = args.workload
    if key == "fleet":
        W = FleetWorkload(cvm, torch, dev, stream, count=args.templates)
        if args.stats == "epilogue":
            W.fleet.SetStats(cvm.STATS_EPILOGUE)
        W.overlap = args.overlap == "on"
        W.fleet.SetOverlap(W.overlap)
        W.fleet.SetWave(args.wave)
    else:
        W = WORKLOADS[key](cvm, torch, dev, stream)
    W.flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    units = _units(key, args)
    r = measure(W, args.form, args, ws, dev, torch, local)
    others = {f: measure(W, f, args, ws, dev, torch, local) for f in FORM if f != args.form}
    W.set_form(args.form)
    value = replica_throughput(units, r["ms"], ws)

    line = None
    if rank == 0:
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        roof = roofline(W.L, W, torch, r["ms"], args.form, sms, reps=3 if key == "fleet" else 20)
        if args.timeline:
            for nm, a, b in timeline(W.L, W.step_dev, torch):
                sys.stderr.write(f"timeline {nm:24s} {a:8.1f} {b:8.1f} us\n")
        res = r["result"]
        line = {"metric": "template*Mpx/s", "value": value, "unit": "template*Mpx/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": _workload_config(key, ws, args), "form": args.form,
                "e2e": {"value": replica_throughput(units, r["e2e_ms"], ws), "unit": "template*Mpx/s",
                        "h2d_bytes_per_step": int(W.h2d), "d2h_bytes_per_step": int(W.d2h),
                        "ms_per_step": r["e2e_ms"], "host_memory": "pageable (the caller's ordinary memory)",
                        "pinned": {"value": replica_throughput(units, r["e2e_pinned_ms"], ws),
                                   "ms_per_step": r["e2e_pinned_ms"],
                                   "host_memory": "page-locked (cvm_host_alloc)"}},
                "gpu_launches": r["launches"], "clocks": r["clocks"], "roofline": roof,
                "result": list(res) if key != "fleet" else {"members": len(res), "first": list(res[0])},
                # the same workload in every arithmetic form, measured in this run
                "forms": {args.form: {"value": value, "ms_per_step": r["ms"],
                                      "e2e": replica_throughput(units, r["e2e_ms"], ws), "e2e_ms_per_step": r["e2e_ms"]}}}
        for f, o in others.items():
            line["forms"][f] = {"value": replica_throughput(units, o["ms"], ws), "ms_per_step": o["ms"],
                                "e2e": replica_throughput(units, o["e2e_ms"], ws), "e2e_ms_per_step": o["e2e_ms"],
                                "clocks": o["clocks"]}
            line["forms"]["ratio_" + args.form + "_over_" + f] = o["ms"] / r["ms"]
        # the fast forms' tile plans the autotuner chose for this workload's shapes
        try:
            line["autotune"] = cvm.autotune_report()
        except Exception:  # an older library without the tuner
            line["autotune"] = None
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(key, args)
        print(json.dumps(line))
    W.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


# ------------------------------------------------------------- frame stream


def stream_flops(cf, gf, color, gray, W, H):
    def one(fl, tpls, cns):
        bk = fl.buckets(W, H)
        return fleet_flops(bk, [fl.bucket_members(b) for b in range(len(bk))], [(t.shape[1], t.shape[0]) for t in tpls],
                           W, H, cns)
    f, g = one(cf, color, [_alpha_cn(t) for t in color]), one(gf, gray, [1] * len(gray))
    return {k: f[k] + g[k] for k in f}


def _stream_config(args, K):
    return {"workload": "Fleet stream: 1920x1080 RGBA frames, 64 colour templates 24x24..128x96 + 8 gray "
                        "matchers on the gray conversion; each frame moves 5% of the rectangles and redraws "
                        f"sigma=2 noise ({K} precomputed frames cycled)",
            "templates": 72, "parent": [1920, 1080], "l2": "frames stream through (no flush)"}


def run_stream(args):
    """A stream of 1920x1080 RGBA frames against 64 colour templates and
    8 gray matchers on each frame's gray conversion, through cvm_stream (the
    per-frame pipeline replayed as a CUDA graph, two frames in flight, host
    frames copied in and results copied out).  Reports frames/s, template
    Mpx/s (72 templates x 2.07 Mpx per frame) and the per-frame device
    latency p50/p99 (upload start to results back, one frame queued
    ahead), beside the same frames through Fleet.FindAll one call at a time."""
    import torch
    import cvmatch_gb300 as cvm
    frames, color, gray = scene_stream_1920x1080()
    H, W = frames[0].shape[:2]
    cvm.SetAutotune(args.autotune == "on")
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
    nvtx = _nvtx(torch)
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        c0 = time.time()
        nvtx.range_push("timed_stream")  # a profiler's launch list can select the timed frames by this range
        for i in range(nfr):
            st.push(frames[i % K])
            if i >= 1:
                lat.append(st.pull()[2])
        lat.append(st.pull()[2])
        nvtx.range_pop()
        wall = time.perf_counter() - t0
        c1 = time.time()
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
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    peak, src = fp32_peak_tflops(sms)
    flops = sum(stream_flops(cf, gf, color, gray, W, H).values())
    ach = flops * fps / 1e12
    line = {"metric": "template*Mpx/s", "value": fps * mpx, "unit": "template*Mpx/s", "n_gpus": 1,
            "steps": nfr, "warmup": args.warmup, "ms_per_step": 1e3 / fps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": _stream_config(args, K), "form": args.form,
            "frames_per_s": fps, "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
            "graphed": graphed, "gpu_launches": per_frame_launches,
            "findall_per_frame_fps": fps_plain, "clocks": clk.summary(c0, c1),
            "roofline": {"bound": "fp32", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                         "traffic": None, "peak_source": src, "alg_flops_per_step": flops},
            "e2e": {"value": fps * mpx, "unit": "template*Mpx/s", "h2d_bytes_per_step": int(frames[0].nbytes),
                    "d2h_bytes_per_step": int((len(color) + len(gray)) * 24)}, "secondary": True}
    print(json.dumps(line))
    return 0


def run_stream_reference(args):
    """The reference's per-frame work on the host cores: the colour fleet
    (a bounded sample of its member tails, scaled as for the fleet), the
    frame's gray conversion and the gray fleet, per frame."""
    import oracle
    frames, color, gray = scene_stream_1920x1080()
    threads = min(16, os.cpu_count() or 1)
    H, W = frames[0].shape[:2]

    def step(i):
        f = frames[i % len(frames)]
        s, _ = _ref_fleet_sample(f, color, 16, threads)
        t0 = time.perf_counter()
        g = oracle.rgba_to_gray(f)
        oracle.fleet_find_all(gray, g, threads=threads)
        return s + time.perf_counter() - t0

    for i in range(max(1, args.warmup)):
        step(i)
    secs = [step(i) for i in range(args.steps)]
    ms = 1e3 * float(np.mean(secs))
    mpx = (len(color) + len(gray)) * W * H / 1e6
    v = mpx / (ms / 1e3)
    line = {"metric": "template*Mpx/s", "value": v, "unit": "template*Mpx/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": _stream_config(args, len(frames)),
            "cpu_baseline": {"value": v, "unit": "template*Mpx/s", "cores": threads, "kind": "port",
                             "sample": "per frame: the colour fleet's frame spectra and 16 of its 64 member tails "
                                       "(scaled as phase 1 + 4 x phase 2), the gray conversion and the whole gray fleet"},
            "e2e": {"value": v, "unit": "template*Mpx/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--frames", type=int, default=1000, help="frames for --workload stream")
    ap.add_argument("--workload", default="fleet", choices=["fleet", "match", "gray", "map", "stream"],
                    help="fleet (default: the reported line, Fleet.FindAll of 256 templates on 2560x1440) or a "
                         "secondary configuration")
    ap.add_argument("--templates", type=int, default=256, help="fleet size for --workload fleet")
    ap.add_argument("--ref-sample", type=int, default=16,
                    help="member tails timed per step by the fleet's reference arm (the rest scaled)")
    ap.add_argument("--form", default="fast", choices=["exact", "fast", "mixed"],
                    help="arithmetic: fast (default; within 1e-4 of the FP64 definition), mixed (the fast form "
                         "with its 1024-point inverse rows on the tensor cores) or exact (the reference's float32 "
                         "bits; cvm_set_form / cvm_fleet_set_form); every form is measured in each run")
    ap.add_argument("--timeline", action="store_true", help="print one profiled step's launch spans to stderr")
    ap.add_argument("--autotune", default="on", choices=["on", "off"],
                    help="the fast forms' tile-plan autotuner (cvm_set_autotune); off runs newGoPlan's plans")
    ap.add_argument("--stats", default="kernel", choices=["kernel", "epilogue"],
                    help="--workload fleet: window statistics from the statistics kernel (default) or formed in "
                         "the inverse-rows epilogue from the frame's summed-area table (cvm_fleet_set_stats)")
    ap.add_argument("--wave", type=int, default=0,
                    help="--workload fleet: member tails per wave (cvm_fleet_set_wave; 0: the workspace budget's)")
    ap.add_argument("--overlap", default="on", choices=["on", "off"],
                    help="--workload fleet: a wave's inverse rows beside the next wave's statistics and columns "
                         "(cvm_fleet_set_overlap)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "stream":
        return run_stream(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
