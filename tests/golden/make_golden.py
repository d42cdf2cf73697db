"""Generates tests/golden/golden.json: fixed inputs and the oracle's outputs.

Run from the repository root:  python tests/golden/make_golden.py

The oracle (oracle/cvm_oracle.c) restates the reference's scalar Go path
op for op and is itself pinned to the reference's recorded golden hash of
case 110 (golden_hashes_test.go:21) and its plan pins (plan_test.go:12-28).
Inputs come from tests/golden/synth.py (splitmix64, platform independent),
so the fixture reproduces on any machine: the CPU tests check the oracle
against it, the GPU tests check the CUDA library against it.

Map digests are SHA-256 over the float32 little-endian map bytes followed
by the six extrema (float32 bits / int32); the reference's own FNV-1a
goldenHash (impl_golden_test.go:27-44) is used for case 110, whose
recorded value comes from the reference.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import oracle  # noqa: E402
from synth import image  # noqa: E402

# The reference's golden shapes (impl_golden_test.go:60-71) on synthetic
# inputs, plus shapes that reach the shrunk last band (impl.go:573-610), an
# odd-log2 row transform and larger multi-tile colour cases.
SOLO_CASES = [
    # name, iw, ih, tw, th, cn, step, ipad, tpad, seed
    ("grayscale", 97, 61, 17, 13, 1, 1, 0, 0, 101),
    ("full RGBA", 97, 61, 17, 13, 4, 4, 0, 0, 102),
    ("RGBA alpha skipped cn3 step4", 120, 90, 24, 18, 3, 4, 0, 0, 103),
    ("strided rows", 300, 200, 31, 29, 1, 1, 7, 3, 104),
    ("template == image", 64, 64, 64, 64, 1, 1, 0, 0, 105),
    ("1x1 template", 50, 40, 1, 1, 4, 4, 0, 0, 106),
    ("multi-block tiling", 640, 400, 96, 32, 3, 4, 0, 0, 107),
    ("packed RGB step3", 128, 96, 5, 4, 3, 3, 0, 0, 108),
    ("tall template", 40, 300, 33, 257, 1, 1, 0, 0, 109),
    ("shrunk band gray", 316, 330, 31, 29, 1, 1, 0, 0, 111),
    ("shrunk band rgba", 316, 359, 24, 18, 4, 4, 0, 0, 112),
    ("shrunk band narrow", 40, 533, 9, 33, 1, 1, 0, 0, 113),
    ("wide gray", 1000, 120, 64, 48, 1, 1, 0, 0, 114),
    ("rgba 2 channels step4", 150, 100, 20, 12, 2, 4, 0, 0, 115),
    ("1-wide template", 200, 60, 1, 40, 1, 1, 0, 0, 116),
    ("1-tall template", 60, 200, 40, 1, 1, 1, 0, 0, 117),
]

FLEET_CASES = [
    # name, pw, ph, step, [(w, h, x, y) crops or (w, h, -seed) independent], seed
    ("fleet colour", 400, 300, 4, [(24, 24, 10, 12), (96, 32, 200, 40), (48, 48, 60, 200), (16, 16, 300, 250),
                                   (64, 40, -7, 0), (30, 90, 150, 100)], 201),
    ("fleet gray", 360, 240, 1, [(24, 24, 5, 7), (80, 30, 100, 150), (16, 64, 300, 20), (50, 50, -9, 0)], 202),
    ("fleet orthogonal", 420, 360, 4, [(300, 8, 52, 40), (8, 300, 300, 30), (20, 20, 100, 100)], 203),
]


def digest(res: np.ndarray, t) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(res, "<f4").tobytes())
    h.update(np.array([np.float32(t[0]).view(np.uint32), t[1] & 0xFFFFFFFF, t[2] & 0xFFFFFFFF,
                       np.float32(t[3]).view(np.uint32), t[4] & 0xFFFFFFFF, t[5] & 0xFFFFFFFF], "<u4").tobytes())
    return h.hexdigest()


def solo_inputs(c):
    name, iw, ih, tw, th, cn, step, ipad, tpad, seed = c
    img = image(seed, ih, iw, step, ipad)
    tpl = image(seed + 1000, th, tw, step, tpad)
    return img, tpl


def fleet_inputs(c):
    name, pw, ph, step, specs, seed = c
    parent = image(seed, ph, pw, step)
    if step == 4:
        parent = parent.copy()
        parent[..., 3] = 255
    tpls = []
    for (w, h, x, y) in specs:
        if x < 0:
            t = image(-x, h, w, step).copy()
            if step == 4:
                t[..., 3] = 255
        else:
            t = parent[y:y + h, x:x + w].copy()
        tpls.append(t)
    return parent, tpls


def canary110():
    iw, ih, tw, th = 200, 150, 32, 32
    img = np.full((ih, iw), 128, np.uint8)
    tpl = np.full((th, tw), 128, np.uint8)
    img[75, 100] = 129
    tpl[5, 7] = 129
    return img, tpl


REFERENCE_PINS = {
    # golden_hashes_test.go:21 -- the reference's recorded FNV-1a 64 of case 110
    "case110_fnv": "0x99534488138e0635",
}


def main():
    out = {"reference_pins": REFERENCE_PINS, "solo": [], "fleet": []}
    for c in SOLO_CASES:
        img, tpl = solo_inputs(c)
        t, res = oracle.match_u8(img, tpl, c[5], threads=4)
        out["solo"].append({"case": list(c), "tuple": [float(t[0]), t[1], t[2], float(t[3]), t[4], t[5]],
                            "digest": digest(res, t)})
    for c in FLEET_CASES:
        parent, tpls = fleet_inputs(c)
        rs = oracle.fleet_find_all(tpls, parent, threads=4)
        out["fleet"].append({"case": [c[0], c[1], c[2], c[3], [list(s) for s in c[4]], c[5]],
                             "results": [[float(r[0]), r[1], r[2], float(r[3]), r[4], r[5]] for r in rs]})
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", len(out["solo"]), "solo and", len(out["fleet"]), "fleet fixtures")


if __name__ == "__main__":
    main()
