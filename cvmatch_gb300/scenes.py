"""The benchmark scene and result file formats of the reference's OpenCV
comparison harness, so a scene set dumped for native OpenCV runs here too.

  CVMS (bench/cmd/dumpscenes/main.go:21-41): "CVMS", int32 LE width,
        int32 LE height, then width*height*4 RGBA bytes, row after row.
  CVMR (bench/cpp/native_bench.cpp:45-53, read by bench/bench_test.go:24-56):
        "CVMR", int32 LE width, int32 LE height, then width*height float32
        LE scores (a MatchMap response).
  manifest.tsv: name, expected x, expected y, parent file, sub file.

``python -m cvmatch_gb300.scenes dump DIR`` writes DIR/<name>.gpu.result.raw
(CVMR) for every manifest entry from this library's MatchMap, for an
element-wise comparison with the native dumps on any machine.
"""
from __future__ import annotations

import os
import struct
import sys
from dataclasses import dataclass
from typing import List

import numpy as np


def write_cvms(path: str, rgba: np.ndarray) -> None:
    rgba = np.ascontiguousarray(rgba, np.uint8)
    if rgba.ndim != 3 or rgba.shape[2] != 4:
        raise ValueError("CVMS holds H x W x 4 RGBA images")
    h, w = rgba.shape[:2]
    with open(path, "wb") as f:
        f.write(b"CVMS" + struct.pack("<ii", w, h))
        f.write(rgba.tobytes())


def read_cvms(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        data = f.read()
    if data[:4] != b"CVMS":
        raise ValueError(f"{path}: bad scene magic")
    w, h = struct.unpack("<ii", data[4:12])
    if len(data) < 12 + w * h * 4:
        raise ValueError(f"{path}: truncated scene")
    return np.frombuffer(data, np.uint8, w * h * 4, 12).reshape(h, w, 4)


def write_cvmr(path: str, resp: np.ndarray) -> None:
    resp = np.ascontiguousarray(resp, "<f4")
    h, w = resp.shape
    with open(path, "wb") as f:
        f.write(b"CVMR" + struct.pack("<ii", w, h))
        f.write(resp.tobytes())


def read_cvmr(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        data = f.read()
    if data[:4] != b"CVMR":
        raise ValueError(f"{path}: bad result dump magic")
    w, h = struct.unpack("<ii", data[4:12])
    n = (len(data) - 12) // 4
    if n < w * h:
        raise ValueError(f"{path}: truncated result dump")
    return np.frombuffer(data, "<f4", w * h, 12).reshape(h, w)


@dataclass
class Scene:
    name: str
    px: int
    py: int
    parent: str
    sub: str


def read_manifest(directory: str) -> List[Scene]:
    out = []
    path = os.path.join(directory, "manifest.tsv")
    if not os.path.exists(path):
        return out
    for line in open(path):
        f = line.rstrip("\n").split("\t")
        if len(f) == 5:
            out.append(Scene(f[0], int(f[1]), int(f[2]), os.path.join(directory, f[3]), os.path.join(directory, f[4])))
    return out


def write_manifest(directory: str, scenes: List[Scene]) -> None:
    with open(os.path.join(directory, "manifest.tsv"), "w") as f:
        for s in scenes:
            f.write(f"{s.name}\t{s.px}\t{s.py}\t{os.path.basename(s.parent)}\t{os.path.basename(s.sub)}\n")


def dump(directory: str) -> int:
    import cvmatch_gb300 as cvm
    n = 0
    for s in read_manifest(directory):
        resp, _, _ = cvm.MatchMap(read_cvms(s.parent), read_cvms(s.sub))
        write_cvmr(os.path.join(directory, s.name + ".gpu.result.raw"), resp)
        n += 1
    return n


if __name__ == "__main__":
    if len(sys.argv) != 3 or sys.argv[1] != "dump":
        sys.exit("usage: python -m cvmatch_gb300.scenes dump DIR")
    print(f"{dump(sys.argv[2])} result maps written")
