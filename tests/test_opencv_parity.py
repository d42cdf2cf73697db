"""The reference's OpenCV comparison harness (bench/bench_test.go:24-107)
on this library: the scene set dumped for native OpenCV (CVMS scenes, a
manifest, CVMR response dumps from bench/cpp/native_bench) is matched with
MatchMap / Match here and compared element by element (<= 1e-3) and at the
peak (value within 1e-4; location equal to OpenCV's first-occurrence argmax
unless OpenCV's own score there is within 2e-3 of its max).  No OpenCV
build exists in this environment, so the GPU comparison runs only where a
dump directory is supplied (CVMATCH_SCENES=<dir>) -- as the reference's test
skips without dumps.  The format round trip always runs."""
import os

import numpy as np
import pytest

from cvmatch_gb300 import scenes

SCENES = os.environ.get("CVMATCH_SCENES", "")


def test_formats_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, (7, 11, 4), dtype=np.uint8)
    p = str(tmp_path / "a.parent.raw")
    scenes.write_cvms(p, img)
    raw = open(p, "rb").read()
    assert raw[:4] == b"CVMS" and int.from_bytes(raw[4:8], "little") == 11 and int.from_bytes(raw[8:12], "little") == 7
    assert np.array_equal(scenes.read_cvms(p), img)
    m = rng.random((5, 9)).astype(np.float32)
    r = str(tmp_path / "a.result.raw")
    scenes.write_cvmr(r, m)
    assert np.array_equal(scenes.read_cvmr(r).view(np.uint32), m.view(np.uint32))
    scenes.write_manifest(str(tmp_path), [scenes.Scene("a", 3, 4, p, p)])
    s = scenes.read_manifest(str(tmp_path))
    assert len(s) == 1 and (s[0].name, s[0].px, s[0].py) == ("a", 3, 4)


def _with_dumps():
    if not SCENES:
        pytest.skip("no native OpenCV result dumps (set CVMATCH_SCENES to a dumpscenes directory)")
    found = [s for s in scenes.read_manifest(SCENES) if os.path.exists(os.path.join(SCENES, s.name + ".result.raw"))]
    if not found:
        pytest.skip("no native result dumps present")
    return found


@pytest.mark.gpu
def test_full_map_parity_with_native():
    import cvmatch_gb300 as cvm
    for s in _with_dumps():
        want = scenes.read_cvmr(os.path.join(SCENES, s.name + ".result.raw"))
        got, w, h = cvm.MatchMap(scenes.read_cvms(s.parent), scenes.read_cvms(s.sub))
        assert (h, w) == want.shape, s.name
        assert float(np.max(np.abs(got.astype(np.float64) - want))) <= 1e-3, s.name


@pytest.mark.gpu
def test_native_peak_values():
    import cvmatch_gb300 as cvm
    for s in _with_dumps():
        want = scenes.read_cvmr(os.path.join(SCENES, s.name + ".result.raw"))
        ww = want.shape[1]
        i = int(np.argmax(want))  # first occurrence, minMaxLoc's order
        cpp_max = float(want.flat[i])
        _, _, _, max_v, max_x, max_y = cvm.Match(scenes.read_cvms(s.parent), scenes.read_cvms(s.sub))
        assert abs(max_v - cpp_max) <= 1e-4, s.name
        if (max_x, max_y) != (i % ww, i // ww):
            assert cpp_max - float(want[max_y, max_x]) <= 2e-3, s.name
