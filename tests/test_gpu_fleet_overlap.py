"""Overlapped fleet waves (cvm_fleet_set_overlap, the fast form's default):
a wave's inverse rows run on a side stream beside the next wave's window
statistics and column pass, the waves alternating between two workspaces.
Only the schedule changes -- every member's tail runs the same kernels on
the same data -- so the results must be the same bits as with the waves in
sequence and as with one wave for the whole fleet.  Small waves
(cvm_fleet_set_wave) force many waves, across several buckets, so that
each workspace is reused many times behind the rows that last read it."""
import numpy as np
import pytest

import cvmatch_gb300 as cvm

pytestmark = pytest.mark.gpu


def _bits(r):
    r = tuple(r)
    return (int(np.float32(r[0]).view(np.uint32)), r[1], r[2], int(np.float32(r[3]).view(np.uint32)), r[4], r[5])


def _frame(rng, h, w):
    img = np.empty((h, w, 4), np.uint8)
    img[..., :3] = rng.integers(0, 256, (h, w, 3))
    for _ in range(15):
        rw, rh = int(rng.integers(4, w // 3)), int(rng.integers(4, h // 3))
        x, y = int(rng.integers(0, w - rw)), int(rng.integers(0, h - rh))
        img[y:y + rh, x:x + rw, :3] = rng.integers(0, 256, 3)
    img[..., 3] = 255
    return img


def _runs(fleet, frame, wave):
    out = {}
    fleet.SetForm(cvm.FORM_FAST)
    try:
        for name, w, ov in (("one wave", 0, True), ("sequence", wave, False), ("overlapped", wave, True)):
            fleet.SetWave(w)
            fleet.SetOverlap(ov)
            fleet.FindAll(frame)  # plans and spectra for this schedule
            out[name] = [_bits(r) for r in fleet.FindAll(frame)]
    finally:
        fleet.SetWave(0)
        fleet.SetOverlap(True)
        fleet.SetForm(cvm.FORM_EXACT)
    return out


@pytest.mark.parametrize("seed,n,wave", [(1, 20, 3), (2, 33, 4), (3, 9, 1)])
def test_overlapped_waves_equal_sequence_and_one_wave(seed, n, wave):
    rng = np.random.default_rng(seed)
    frame = _frame(rng, 600, 900)
    tpls = []
    for i in range(n):
        # small, wide and tall members: bucketize keeps them in three buckets
        k = i % 3
        if k == 0:
            tw, th = int(rng.integers(8, 60)), int(rng.integers(8, 60))
        elif k == 1:
            tw, th = int(rng.integers(250, 400)), int(rng.integers(6, 16))
        else:
            tw, th = int(rng.integers(6, 16)), int(rng.integers(250, 400))
        x, y = int(rng.integers(0, 900 - tw)), int(rng.integers(0, 600 - th))
        tpls.append(frame[y:y + th, x:x + tw].copy())
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    assert len(fleet.buckets(900, 600)) == 3
    out = _runs(fleet, frame, wave)
    assert out["overlapped"] == out["sequence"] == out["one wave"]
    assert cvm.device_status() == 0


def test_c4_overlapped_waves_equal_sequence():
    import bench
    frame, tpls, _ = bench.scene_fleet_2560x1440()
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    fleet.SetForm(cvm.FORM_FAST)
    try:
        fleet.SetOverlap(False)
        fleet.FindAll(frame)
        seq = [_bits(r) for r in fleet.FindAll(frame)]
        fleet.SetOverlap(True)
        ovl = [_bits(r) for r in fleet.FindAll(frame)]
    finally:
        fleet.SetOverlap(True)
        fleet.SetForm(cvm.FORM_EXACT)
    assert len(ovl) == 256 and ovl == seq
    assert cvm.device_status() == 0
