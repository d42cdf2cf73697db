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


def test_stream_graph_with_overlapped_waves():
    """A frame stream whose fast-form colour fleet runs in several
    overlapped waves: the side stream's rows join the captured graph, and
    every frame's results equal Fleet.FindAll's on that frame."""
    rng = np.random.default_rng(77)
    H, W = 320, 480
    base = _frame(rng, H, W)
    frames = []
    for i in range(4):
        f = base.copy()
        y, x = int(rng.integers(0, H - 40)), int(rng.integers(0, W - 60))
        f[y:y + 40, x:x + 60, :3] = rng.integers(0, 256, (40, 60, 3), dtype=np.uint8)
        frames.append(f)
    tc = []
    for i in range(7):
        tw, th = int(rng.integers(12, 90)), int(rng.integers(12, 70))
        x, y = int(rng.integers(0, W - tw)), int(rng.integers(0, H - th))
        tc.append(base[y:y + th, x:x + tw].copy())
    tg = [cvm.rgba_to_gray(base[40:70, 60:100])]
    cf = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tc])
    gf = cvm.NewFleet(*[cvm.NewGrayMatcher(t) for t in tg])
    cf.SetForm(cvm.FORM_FAST)
    cf.SetWave(2)  # four waves of the colour fleet, overlapped
    try:
        st = cvm.NewStream(cf, gf, W, H)
        graphed, launches = st.info()
        assert graphed and launches > 0
        got = []
        for i, f in enumerate(frames):
            st.push(f)
            if i >= 1:
                got.append(st.pull())
        got.append(st.pull())
        for f, (rc, rg, ms) in zip(frames, got):
            assert [_bits(r) for r in rc] == [_bits(r) for r in cf.FindAll(f)]
            assert [_bits(r) for r in rg] == [_bits(r) for r in gf.FindAll(cvm.rgba_to_gray(f))]
    finally:
        cf.SetWave(0)
        cf.SetForm(cvm.FORM_EXACT)
    assert cvm.device_status() == 0


def test_c4_fast_form_splits_its_bucket():
    """The fast form's own buckets (fast_buckets): C4's single bucket of the
    reference (256 members up to 192 x 128) runs as two -- the members up
    to 49 rows high on a grid of 9 tiles, the rest on 12 -- while the
    exact form keeps the reference's bucket; both forms' results are held
    to their bars by the full-size tests."""
    import bench
    frame, tpls, _ = bench.scene_fleet_2560x1440()
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    assert len(fleet.buckets(2560, 1440)) == 1  # the reference's bucketing
    fleet.SetForm(cvm.FORM_FAST)
    try:
        fleet.FindAll(frame)
    finally:
        fleet.SetForm(cvm.FORM_EXACT)
    tuned = [e for e in cvm.autotune_report()
             if e.get("fleet") and e.get("frame") == [2560, 1440] and e.get("form") == cvm.FORM_FAST]
    live = [t for t in tpls if t[..., :3].reshape(-1, 3).std(axis=0).max() > 0]  # flat members join no bucket
    nshort = sum(1 for t in live if t.shape[0] <= 49)
    assert 32 <= nshort <= len(live) - 32
    assert any(e["bucket"][1] <= 49 and e["members"] == nshort for e in tuned), tuned
    assert any(e["bucket"][1] > 49 and e["members"] == len(live) - nshort for e in tuned), tuned


def test_split_buckets_with_regions_of_interest_vs_fp64():
    """A fleet whose fast form splits its bucket (short and tall members on
    a tall frame), with regions of interest on every fifth member: every
    sampled member's extrema within 1e-4 of the FP64 map (restricted to its
    region where it has one), at the FP64 map's locations wherever its
    top-2 margin exceeds 1e-4 (cvmatch_test.go:13-81)."""
    from oracle import fp64
    rng = np.random.default_rng(21)
    H, W = 1400, 1200
    frame = _frame(rng, H, W)
    tpls, at = [], []
    for i in range(90):
        if i % 2 == 0:
            tw, th = int(rng.integers(16, 150)), int(rng.integers(12, 40))
        else:
            tw, th = int(rng.integers(16, 150)), int(rng.integers(100, 170))
        x, y = int(rng.integers(0, W - tw)), int(rng.integers(0, H - th))
        tpls.append(frame[y:y + th, x:x + tw].copy())
        at.append((x, y))
    live = [i for i, t in enumerate(tpls) if t[..., :3].reshape(-1, 3).std(axis=0).max() > 0]
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    rois = {}
    for i in live[::5]:
        x, y = at[i]
        rois[i] = (x - 20, y - 20, tpls[i].shape[1] + 60, tpls[i].shape[0] + 60)
        fleet.SetROI(i, *rois[i])
    fleet.SetForm(cvm.FORM_FAST)
    try:
        got = [tuple(r) for r in fleet.FindAll(frame)]
    finally:
        fleet.SetForm(cvm.FORM_EXACT)
    tuned = [e for e in cvm.autotune_report()
             if e.get("fleet") and e.get("frame") == [W, H] and e.get("form") == cvm.FORM_FAST]
    assert sum(1 for e in tuned if e["members"] >= 32) >= 2, tuned  # the bucket ran split
    F = fp64.Frame(frame, 3)
    for i in sorted(set(live[::7]) | set(list(rois)[:6])):
        t = tpls[i]
        th, tw = t.shape[:2]
        m64 = F.match(t)
        off = (0, 0)
        if i in rois:
            x, y, w, h = rois[i]
            x0, y0 = max(x, 0), max(y, 0)
            x1, y1 = min(x + w - tw + 1, m64.shape[1]), min(y + h - th + 1, m64.shape[0])
            m64, off = m64[y0:y1, x0:x1], (x0, y0)
        fp64.check_extrema(got[i], m64, 1e-4, name=f"member {i} {tw}x{th}", off=off)
        assert got[i][4:6] == at[i], (i, got[i], at[i])  # the planted copy
    assert cvm.device_status() == 0
