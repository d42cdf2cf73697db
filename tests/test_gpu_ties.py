"""First occurrence under dense ties: the extrema scan's strict compares
(minMaxLoc as impl.go:1023-1047 and 1104-1112 keep it) must report the
first position in raster order among equal values, also when the equal
values sit in different CTAs, tiles and row pairs and meet only in the
partial-extrema merge -- the GPU counterpart of the reference's
TestMinMaxRowKernel with ties in every lane (impl_simd_test.go:71-122).

On a periodic frame the score map holds the template's copies every
period; the float32 ladder clamps the ones whose rounded quotient reaches
1 to exactly 1.0 (and windows below the lim guard score exactly 0), so the
maximum repeats many times.  The exact form must give the oracle's map
bit for bit and the oracle's (the reference's) first-occurrence extrema,
for single matches and for a fleet."""
import numpy as np
import pytest

import cvmatch_gb300 as cvm
import oracle

pytestmark = pytest.mark.gpu


def _periodic(h, w, period, seed, gray=False):
    rng = np.random.default_rng(seed)
    tile = rng.integers(0, 256, (period, period, 4), dtype=np.uint8)
    frame = np.tile(tile, (h // period + 1, w // period + 1, 1))[:h, :w].copy()
    frame[..., 3] = 255
    if gray:
        frame = oracle.rgba_to_gray(frame)
    return np.ascontiguousarray(frame)


def _first(m, fn):
    flat = np.flatnonzero(m == fn(m))[0]
    return int(flat % m.shape[1]), int(flat // m.shape[1])


@pytest.mark.parametrize("h,w,period,ty,tx,th,tw,gray", [
    (600, 1100, 16, 32, 48, 48, 64, False),
    (480, 1400, 8, 40, 16, 24, 40, False),
    (700, 900, 32, 64, 96, 64, 96, True),
])
def test_dense_ties_match_first_occurrence(h, w, period, ty, tx, th, tw, gray):
    frame = _periodic(h, w, period, seed=h + w, gray=gray)
    tpl = np.ascontiguousarray(frame[ty:ty + th, tx:tx + tw])
    cn = 1 if gray else 3
    prev = cvm.SetForm(cvm.FORM_EXACT)
    try:
        got, gmap = cvm.match_u8(frame, tpl, cn)
    finally:
        cvm.SetForm(prev)
    want, wmap = oracle.match_u8(frame, tpl, cn, threads=16)
    assert np.array_equal(gmap.view(np.uint32), wmap.view(np.uint32))
    ties = int(np.count_nonzero(wmap == wmap.max()))
    assert ties >= 4, ties  # the case exercises ties
    assert tuple(got[4:6]) == _first(wmap, np.max) and tuple(got[1:3]) == _first(wmap, np.min)
    assert tuple(got) == tuple(want)
    assert cvm.device_status() == 0


def test_dense_ties_fleet_first_occurrence():
    frame = _periodic(720, 1280, 16, seed=5)
    tpls = [np.ascontiguousarray(frame[y:y + th, x:x + tw])
            for (y, x, th, tw) in ((16, 32, 48, 48), (64, 80, 32, 96), (0, 0, 40, 24), (96, 160, 64, 64))]
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    got = [tuple(r) for r in fleet.FindAll(frame)]
    want, maps = oracle.fleet_find_all(tpls, frame, threads=16, want_maps=True)
    for i, m in enumerate(maps):
        assert int(np.count_nonzero(m == m.max())) >= 2, i
        assert got[i][4:6] == _first(m, np.max) and got[i][1:3] == _first(m, np.min), (i, got[i])
        assert np.float32(got[i][3]).view(np.uint32) == np.float32(want[i][3]).view(np.uint32)
        assert np.float32(got[i][0]).view(np.uint32) == np.float32(want[i][0]).view(np.uint32)
    assert cvm.device_status() == 0
