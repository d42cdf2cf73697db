"""Seeded random fleets at odd sizes: every member's result in the exact
form bit-identical to the oracle's FindAll (fleet.go:176-332), and in the
fast form within 1e-4 of the FP64 definition (cvmatch_test.go:13-81) with
the extremum locations the FP64 map and the reference's map determine.

The cases sweep the fleet paths' size-dependent branches: frames shorter
than a 16-row block (no block sums), templates too wide for the u32 block
sums, shrunk last bands, several buckets, members whose windows run to the
frame's edge, varying alpha (four-channel members), flat members, and
fleets large enough for the autotuner to time candidate plans.
"""
import numpy as np
import pytest

import cvmatch_gb300 as cvm
import oracle
from oracle import fp64

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _frame(rng, h, w, alpha_varies):
    img = np.empty((h, w, 4), np.uint8)
    img[..., :3] = rng.integers(0, 256, (h, w, 3))
    for _ in range(12):
        rw, rh = int(rng.integers(2, max(3, w // 2))), int(rng.integers(2, max(3, h // 2)))
        x, y = int(rng.integers(0, w - rw + 1)), int(rng.integers(0, h - rh + 1))
        img[y:y + rh, x:x + rw, :3] = rng.integers(0, 256, 3)
    img[..., 3] = rng.integers(0, 256, (h, w)) if alpha_varies else 255
    return img


def _members(rng, img, n, tmax, hmax):
    h, w = img.shape[:2]
    out = []
    for i in range(n):
        tw, th = int(rng.integers(1, min(tmax, w) + 1)), int(rng.integers(1, min(hmax, h) + 1))
        x, y = int(rng.integers(0, w - tw + 1)), int(rng.integers(0, h - th + 1))
        t = img[y:y + th, x:x + tw].copy()
        if i % 5 == 3:
            t[..., :3] = 77  # flat
        out.append(t)
    return out


CASES = [
    # (seed, frame h, frame w, members, max template w, max template h, varying alpha)
    (1, 12, 300, 6, 60, 12, False),      # shorter than a 16-row block
    (2, 150, 1500, 5, 1400, 80, False),   # members up to ~1330 px wide (near the block sums' bound)
    (3, 333, 517, 9, 120, 90, False),     # odd sizes, several buckets
    (4, 200, 260, 7, 200, 150, True),     # varying alpha: four-channel members
    (5, 97, 641, 12, 33, 41, False),      # many small members (autotuned buckets)
    (6, 400, 300, 4, 300, 399, False),    # windows to the frame's edge
]


# and twelve more drawn from a seeded generator: frames 8..600 x 8..900,
# 1..16 members, templates up to the frame
_g = np.random.default_rng(2024)
for _s in range(12):
    _h, _w = int(_g.integers(8, 601)), int(_g.integers(8, 901))
    CASES.append((100 + _s, _h, _w, int(_g.integers(1, 17)), int(_g.integers(1, _w + 1)), int(_g.integers(1, _h + 1)),
                  bool(_g.integers(0, 4) == 0)))


@pytest.mark.parametrize("case", CASES, ids=[f"seed{c[0]}" for c in CASES])
def test_random_fleet_exact_and_fast(case):
    seed, h, w, n, tmax, hmax, alpha = case
    rng = np.random.default_rng(seed)
    img = _frame(rng, h, w, alpha)
    tpls = _members(rng, img, n, tmax, hmax)
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    got = [tuple(r) for r in fleet.FindAll(img)]
    want, ref_maps = oracle.fleet_find_all(tpls, img, threads=16, want_maps=True)
    for i, (g, r) in enumerate(zip(got, want)):
        assert np.float32(g[0]).view(np.uint32) == np.float32(r[0]).view(np.uint32) and g[1:3] == r[1:3], (i, g, r)
        assert np.float32(g[3]).view(np.uint32) == np.float32(r[3]).view(np.uint32) and g[4:6] == r[4:6], (i, g, r)
    fleet.SetForm(cvm.FORM_FAST)
    fast = fleet.FindAll(img)
    F = fp64.Frame(img, 4 if alpha else 3)
    for i, t in enumerate(tpls):
        if ref_maps[i] is None:  # flat member: the reference's fixed answer
            assert tuple(fast[i]) == tuple(got[i]), i
            continue
        fp64.check_extrema(tuple(fast[i]), F.match(t), TOL, ref_map=ref_maps[i], name=f"seed {seed} member {i}")
    assert cvm.device_status() == 0


def _roi_box(roi, tw, th, rw, rh):
    """Result positions [x0, x1) x [y0, y1) whose window lies inside roi."""
    x, y, w, h = roi
    x0, y0 = max(x, 0), max(y, 0)
    return x0, y0, min(x + w - tw + 1, rw), min(y + h - th + 1, rh)


@pytest.mark.parametrize("seed", [301, 302, 303, 304])
def test_random_fleet_regions_of_interest(seed):
    """Random regions of interest on random fleets: in the exact form each
    restricted member's result is the first-occurrence extrema of the
    oracle's FindAll map over its region (bit for bit); in the fast form
    those extrema within 1e-4 of the FP64 map's over the region, located
    where the FP64 and the reference's restricted maps determine them; an
    empty region gives (NaN, -1, -1, NaN, -1, -1)."""
    rng = np.random.default_rng(seed)
    h, w = int(rng.integers(60, 400)), int(rng.integers(60, 600))
    img = _frame(rng, h, w, False)
    # (no flat members: every channel constant over the template, the
    # reference's fixed answer, is covered with a region elsewhere)
    tpls = [t for t in _members(rng, img, 8, min(w, 120), min(h, 100))
            if t[..., :3].reshape(-1, 3).std(axis=0).max() > 0]
    rois = {}
    for i, t in enumerate(tpls):
        if rng.integers(0, 3) == 0:
            continue
        rw_, rh_ = int(rng.integers(1, w + 1)), int(rng.integers(1, h + 1))
        rois[i] = (int(rng.integers(-20, w)), int(rng.integers(-20, h)), rw_, rh_)
    want, maps = oracle.fleet_find_all(tpls, img, threads=16, want_maps=True)
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    for i, r in rois.items():
        fleet.SetROI(i, *r)
    exact = fleet.FindAll(img)
    fleet.SetForm(cvm.FORM_FAST)
    fast = fleet.FindAll(img)
    F = fp64.Frame(img, 3)
    for i, t in enumerate(tpls):
        th, tw = t.shape[:2]
        m = maps[i]
        if i not in rois:
            g = tuple(exact[i])
            assert np.float32(g[0]).view(np.uint32) == np.float32(want[i][0]).view(np.uint32) and g[1:3] == want[i][1:3]
            assert np.float32(g[3]).view(np.uint32) == np.float32(want[i][3]).view(np.uint32) and g[4:6] == want[i][4:6]
            continue
        x0, y0, x1, y1 = _roi_box(rois[i], tw, th, m.shape[1], m.shape[0])
        if x1 <= x0 or y1 <= y0:
            for r in (exact[i], fast[i]):
                assert np.isnan(r[0]) and np.isnan(r[3]) and tuple(r)[1:3] == (-1, -1) and tuple(r)[4:6] == (-1, -1)
            continue
        sub = m[y0:y1, x0:x1]
        iy, ix = np.unravel_index(int(np.argmin(sub)), sub.shape)
        jy, jx = np.unravel_index(int(np.argmax(sub)), sub.shape)
        g = tuple(exact[i])
        assert np.float32(g[0]).view(np.uint32) == np.float32(sub[iy, ix]).view(np.uint32), (i, g)
        assert np.float32(g[3]).view(np.uint32) == np.float32(sub[jy, jx]).view(np.uint32), (i, g)
        assert g[1:3] == (x0 + int(ix), y0 + int(iy)) and g[4:6] == (x0 + int(jx), y0 + int(jy)), (i, g)
        m64 = F.match(t)[y0:y1, x0:x1]
        fp64.check_extrema(tuple(fast[i]), m64, TOL, ref_map=sub, name=f"seed {seed} member {i}", off=(x0, y0))
    assert cvm.device_status() == 0
