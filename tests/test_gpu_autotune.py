"""The fast forms' tile-plan autotuner (cvm_set_autotune,
cvm_autotune_report): the first fast-form call of a shape times candidate
plans and caches the fastest; a fleet's buckets are tuned the same way on
trial fleets of their own members; the exact form always keeps newGoPlan's
plan (impl.go:246-295, fleet.go:356-365).  Whatever plan it picks, the scores meet the fast form's
bar against FP64 (cvmatch_test.go:13-81), repeat exactly on later calls,
and Matcher.Find equals the one-shot Match of the same shape.
"""
import numpy as np
import pytest

import cvmatch_gb300 as cvm
import oracle
from oracle import fp64

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _scene(seed, h, w):
    rng = np.random.default_rng(seed)
    img = np.empty((h, w, 4), np.uint8)
    img[..., :3] = rng.integers(0, 256, (h, w, 3))
    img[..., 3] = 255
    for _ in range(30):
        rw, rh = int(rng.integers(8, w // 3)), int(rng.integers(8, h // 3))
        x, y = int(rng.integers(0, w - rw)), int(rng.integers(0, h - rh))
        img[y:y + rh, x:x + rw, :3] = rng.integers(0, 256, 3)
    return img


def _entry(frame_wh, tpl_wh, form):
    for e in cvm.autotune_report():
        if e["frame"] == list(frame_wh) and e.get("template") == list(tpl_wh) and e["form"] == form:
            return e
    return None


@pytest.mark.parametrize("form", [cvm.FORM_FAST, cvm.FORM_MIXED])
def test_tuned_plan_meets_the_bar_and_repeats(form):
    img = _scene(211 + form, 700, 1300)
    t = img[300:340, 600:664].copy()
    prev_t = cvm.SetAutotune(True)
    prev = cvm.SetForm(form)
    try:
        m1, _, _ = cvm.MatchMap(img, t)
        e = _entry((1300, 700), (64, 40), form)
        assert e is not None and len(e["candidates"]) >= 2
        base = oracle.plan(64, 40, 1300 - 63, 700 - 39)
        assert e["candidates"][0]["plan"] == [base.dft_w, base.dft_h]  # newGoPlan's choice is timed first
        assert all(c["ms"] > 0 for c in e["candidates"])
        print(f"\ntuned plan {e['plan']} from {[(c['plan'], round(c['ms'], 4)) for c in e['candidates']]}")
        m2, _, _ = cvm.MatchMap(img, t)
        assert np.array_equal(m1.view(np.uint32), m2.view(np.uint32))   # the cached plan: identical results
        r = tuple(cvm.Match(img, t))
        assert tuple(cvm.NewMatcher(t).Find(img)) == r                     # Matcher runs the same plan
        m64 = fp64.ref_match_f64(img, t, 3)
        err = np.abs(m1.astype(np.float64) - m64).max()
        print(f"tuned-plan map max|err| against FP64 {err:.2e}")
        assert err <= TOL
        assert fp64.first_argmax(m1) == (600, 300)
    finally:
        cvm.SetForm(prev)
        cvm.SetAutotune(prev_t)
    assert cvm.device_status() == 0


def test_exact_form_never_tunes_and_stays_bit_exact():
    img = _scene(223, 500, 900)
    t = img[100:148, 200:232].copy()
    prev_t = cvm.SetAutotune(True)
    try:
        assert cvm.SetForm(cvm.FORM_EXACT) is not None
        got, m = cvm.match_u8(img, t, 3)
        assert _entry((900, 500), (32, 48), cvm.FORM_EXACT) is None
        want, wm = oracle.match_u8(img, t, 3, threads=16)
        assert got == want and np.array_equal(m.view(np.uint32), wm.view(np.uint32))
    finally:
        cvm.SetAutotune(prev_t)


def test_autotune_off_runs_newgoplan():
    img = _scene(227, 480, 800)
    t = img[50:90, 60:110].copy()
    prev_t = cvm.SetAutotune(False)
    prev = cvm.SetForm(cvm.FORM_FAST)
    try:
        m, _, _ = cvm.MatchMap(img, t)
        assert _entry((800, 480), (50, 40), cvm.FORM_FAST) is None
        err = np.abs(m.astype(np.float64) - fp64.ref_match_f64(img, t, 3)).max()
        assert err <= TOL
    finally:
        cvm.SetForm(prev)
        cvm.SetAutotune(prev_t)


def test_fleet_buckets_tuned_meet_the_bar():
    """A 24-member fleet on 2560 x 1440 in the fast form: each bucket with
    four or more members is tuned (its entry lists the timed candidates,
    newGoPlan's first), every member meets the bar against FP64 and the
    second FindAll repeats the first exactly."""
    import bench
    frame, tpls, where = bench.scene_fleet_2560x1440(count=24)
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    prev_t = cvm.SetAutotune(True)
    try:
        fleet.SetForm(cvm.FORM_FAST)
        r1 = fleet.FindAll(frame)
        r2 = fleet.FindAll(frame)
    finally:
        cvm.SetAutotune(prev_t)
    assert [tuple(r) for r in r1] == [tuple(r) for r in r2]
    tuned = [e for e in cvm.autotune_report() if e.get("fleet") and e["frame"] == [2560, 1440]]
    big = [b for b in fleet.buckets(2560, 1440) if b[8] >= 4]
    for e in tuned:
        base = oracle.plan(e["bucket"][0], e["bucket"][1], 2560 - e["bucket"][0] + 1, 1440 - e["bucket"][1] + 1)
        assert e["candidates"][0]["plan"] == [base.dft_w, base.dft_h]
        assert all(c["ms_per_member"] >= 0 and c["ms"] > 0 for c in e["candidates"])
        print(f"\nbucket {e['bucket']} x{e['members']}: plan {e['plan']} from "
              f"{[(c['plan'], round(c['ms'], 3)) for c in e['candidates']]}")
    assert tuned or not big
    _, ref_maps = oracle.fleet_find_all(tpls, frame, threads=16, want_maps=True)
    F = fp64.Frame(frame, 3)
    for i, t in enumerate(tpls):
        fp64.check_extrema(tuple(r1[i]), F.match(t), TOL, ref_map=ref_maps[i], name=f"member {i}")
        if where[i] is not None:
            assert (r1[i].MaxX, r1[i].MaxY) == where[i]
    assert cvm.device_status() == 0
