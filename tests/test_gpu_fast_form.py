"""The fast form (CVM_FORM_FAST) against the FP64 definition, at the
metric's bar.

The fast form leaves the reference's float32 op sequence (zero-mean
templates, the frame offset by -128, channels summed in the frequency
domain), so its scores are checked against the FP64 TM_CCOEFF_NORMED
definition of cvmatch_test.go:13-81 rather than bit for bit: every score
(maps) and every extremum within TOL = 1e-4 of the FP64 value, and every
extremum's location equal to the FP64 map's first-occurrence location
wherever that map's top-2 margin exceeds TOL, and to the reference's own
(the oracle's float32 map, bit-identical to the reference's) wherever the
reference map's margin does.  The measured errors are printed (pytest -s).
"""
import numpy as np
import pytest

import cvmatch_gb300 as cvm
import oracle
from oracle import fp64

pytestmark = pytest.mark.gpu

TOL = 1e-4


def scene(seed, h, w):
    """Noise background, flat rectangles and horizontal gradients (UI-like
    near-flat windows are where float32 correlation loses the most)."""
    rng = np.random.default_rng(seed)
    img = np.empty((h, w, 4), np.uint8)
    img[..., :3] = rng.integers(0, 256, (h, w, 3))
    img[..., 3] = 255
    for i in range(24):
        rw, rh = rng.integers(4, max(5, w // 3)), rng.integers(4, max(5, h // 3))
        x, y = rng.integers(0, w - rw), rng.integers(0, h - rh)
        if i % 3 == 2:
            ramp = np.linspace(rng.integers(0, 128), rng.integers(128, 256), rw)
            img[y:y + rh, x:x + rw, :3] = ramp[None, :, None].astype(np.uint8)
        else:
            img[y:y + rh, x:x + rw, :3] = rng.integers(0, 256, 3)
    return img


def members(img, seed):
    rng = np.random.default_rng(seed)
    sizes = [(24, 24), (64, 48), (33, 17), (48, 40), (16, 16), (40, 56)]
    tpls, at = [], []
    for i, (w, h) in enumerate(sizes):
        x, y = int(rng.integers(0, img.shape[1] - w)), int(rng.integers(0, img.shape[0] - h))
        t = img[y:y + h, x:x + w].astype(np.int32)
        if i % 2:  # a*x+b shifted copy
            t = np.clip(np.rint(t * rng.uniform(0.9, 1.1) + rng.uniform(-10, 10)), 0, 255)
        t = t.astype(np.uint8)
        t[..., 3] = 255
        tpls.append(t)
        at.append((x, y))
    absent = scene(seed + 100, 30, 44)  # from an independent seed
    tpls.append(absent)
    at.append(None)
    return tpls, at


def check(got, m64, name, ref_map=None, off=(0, 0)):
    return fp64.check_extrema(tuple(got), m64, TOL, ref_map=ref_map, name=name, off=off)


@pytest.mark.parametrize("gray", [False, True])
def test_fast_fleet_vs_fp64(gray):
    img = scene(5, 300, 420)
    tpls, at = members(img, 7)
    if gray:
        ms = [cvm.NewGrayMatcher(t) for t in tpls]
    else:
        ms = [cvm.NewMatcher(t) for t in tpls]
    fleet = cvm.NewFleet(*ms)
    fleet.SetForm(cvm.FORM_FAST)
    got = fleet.FindAll(img)
    src = oracle.rgba_to_gray(img) if gray else img
    tts = [oracle.rgba_to_gray(t) if gray else t for t in tpls]
    _, ref_maps = oracle.fleet_find_all(tts, src, threads=16, want_maps=True)
    worst = 0.0
    for i, t in enumerate(tpls):
        tt = tts[i]
        m64 = oracle.ref_match_f64(src, tt, 1 if gray else 3, threads=16)
        worst = max(worst, check(got[i], m64, f"member {i} {t.shape[1]}x{t.shape[0]}", ref_map=ref_maps[i]))
        if at[i] is not None and i % 2 == 0:  # exact crops are found where they were cut
            assert (got[i].MaxX, got[i].MaxY) == at[i]
    print(f"\nworst extremum error against FP64: {worst:.2e}")


def test_fast_fleet_varying_alpha_member():
    img = scene(9, 240, 320)
    t = img[50:90, 100:148].copy()
    t.reshape(-1, 4)[::3, 3] = np.arange(t.reshape(-1, 4)[::3].shape[0]) % 256  # cn = 4 for this member
    flat = np.full((20, 20, 4), 77, np.uint8)
    flat[..., 3] = 255
    tpls = [t, img[10:42, 20:52].copy(), flat]
    fleet = cvm.NewFleet(*[cvm.NewMatcher(x) for x in tpls])
    fleet.SetForm(cvm.FORM_FAST)
    got = fleet.FindAll(img)
    _, ref_maps = oracle.fleet_find_all(tpls, img, threads=16, want_maps=True)
    check(got[0], oracle.ref_match_f64(img, t, 4, threads=16), "varying alpha (cn 4)", ref_map=ref_maps[0])
    check(got[1], oracle.ref_match_f64(img, tpls[1], 3, threads=16), "constant alpha (cn 3)", ref_map=ref_maps[1])
    assert tuple(got[2]) == (1.0, 0, 0, 1.0, 0, 0)  # flat member: impl.go:1137-1144


def test_fast_fleet_roi_member():
    img = scene(13, 260, 380)
    t = img[120:150, 200:240].copy()
    fleet = cvm.NewFleet(cvm.NewMatcher(t), cvm.NewMatcher(img[20:40, 30:60].copy()))
    fleet.SetForm(cvm.FORM_FAST)
    fleet.SetROI(0, 150, 90, 140, 100)
    got = fleet.FindAll(img)
    m64 = oracle.ref_match_f64(img, t, 3, threads=16)
    th, tw = t.shape[:2]
    sub = m64[90:90 + 100 - th + 1, 150:150 + 140 - tw + 1]
    _, ref_maps = oracle.fleet_find_all([t, img[20:40, 30:60].copy()], img, threads=16, want_maps=True)
    ref_sub = ref_maps[0][90:90 + 100 - th + 1, 150:150 + 140 - tw + 1]
    check(got[0], sub, "ROI member", ref_map=ref_sub, off=(150, 90))
    assert (got[0].MaxX, got[0].MaxY) == (200, 120)
    assert 150 <= got[0].MinX < 150 + 140 - tw + 1 and 90 <= got[0].MinY < 90 + 100 - th + 1


def test_form_switch_restores_bit_exact_results():
    img = scene(17, 200, 300)
    tpls, _ = members(img, 19)
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    exact = fleet.FindAll(img)
    want = oracle.fleet_find_all(tpls, img, threads=8)
    fleet.SetForm(cvm.FORM_FAST)
    fast = fleet.FindAll(img)
    fleet.SetForm(cvm.FORM_EXACT)
    again = fleet.FindAll(img)
    for e, a, w in zip(exact, again, want):
        assert tuple(e) == tuple(a) == tuple(w)
    assert any(tuple(f) != tuple(e) for f, e in zip(fast, exact))  # the fast form is a different arithmetic
    with pytest.raises(cvm.CvmatchError):
        fleet.SetForm(7)


# ------------------------------------------------- one-shot matches, Matcher


@pytest.fixture
def fast_form():
    prev = cvm.SetForm(cvm.FORM_FAST)
    yield
    cvm.SetForm(prev)


def ref(img, t, cn):
    """The reference's own float32 map (the oracle is bit-identical to it)."""
    return oracle.match_u8(img, t, cn, threads=16)[1]


def map_check(m, m64, name, tol=TOL, ref_map=None):
    """Every score within tol of FP64, and the map's first-occurrence
    extrema located as check() requires."""
    err = np.abs(m.astype(np.float64) - m64)
    print(f"\n{name}: map max|err| {err.max():.2e}  >1e-4: {int((err > 1e-4).sum())} of {err.size}")
    assert err.max() <= tol
    (mnx, mny), (mxx, mxy) = fp64.first_argmin(m), fp64.first_argmax(m)
    check((m[mny, mnx], mnx, mny, m[mxy, mxx], mxx, mxy), m64, name, ref_map=ref_map)
    return err.max()


def test_fast_match_map_vs_fp64(fast_form):
    img = scene(23, 260, 400)
    t = img[100:140, 150:214].copy()
    m, _, _ = cvm.MatchMap(img, t)
    map_check(m, oracle.ref_match_f64(img, t, 3, threads=16), "MatchMap RGBA", ref_map=ref(img, t, 3))
    # Match returns the map's first-occurrence extrema
    r = tuple(cvm.Match(img, t))
    iy, ix = np.unravel_index(int(np.argmin(m)), m.shape)
    jy, jx = np.unravel_index(int(np.argmax(m)), m.shape)
    assert r == (float(m[iy, ix]), ix, iy, float(m[jy, jx]), jx, jy)
    assert (r[4], r[5]) == (150, 100)
    # MatchGray
    g, gt = oracle.rgba_to_gray(img), oracle.rgba_to_gray(t)
    _, mg = cvm.match_u8(g, gt, 1)
    map_check(mg, oracle.ref_match_f64(g, gt, 1, threads=16), "gray", ref_map=ref(g, gt, 1))


def test_fast_varying_alpha_map(fast_form):
    img = scene(29, 200, 300)
    img[..., 3] = np.arange(300, dtype=np.uint8)[None, :]  # parent alpha varies: cn = 4
    t = img[60:90, 80:120].copy()
    m, _, _ = cvm.MatchMap(img, t)
    map_check(m, oracle.ref_match_f64(img, t, 4, threads=16), "MatchMap RGBA, varying alpha", ref_map=ref(img, t, 4))
    jy, jx = np.unravel_index(int(np.argmax(m)), m.shape)
    assert (jx, jy) == (80, 60)


def test_fast_matcher_equals_one_shot(fast_form):
    img = scene(31, 240, 360)
    t = img[30:62, 40:88].copy()
    m = cvm.NewMatcher(t)
    a, b = m.Find(img), cvm.Match(img, t)
    assert tuple(a) == tuple(b)  # same zero-mean spectra from host or device sums
    cvm.SetForm(cvm.FORM_EXACT)  # the matcher rebuilds its spectra for the exact form
    assert tuple(m.Find(img)) == oracle.match_u8(img, t, 3, want_map=False)[0]


def test_fast_flat_template_and_exact_default():
    assert cvm.SetForm(cvm.FORM_FAST) == cvm.FORM_EXACT
    try:
        img = scene(37, 120, 160)
        flat = np.full((20, 30, 4), 50, np.uint8)
        flat[..., 3] = 255
        assert tuple(cvm.Match(img, flat)) == (1.0, 0, 0, 1.0, 0, 0)  # impl.go:1137-1144
        m, _, _ = cvm.MatchMap(img, flat)
        assert (m == 1.0).all()
    finally:
        cvm.SetForm(cvm.FORM_EXACT)
    with pytest.raises(cvm.CvmatchError):
        cvm.SetForm(5)


def test_fast_stream_equals_fast_find_all():
    """A frame stream whose fleets are in the fast form gives exactly their
    fast-form FindAll results on every frame (same kernels, graph replay)."""
    H, W = 260, 380
    base = scene(41, H, W)
    rng = np.random.default_rng(43)
    frames = []
    for _ in range(4):
        f = base.copy()
        y, x = int(rng.integers(0, H - 40)), int(rng.integers(0, W - 60))
        f[y:y + 40, x:x + 60, :3] = rng.integers(0, 256, (40, 60, 3), dtype=np.uint8)
        frames.append(f)
    cf = cvm.NewFleet(*[cvm.NewMatcher(t) for t in (base[10:34, 20:60].copy(), base[100:150, 200:230].copy())])
    gf = cvm.NewFleet(cvm.NewGrayMatcher(oracle.rgba_to_gray(base[50:80, 50:90])))
    cf.SetForm(cvm.FORM_FAST)
    gf.SetForm(cvm.FORM_FAST)
    st = cvm.NewStream(cf, gf, W, H)
    got = []
    for i, f in enumerate(frames):
        st.push(f)
        if i >= 1:
            got.append(st.pull())
    got.append(st.pull())
    for f, (rc, rg, _) in zip(frames, got):
        assert [tuple(r) for r in rc] == [tuple(r) for r in cf.FindAll(f)]
        assert [tuple(r) for r in rg] == [tuple(r) for r in gf.FindAll(oracle.rgba_to_gray(f))]


# ------------------------------------------------ more inputs, fast form


def _recipe(m, thresh, rx, ry):
    """The MatchMap recipe of cvmatch_test.go:324-381, in numpy."""
    h, w = m.shape
    out = []
    for y, x in np.argwhere(~(m < thresh)):
        win = m[max(0, y - ry):min(h, y + ry + 1), max(0, x - rx):min(w, x + rx + 1)]
        if not np.any(win > m[y, x]):
            out.append((int(x), int(y)))
    return out


def test_fast_peaks_equal_recipe_on_the_fast_map(fast_form):
    img = scene(47, 180, 260)
    tpl = img[40:60, 100:130].copy()
    m, _, _ = cvm.MatchMap(img, tpl)
    want = _recipe(m, 0.3, 4, 3)
    hits, n = cvm.MatchMapPeaks(img, tpl, 0.3, 4, 3, max_peaks=len(want) + 3)
    assert n == len(want) and hits == want and n > 0


def test_fast_sub_image_strides(fast_form):
    big = scene(53, 300, 420)
    view = big[20:260, 30:400]           # a sub-image: row stride wider than its width
    t = big[120:150, 200:248]            # template as a view too
    m, _, _ = cvm.MatchMap(view, t)
    map_check(m, oracle.ref_match_f64(np.ascontiguousarray(view), np.ascontiguousarray(t), 3, threads=16),
              "sub-image views", ref_map=ref(view, t, 3))
    jy, jx = np.unravel_index(int(np.argmax(m)), m.shape)
    assert (jx, jy) == (170, 100)


def test_fast_template_alpha_varies(fast_form):
    img = scene(59, 200, 280)
    t = img[50:80, 60:100].copy()
    t[::2, ::3, 3] = 7                    # the template's alpha varies: cn = 4
    m, _, _ = cvm.MatchMap(img, t)
    map_check(m, oracle.ref_match_f64(img, t, 4, threads=16), "template alpha varies", ref_map=ref(img, t, 4))


@pytest.mark.parametrize("cn,step", [(2, 2), (4, 4), (3, 4)])
def test_fast_match_u8_channels(fast_form, cn, step):
    rng = np.random.default_rng(61 + cn)
    img = scene(67, 160, 230)[..., :step].copy()
    img[40:90, 60:140] = rng.integers(0, 256, (50, 80, step), dtype=np.uint8)
    t = img[50:80, 70:110].copy()
    _, m = cvm.match_u8(img, t, cn)
    map_check(m, oracle.ref_match_f64(img, t, cn, threads=16), f"match_u8 cn={cn} step={step}", ref_map=ref(img, t, cn))


def test_fast_large_gray_template_mean_subtracted(fast_form):
    """A gray template of 258 x 256 pixels: area * 255 >= 2^24, so the
    zero-mean spectrum is built from T - mean(T) in float instead of the
    exact integers area*T - sum(T)."""
    rng = np.random.default_rng(71)
    img = oracle.rgba_to_gray(scene(73, 420, 560))
    img[100:356, 150:408] = rng.integers(0, 256, (256, 258), dtype=np.uint8)
    t = img[100:356, 150:408].copy()
    assert t.shape[0] * t.shape[1] * 255 >= 1 << 24
    _, m = cvm.match_u8(img, t, 1)
    map_check(m, oracle.ref_match_f64(img, t, 1, threads=16), "258x256 gray template", ref_map=ref(img, t, 1))
    jy, jx = np.unravel_index(int(np.argmax(m)), m.shape)
    assert (jx, jy) == (150, 100)


def test_fast_form_routes_transforms_above_4096_to_the_exact_kernels(fast_form):
    """A 4100-px-wide template needs 8192-point row transforms, beyond the
    fast form's length-specialised kernels: the match runs the exact form's
    kernels instead, so its result is the reference's, bit for bit."""
    img = np.ascontiguousarray(scene(79, 60, 4200))
    tpl = img[11:51, 50:4150].copy()
    t, m = cvm.match_u8(img, tpl, 4)
    want, wmap = oracle.match_u8(img, tpl, 4, threads=16)
    assert t == want and np.array_equal(m.view(np.uint32), wmap.view(np.uint32))
    assert (t[4], t[5]) == (50, 11)
    # a fleet with such a member and an ordinary one: each bucket in its own form
    small = img[5:25, 300:340].copy()
    fleet = cvm.NewFleet(cvm.NewMatcher(tpl), cvm.NewMatcher(small))
    fleet.SetForm(cvm.FORM_FAST)
    got = fleet.FindAll(img)
    ref = oracle.fleet_find_all([tpl, small], img, threads=16)
    assert tuple(got[0]) == ref[0]
    check(got[1], oracle.ref_match_f64(img, small, 4, threads=16), "ordinary bucket beside it")


# ------------------------------------------ plan classes and buckets, fast form


def test_fast_shrunk_last_band_solo_and_fleet(fast_form):
    """A 64x48 template on a 337x292 frame plans 256x128 tiles whose last
    band is shrunk to 64 rows (a second plan class, shrinkDH,
    impl.go:573-582): the one-shot map and the fleet member (its own bucket)
    against FP64."""
    img = scene(83, 292, 337)
    t = img[120:168, 200:264].copy()
    p = oracle.plan(64, 48, 337 - 63, 292 - 47)
    assert oracle.shrink_dh(p, 292 - 47, 48) > 0
    m, _, _ = cvm.MatchMap(img, t)
    m64 = oracle.ref_match_f64(img, t, 3, threads=16)
    map_check(m, m64, "shrunk last band, one-shot", ref_map=ref(img, t, 3))
    small = img[10:30, 20:44].copy()
    fleet = cvm.NewFleet(cvm.NewMatcher(t), cvm.NewMatcher(small))
    fleet.SetForm(cvm.FORM_FAST)
    got = fleet.FindAll(img)
    _, ref_maps = oracle.fleet_find_all([t, small], img, threads=16, want_maps=True)
    check(got[0], m64, "shrunk last band, fleet member", ref_map=ref_maps[0])
    check(got[1], oracle.ref_match_f64(img, small, 3, threads=16), "fleet member in the same bucket",
          ref_map=ref_maps[1])
    assert (got[0].MaxX, got[0].MaxY) == (200, 120)


def test_fast_fleet_several_buckets(fast_form):
    """Wide, tall and square members fall into different buckets (bucketize,
    fleet.go:111-171), each with its own plan and frame spectra."""
    img = scene(89, 260, 400)
    tpls = [img[40:48, 52:352].copy(), img[30:230, 300:308].copy(), img[100:140, 100:140].copy(),
            img[10:26, 10:26].copy()]
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    fleet.SetForm(cvm.FORM_FAST)
    got = fleet.FindAll(img)
    _, ref_maps = oracle.fleet_find_all(tpls, img, threads=16, want_maps=True)
    for i, t in enumerate(tpls):
        check(got[i], oracle.ref_match_f64(img, t, 3, threads=16), f"bucket member {i} {t.shape[1]}x{t.shape[0]}",
              ref_map=ref_maps[i])


@pytest.mark.parametrize("alpha", ["const", "template", "parent"])
def test_fast_device_resident_colour_match(fast_form, alpha):
    """cvm_match_device in the fast form (its template spectrum starts
    beside the statistics launch, all four channels, from sums the row
    kernel takes itself) with constant alpha planes (cn 3) or a template
    or parent alpha plane that varies (cn 4), against FP64."""
    torch = pytest.importorskip("torch")
    L = cvm.lib()
    img = scene(97, 210, 330)
    t = img[60:100, 120:168].copy()
    if alpha == "template":
        t[::3, ::2, 3] = 9
    if alpha == "parent":
        img[5, 7, 3] = 3
    cn = 3 if alpha == "const" else 4
    th, tw = t.shape[:2]
    rw, rh = img.shape[1] - tw + 1, img.shape[0] - th + 1
    d_img, d_tpl = torch.from_numpy(img).cuda(), torch.from_numpy(t).cuda()
    d_map = torch.empty((rh, rw), dtype=torch.float32, device="cuda")
    d_out = torch.zeros(6, dtype=torch.int32, device="cuda")
    for _ in range(2):  # the second call reuses the pooled buffers
        rc = L.cvm_match_device(d_img.data_ptr(), img.strides[0], img.shape[1], img.shape[0], d_tpl.data_ptr(),
                                t.strides[0], tw, th, d_map.data_ptr(), d_out.data_ptr(),
                                torch.cuda.current_stream().cuda_stream)
        assert rc == 0
        torch.cuda.synchronize()
        m = d_map.cpu().numpy()
        map_check(m, oracle.ref_match_f64(img, t, cn, threads=16), f"device-resident, alpha {alpha}",
                  ref_map=ref(img, t, cn))
        jy, jx = np.unravel_index(int(np.argmax(m)), m.shape)
        assert (jx, jy) == (120, 60)


@pytest.mark.parametrize("form", ["fast", "mixed"])
def test_near_flat_windows_vs_fp64(form):
    """A low-contrast frame (200 + a few grey levels of +-1): every window
    is near-flat (its variance, summed over the channels, below one grey
    level squared), so every quotient takes the double-precision path; the
    scores still meet the 1e-4 bar against FP64 and the peak is where the
    template was cut.  1024-wide tiles, so the mixed form runs its
    tensor-core rows here."""
    rng = np.random.default_rng(101)
    img = np.empty((300, 1920, 4), np.uint8)
    img[..., :3] = np.clip(np.rint(200 + rng.standard_normal((300, 1920, 3)) * 0.4), 0, 255)
    img[..., 3] = 255
    t = img[120:152, 400:496].copy()
    assert oracle.plan(96, 32, 1920 - 95, 300 - 31).dft_w == 1024
    prev = cvm.SetForm(cvm.FORM_FAST if form == "fast" else cvm.FORM_MIXED)
    prev_t = cvm.SetAutotune(False)  # newGoPlan's 1024-wide tiles
    try:
        m, _, _ = cvm.MatchMap(img, t)
    finally:
        cvm.SetForm(prev)
        cvm.SetAutotune(prev_t)
    assert cvm.device_status() == 0
    map_check(m, fp64.ref_match_f64(img, t, 3), f"near-flat windows ({form})", ref_map=ref(img, t, 3))
    assert fp64.first_argmax(m) == (400, 120)
