"""Parity of the CUDA path with the oracle, through the C ABI, on a GB300.

The bar is bit identity: the CUDA kernels run the reference's per-element
op sequence, so every score map and extremum must equal the oracle's (and
therefore the reference's) bits.  Size-independent properties cover the
full-size configurations; the reference's semantic tests (cvmatch_test.go,
matcher_test.go, fleet_test.go) are mirrored on synthetic inputs.
"""
import json
import os
import sys
import threading

import numpy as np
import pytest

import cvmatch_gb300 as cvm
import oracle

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402
from synth import image  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def same_tuple(a, b):
    return (np.float32(a[0]).view(np.uint32) == np.float32(b[0]).view(np.uint32) and a[1:3] == b[1:3]
            and np.float32(a[3]).view(np.uint32) == np.float32(b[3]).view(np.uint32) and a[4:6] == b[4:6])


def rgba(seed, h, w, alpha=255):
    a = image(seed, h, w, 4).copy()
    if alpha is not None:
        a[..., 3] = alpha
    return a


# ------------------------------------------------------------ golden pins


def test_case110_reference_hash_on_gpu():
    img, tpl = make_golden.canary110()
    t, res = cvm.match_u8(img, tpl, 1)
    assert hex(oracle.fnv_golden_hash(res, t)) == GOLDEN["reference_pins"]["case110_fnv"]


@pytest.mark.parametrize("idx", range(len(make_golden.SOLO_CASES)))
def test_solo_fixture_bit_exact(idx):
    c = make_golden.SOLO_CASES[idx]
    img, tpl = make_golden.solo_inputs(c)
    t, res = cvm.match_u8(img, tpl, c[5])
    assert make_golden.digest(res, t) == GOLDEN["solo"][idx]["digest"], c[0]


@pytest.mark.parametrize("idx", range(len(make_golden.SOLO_CASES)))
def test_solo_matches_live_oracle(idx):
    c = make_golden.SOLO_CASES[idx]
    img, tpl = make_golden.solo_inputs(c)
    t, res = cvm.match_u8(img, tpl, c[5])
    to, ro = oracle.match_u8(img, tpl, c[5], threads=4)
    assert np.array_equal(bits(res), bits(ro))
    assert same_tuple(t, to)


@pytest.mark.parametrize("idx", range(len(make_golden.FLEET_CASES)))
def test_fleet_fixture_bit_exact(idx):
    c = make_golden.FLEET_CASES[idx]
    parent, tpls = make_golden.fleet_inputs(c)
    ms = [cvm.NewMatcher(t) if c[3] == 4 else cvm.NewGrayMatcher(t) for t in tpls]
    got = cvm.NewFleet(*ms).FindAll(parent)
    want = GOLDEN["fleet"][idx]["results"]
    for g, w in zip(got, want):
        assert same_tuple(tuple(g), tuple(w)), (g, w)


# ------------------------------------------------------ FP64 definition


@pytest.mark.parametrize("shape", [
    (97, 61, 17, 13, 1, 0, 0), (97, 61, 17, 13, 4, 0, 0), (64, 64, 64, 64, 1, 0, 0),
    (50, 40, 1, 1, 4, 0, 0), (300, 200, 31, 29, 1, 7, 3), (40, 300, 33, 257, 1, 0, 0),
    (128, 96, 5, 4, 3, 0, 0)])
def test_against_fp64_definition(shape):
    iw, ih, tw, th, cn, ipad, tpad = shape
    img = image(42 + iw, ih, iw, cn, ipad)
    tpl = image(43 + tw, th, tw, cn, tpad)
    t, res = cvm.match_u8(img, tpl, cn)
    ref = oracle.ref_match_f64(img, tpl, cn)
    assert np.max(np.abs(res.astype(np.float64) - ref)) <= 1e-4
    flat = res.ravel()
    assert t[2] * res.shape[1] + t[1] == int(np.argmin(flat))
    assert t[5] * res.shape[1] + t[4] == int(np.argmax(flat))


# ------------------------------------------------ public API semantics


def test_planted_template_match_and_gray():
    parent = rgba(7, 400, 640)
    sub = parent[77:77 + 48, 123:123 + 64].copy()
    for fn in (cvm.Match, cvm.MatchGray):
        _, _, _, v, x, y = fn(parent, sub)
        assert (x, y) == (123, 77) and v >= 0.999


def test_match_equals_oracle_cn3_bitwise():
    parent = rgba(8, 300, 420)
    sub = parent[40:72, 100:196].copy()
    t = cvm.Match(parent, sub)
    to, _ = oracle.match_u8(parent, sub, 3, want_map=False)
    assert same_tuple(t, to)
    m, w, h = cvm.MatchMap(parent, sub)
    _, mo = oracle.match_u8(parent, sub, 3)
    assert (w, h) == (420 - 96 + 1, 300 - 32 + 1) and np.array_equal(bits(m), bits(mo))


def test_sub_image_input():
    parent = rgba(9, 240, 320)
    region = parent[60:140, 50:130]  # a view with the parent's stride
    _, _, _, v, x, y = cvm.Match(parent, region)
    assert (x, y) == (50, 60) and v >= 0.999


def test_gray_plane_input():
    y = image(11, 150, 200, 1).copy()
    sub = y[20:50, 60:100].copy()
    _, _, _, v, x, yy = cvm.MatchGray(y, sub)
    assert (x, yy) == (60, 20) and v >= 0.999


def test_flat_template():
    parent = np.zeros((100, 100, 4), np.uint8)
    sub = np.zeros((10, 10, 4), np.uint8)
    assert cvm.Match(parent, sub) == (1.0, 0, 0, 1.0, 0, 0)
    m, w, h = cvm.MatchMap(rgba(3, 100, 100), sub)
    assert np.all(m == 1.0)


def test_bad_input_raises():
    with pytest.raises(cvm.CvmatchError, match="bad match arguments"):
        cvm.Match(np.zeros((10, 10, 4), np.uint8), np.zeros((20, 20, 4), np.uint8))


def test_constant_alpha_skip_and_varying_alpha():
    iw, ih, tw, th = 120, 90, 24, 18
    img = rgba(21, ih, iw, None)
    tpl = rgba(22, th, tw, None)
    for a_img, a_tpl in ((200, 55), (0, 255), (128, 128)):
        img[..., 3] = a_img
        tpl[..., 3] = a_tpl
        m, _, _ = cvm.MatchMap(img, tpl)
        _, m3 = oracle.match_u8(img, tpl, 3)
        assert np.array_equal(bits(m), bits(m3))
    img = rgba(23, 80, 100, None)  # varying alpha: full 4 channels
    sub = img[30:46, 40:60].copy()
    m, _, _ = cvm.MatchMap(img, sub)
    _, m4 = oracle.match_u8(img, sub, 4)
    assert np.array_equal(bits(m), bits(m4))
    ref = oracle.ref_match_f64(img, sub, 4)
    assert np.max(np.abs(m - ref)) <= 1e-4
    _, _, _, v, x, y = cvm.Match(img, sub)
    assert (x, y) == (40, 30) and v >= 0.999


def test_alpha_mixed_constancy():
    parent = rgba(92, 90, 120, None)  # varying alpha
    sub = parent[40:58, 60:84].copy()
    sub[..., 3] = 128  # constant template alpha: still the 4-channel path
    m, _, _ = cvm.MatchMap(parent, sub)
    _, m4 = oracle.match_u8(parent, sub, 4)
    assert np.array_equal(bits(m), bits(m4))


@pytest.mark.parametrize("W,pw", [(48, 43), (48, 48), (44, 41), (42, 42)])
def test_parent_alpha_scan_one_pixel(W, pw):
    """alphaConst (cvmatch.go:146-168) of a device-resident parent: one
    alpha byte different anywhere (first row, middle, a row's last pixels
    past the last whole group of four, the very last pixel) switches the
    match to four channels.  Pitches W*4 that are multiples of 16 take the
    vector scan, the others the byte scan."""
    torch = pytest.importorskip("torch")
    L = cvm.lib()
    ph = 37
    base = rgba(77, ph, W, 200)
    tpl = base[9:25, 11:31].copy()
    for where in (None, (0, 1), (ph // 2, pw // 2), (3, pw - 1), (ph - 1, pw - 1)):
        img = base.copy()
        if where is not None:
            img[where[0], where[1], 3] = 201
        view = img[:, :pw]
        d_img = torch.from_numpy(img).cuda()
        d_tpl = torch.from_numpy(tpl).cuda()
        rw, rh = pw - 20 + 1, ph - 16 + 1
        d_map = torch.empty((rh, rw), dtype=torch.float32, device="cuda")
        d_out = torch.zeros(6, dtype=torch.int32, device="cuda")
        rc = L.cvm_match_device(d_img.data_ptr(), W * 4, pw, ph, d_tpl.data_ptr(), tpl.strides[0], 20, 16,
                                d_map.data_ptr(), d_out.data_ptr(), torch.cuda.current_stream().cuda_stream)
        assert rc == 0
        torch.cuda.synchronize()
        _, want = oracle.match_u8(view, tpl, 3 if where is None else 4)
        assert np.array_equal(bits(d_map.cpu().numpy()), bits(want)), where


@pytest.mark.parametrize("pw,ph,pad,gray,alpha_at", [(1024, 600, 0, False, None), (1001, 530, 3, False, None),
                                                     (1501, 700, 0, True, None), (1500, 700, 4, True, None),
                                                     (1024, 600, 0, False, (599, 1023)), (1001, 530, 3, False, (0, 1)),
                                                     (1002, 530, 0, False, (300, 500)), (1600, 700, 0, True, None),
                                                     (1600, 700, 16, True, None)])
def test_pinned_host_frame_ingest(pw, ph, pad, gray, alpha_at):
    """Frames in page-locked host memory (cvm_host_alloc) are read by a
    kernel over the host link; 16-byte, 4-byte and 1-byte row alignments,
    and one differing alpha byte (the 4-channel path), must all give the
    oracle's map bit for bit."""
    import ctypes as C
    L = cvm.lib()
    bpp = 1 if gray else 4
    stride = pw * bpp + pad
    nbytes = stride * ph
    hp = L.cvm_host_alloc(nbytes)
    assert hp
    try:
        buf = np.ctypeslib.as_array((C.c_uint8 * nbytes).from_address(hp)).reshape(ph, stride)
        src = image(31 + pw, ph, pw, bpp)
        if not gray:
            src[..., 3] = 255
            if alpha_at is not None:
                src[alpha_at[0], alpha_at[1], 3] = 254
        buf[:, :pw * bpp] = src.reshape(ph, pw * bpp)
        view = buf[:, :pw * bpp].reshape((ph, pw) if gray else (ph, pw, bpp))
        tpl = np.ascontiguousarray(view[100:140, 200:260])
        rw, rh = pw - 60 + 1, ph - 40 + 1
        got = np.empty((rh, rw), np.float32)
        if gray:
            r = cvm._CResult()
            rc = L.cvm_match_u8(hp, stride, pw, ph, tpl.ctypes.data, tpl.strides[0], 60, 40, 1, 1,
                                got.ctypes.data, C.byref(r))
        else:
            rc = L.cvm_match_map(hp, stride, pw, ph, tpl.ctypes.data, tpl.strides[0], 60, 40, got.ctypes.data)
        assert rc == 0
        _, want = oracle.match_u8(view, tpl, 1 if gray else (3 if alpha_at is None else 4))
        assert np.array_equal(bits(got), bits(want))
    finally:
        L.cvm_host_free(hp)


def test_pinned_fused_ingest_template_cases():
    """A page-locked frame with 16-byte rows takes the fused ingest (the
    template's parameters derived on the host, the frame's alpha scan done
    by the copy, the parameters the scan selects stored by its last CTA).
    Consecutive calls alternate the outcomes: a template whose alpha varies
    over a constant frame (cn 4), a constant template alpha other than the
    frame's (cn 3), the frame's alpha varying (cn 4), flat templates (the
    flat result), each equal to the oracle bit for bit."""
    import ctypes as C
    L = cvm.lib()
    pw, ph = 1024, 600
    nbytes = pw * 4 * ph
    hp = L.cvm_host_alloc(nbytes)
    assert hp
    try:
        buf = np.ctypeslib.as_array((C.c_uint8 * nbytes).from_address(hp)).reshape(ph, pw, 4)
        base = np.ascontiguousarray(image(77 + pw, ph, pw, 4)).copy()
        base[..., 3] = 255
        t_var = np.ascontiguousarray(base[100:140, 200:260]).copy()
        t_var[5, 7, 3] = 3
        t_const = np.ascontiguousarray(base[300:340, 500:560]).copy()
        t_const[..., 3] = 7
        t_flat = np.zeros((40, 60, 4), np.uint8)
        t_flat[..., :3] = 90
        t_flat[..., 3] = 255
        t_zero = np.zeros((40, 60, 4), np.uint8)
        cases = [(t_var, None, 4), (t_const, None, 3), (t_const, (599, 1023), 4), (t_flat, None, 3),
                 (t_var, None, 4), (t_zero, (10, 10), 4), (t_const, None, 3)]
        for tpl, alpha_at, cn in cases:
            buf[:] = base
            if alpha_at is not None:
                buf[alpha_at[0], alpha_at[1], 3] = 254
            got = np.empty((ph - 40 + 1, pw - 60 + 1), np.float32)
            rc = L.cvm_match_map(hp, pw * 4, pw, ph, tpl.ctypes.data, tpl.strides[0], 60, 40, got.ctypes.data)
            assert rc == 0
            r = cvm._CResult()
            rc = L.cvm_match(hp, pw * 4, pw, ph, tpl.ctypes.data, tpl.strides[0], 60, 40, C.byref(r))
            assert rc == 0
            want_t, want = oracle.match_u8(buf, tpl, cn)
            assert np.array_equal(bits(got), bits(want)), (cn, alpha_at)
            assert same_tuple(r.tuple(), want_t), (cn, alpha_at, r.tuple(), want_t)
    finally:
        L.cvm_host_free(hp)


def test_find_all_occurrences_via_map():
    rng = np.random.default_rng(101)
    parent = np.empty((300, 400, 4), np.uint8)
    parent[..., :3] = rng.integers(0, 64, (300, 400, 3))
    parent[..., 3] = 255
    tpl = rgba(102, 24, 32)
    spots = [(10, 12), (200, 40), (350, 260), (60, 240), (180, 150)]
    for x, y in spots:
        parent[y:y + 24, x:x + 32] = tpl
    resp, w, h = cvm.MatchMap(parent, tpl)
    hits = []
    for y in range(h):
        for x in np.nonzero(resp[y] >= 0.999)[0]:
            nb = resp[max(0, y - 12):y + 13, max(0, x - 16):x + 17]
            if not np.any(nb > resp[y, x]):
                hits.append((int(x), y))
    assert sorted(hits) == sorted(spots)


def test_gray_conversion_and_alpha_scan():
    for w, h, pad in ((1, 1, 0), (7, 3, 0), (33, 5, 2), (641, 2, 3)):
        pix = image(8 + w, h, w, 4, pad)
        got = cvm.rgba_to_gray(pix)
        p = pix.astype(np.uint32)
        want = ((4899 * p[..., 0] + 9617 * p[..., 1] + 1868 * p[..., 2] + 8192) >> 14).astype(np.uint8)
        assert np.array_equal(got, want)
    a = rgba(5, 50, 70)
    assert cvm.alpha_const(a)
    a[49, 69, 3] = 3
    assert not cvm.alpha_const(a)


# -------------------------------------------------------------- Matcher


def test_matcher_find_equals_match():
    parent = rgba(31, 240, 320)
    sub = parent[80:104, 100:132].copy()
    want = cvm.Match(parent, sub)
    m = cvm.NewMatcher(sub)
    for _ in range(3):
        assert same_tuple(m.Find(parent), want)
    g = cvm.NewGrayMatcher(sub)
    wantg = cvm.MatchGray(parent, sub)
    for _ in range(3):
        assert same_tuple(g.Find(parent), wantg)


def test_matcher_geometry_change():
    full = rgba(33, 400, 560)
    sub = full[100:196, 200:296].copy()
    crop = full[:400 - 24, :560 - 40]
    m = cvm.NewMatcher(sub)
    for _ in range(2):
        for parent in (full, crop):
            assert same_tuple(m.Find(parent), cvm.Match(parent, sub))


def test_matcher_concurrent():
    parent = rgba(35, 300, 400, None)
    sub = parent[10:50, 20:70].copy()
    want = cvm.Match(parent, sub)
    m = cvm.NewMatcher(sub)
    out = [None] * 8

    def work(i):
        out[i] = m.Find(parent)

    ts = [threading.Thread(target=work, args=(i,)) for i in range(8)]
    [t.start() for t in ts]
    [t.join() for t in ts]
    assert all(same_tuple(o, want) for o in out)


def test_concurrent_match_calls():
    parent = rgba(31, 240, 320)
    sub = parent[80:104, 100:132].copy()
    want, wantg = cvm.Match(parent, sub), cvm.MatchGray(parent, sub)
    errs = []

    def work():
        for _ in range(5):
            if not same_tuple(cvm.Match(parent, sub), want) or not same_tuple(cvm.MatchGray(parent, sub), wantg):
                errs.append(1)

    ts = [threading.Thread(target=work) for _ in range(8)]
    [t.start() for t in ts]
    [t.join() for t in ts]
    assert not errs


# ---------------------------------------------------------------- Fleet


def desk(seed=41):
    rng = np.random.default_rng(seed)
    img = np.empty((700, 1000, 4), np.uint8)
    img[..., :3] = rng.integers(0, 256, (700, 1000, 3))
    img[..., 3] = 255
    for _ in range(30):
        w, h = rng.integers(20, 300, 2)
        x, y = rng.integers(0, 1000 - w), rng.integers(0, 700 - h)
        img[y:y + h, x:x + w, :3] = rng.integers(0, 256, 3)
    return img


def crops(img, seed=11, n=12):
    rng = np.random.default_rng(seed)
    sizes = [(24, 24), (96, 32), (48, 48), (300, 200), (16, 16), (64, 128)]
    out, at = [], []
    for i in range(n):
        w, h = sizes[i % len(sizes)]
        x, y = int(rng.integers(0, img.shape[1] - w)), int(rng.integers(0, img.shape[0] - h))
        out.append(img[y:y + h, x:x + w].copy())
        at.append((x, y))
    return out, at


@pytest.mark.parametrize("gray", [False, True])
def test_fleet_bit_exact_vs_oracle(gray):
    img = desk()
    subs, at = crops(img)
    ms = [cvm.NewGrayMatcher(s) if gray else cvm.NewMatcher(s) for s in subs]
    got = cvm.NewFleet(*ms).FindAll(img)
    if gray:
        gimg = oracle.rgba_to_gray(img)
        want = oracle.fleet_find_all([oracle.rgba_to_gray(s) for s in subs], gimg, threads=8)
    else:
        want = oracle.fleet_find_all(subs, img, threads=8)
    for g, w in zip(got, want):
        assert same_tuple(tuple(g), w)
    hits = sum((g.MaxX, g.MaxY) == a for g, a in zip(got, at))
    assert hits >= len(got) * 2 // 3


@pytest.mark.parametrize("form", ["exact", "fast"])
def test_fleet_agrees_with_solo_matches(form):
    """fleet_test.go:50-88: every member of a multi-member fleet (run on its
    bucket's plan) agrees with a one-shot Match of the same template (run on
    its own plan) within 1e-3, at the same extremum locations on clear
    matches; in the exact form the plans differ only in rounding, in the
    fast form both sides are within 1e-4 of the FP64 definition."""
    img = desk(49)
    subs, at = crops(img, seed=13, n=12)
    prev = cvm.SetForm(cvm.FORM_FAST if form == "fast" else cvm.FORM_EXACT)
    try:
        fleet = cvm.NewFleet(*[cvm.NewMatcher(s) for s in subs])
        if form == "fast":
            fleet.SetForm(cvm.FORM_FAST)
        got = fleet.FindAll(img)
        solo = [cvm.Match(img, s) for s in subs]
    finally:
        cvm.SetForm(prev)
    assert len(got) == len(subs)
    for i, (g, s) in enumerate(zip(got, solo)):
        g, s = tuple(g), tuple(s)
        if subs[i][..., :3].reshape(-1, 3).std(axis=0).max() == 0:  # flat: the fixed answer
            assert g == s == (1.0, 0, 0, 1.0, 0, 0), (i, g, s)
            continue
        assert abs(g[0] - s[0]) <= 1e-3 and abs(g[3] - s[3]) <= 1e-3, (i, g, s)
        assert s[3] > 0.999 and g[4:6] == s[4:6] == at[i], (i, g, s, at[i])  # the planted copy


def test_fleet_single_member_equals_find():
    img = desk(43)
    sub = img[100:132, 200:296].copy()
    m = cvm.NewMatcher(sub)
    (r,) = cvm.NewFleet(m).FindAll(img)
    assert same_tuple(tuple(r), m.Find(img))


def test_fleet_flat_members_and_all_flat():
    img = desk(45)
    subs, _ = crops(img, n=3)
    flat = np.zeros((300, 400, 4), np.uint8)
    flat[..., :3] = 30
    flat[..., 3] = 255
    ms = [cvm.NewMatcher(flat), cvm.NewMatcher(subs[0]), cvm.NewMatcher(subs[1])]
    got = cvm.NewFleet(*ms).FindAll(img)
    assert tuple(got[0]) == (1.0, 0, 0, 1.0, 0, 0)
    for i in (1, 2):
        assert (got[i].MaxX, got[i].MaxY) == ms[i].Find(img)[4:6]
    assert tuple(cvm.NewFleet(cvm.NewMatcher(flat)).FindAll(img)[0]) == (1.0, 0, 0, 1.0, 0, 0)


def test_fleet_mixed_alpha_and_orthogonal():
    img = desk(47)
    subs, at = crops(img, n=3)
    va = subs[0].copy()
    va.reshape(-1, 4)[::4, 3] = np.arange(va.reshape(-1, 4)[::4].shape[0]) % 256
    wide = img[40:48, 52:352].copy()
    tall = img[150:450, 700:708].copy()
    tpls = [va, subs[1], subs[2], wide, tall]
    got = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls]).FindAll(img)
    want = oracle.fleet_find_all(tpls, img, threads=8)
    for g, w in zip(got, want):
        assert same_tuple(tuple(g), w)


def test_fleet_determinism_order_repeat_isolation():
    img = desk(49)
    subs, _ = crops(img)
    ms = [cvm.NewGrayMatcher(s) for s in subs]
    base = cvm.NewFleet(*ms).FindAll(img)
    rev = cvm.NewFleet(*ms[::-1]).FindAll(img)
    assert [tuple(r) for r in rev[::-1]] == [tuple(b) for b in base]
    fl = cvm.NewFleet(ms)
    assert fl.FindAll(img) == fl.FindAll(img) == base
    lst = [ms[0], ms[1]]
    f2 = cvm.NewFleet(lst)
    want = f2.FindAll(img)
    lst[0] = ms[3]
    assert f2.FindAll(img) == want


def test_fleet_concurrent():
    img = desk(51)
    subs, _ = crops(img, n=6)
    fl = cvm.NewFleet(*[cvm.NewMatcher(s) for s in subs])
    out = [None] * 4

    def work(i):
        out[i] = fl.FindAll(img)

    ts = [threading.Thread(target=work, args=(i,)) for i in range(4)]
    [t.start() for t in ts]
    [t.join() for t in ts]
    assert all(o == out[0] for o in out)


def test_fleet_mixed_modes_rejected():
    a = rgba(1, 20, 20)
    with pytest.raises(cvm.CvmatchError, match="fleet mixes color and gray matchers"):
        cvm.NewFleet(cvm.NewMatcher(a), cvm.NewGrayMatcher(a))


# ------------------------------------------------- benchmark-sized configs


def test_gray_640x480_bit_exact():
    import bench
    frame, tpl, (x, y) = bench.scene_gray_640x480()
    t = cvm.MatchGray(frame, tpl)
    g, gt = oracle.rgba_to_gray(frame), oracle.rgba_to_gray(tpl)
    to, _ = oracle.match_u8(g, gt, 1, threads=8, want_map=False)
    assert same_tuple(t, to) and (t[4], t[5]) == (x, y)


def test_rgba_1920x1080_bit_exact():
    import bench
    frame, tpl, (x, y) = bench.scene_ui_1920x1080()
    m, w, h = cvm.MatchMap(frame, tpl)
    to, mo = oracle.match_u8(frame, tpl, 3, threads=16)
    assert np.array_equal(bits(m), bits(mo))
    t = cvm.Match(frame, tpl)
    assert same_tuple(t, to)
    assert (t[4], t[5]) == (x, y)


def test_gray_3840x2160_map_bit_exact():
    import bench
    g, tpl, (x, y) = bench.scene_gray_3840x2160()
    t, m = cvm.match_u8(g, tpl, 1)
    to, mo = oracle.match_u8(g, tpl, 1, threads=16)
    assert np.array_equal(bits(m), bits(mo)) and same_tuple(t, to)
    assert (t[4], t[5]) == (x, y)
    assert np.all(np.abs(m) <= 1.0)


# ---------------------------------------------------- rare arithmetic paths


def test_lanes_above_2_53_gray():
    """area*s2 exceeds 2^53: float32(float64(v)) rounds twice; the GPU's
    integer emulation of the first rounding must give the same bits."""
    img = image(601, 1100, 1100, 1).copy()
    img[:] = 160 + (img % 96)
    tpl = img[37:1037, 41:1041].copy()
    t, m = cvm.match_u8(img, tpl, 1)
    to, mo = oracle.match_u8(img, tpl, 1, threads=16)
    assert np.array_equal(bits(m), bits(mo)) and same_tuple(t, to)


def test_lanes_above_2_53_colour():
    img = image(602, 520, 720, 4).copy()
    img[:] = 200 + (img % 56)
    tpl = img[10:510, 12:712].copy()
    t, m = cvm.match_u8(img, tpl, 4)
    to, mo = oracle.match_u8(img, tpl, 4, threads=16)
    assert np.array_equal(bits(m), bits(mo)) and same_tuple(t, to)


def test_very_wide_colour_template_global_column_arrays():
    """A 4100-px-wide RGBA template: the normalisation's column arrays no
    longer fit shared memory and live in global scratch."""
    img = image(603, 60, 4200, 4).copy()
    tpl = img[11:51, 50:4150].copy()
    t, m = cvm.match_u8(img, tpl, 4)
    to, mo = oracle.match_u8(img, tpl, 4, threads=16)
    assert np.array_equal(bits(m), bits(mo)) and same_tuple(t, to)
    assert (t[4], t[5]) == (50, 11)


def test_fleet_block_sums_and_a_member_too_wide_for_them():
    """A fleet's vertical slides start from 16-row block sums of the shared
    row prefix (u32).  Sixteen rows of a colour member's squared window sum
    stay below 2^32 only for templates narrower than ~1376 px, so a fleet
    holding a 1400-px member starts every slide row by row: both kinds of
    fleet bit-exact against the oracle, and the fast form within 1e-4 of
    FP64 on the wide fleet."""
    from oracle import fp64
    img = rgba(91, 150, 1500)
    small = [img[20:60, 100:164].copy(), img[70:102, 900:940].copy(), img[5:125, 300:348].copy()]
    wide = small + [img[10:90, 40:1440].copy()]
    for tpls in (small, wide):
        fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
        got = [tuple(r) for r in fleet.FindAll(img)]
        want = oracle.fleet_find_all(tpls, img, threads=16)
        assert all(same_tuple(g, w) for g, w in zip(got, want)), (len(tpls), got, want)
    fleet.SetForm(cvm.FORM_FAST)
    fast = fleet.FindAll(img)
    F = fp64.Frame(img, 3)
    for i, t in enumerate(wide):
        fp64.check_extrema(tuple(fast[i]), F.match(t), 1e-4, name=f"member {i}")


def test_very_wide_tall_gray_template_without_block_sums():
    """A 4200 x 64 gray template: sixteen rows of its squared window sums
    can exceed 2^32, so the vertical slide starts row by row instead of
    from 16-row block sums; bit-exact against the oracle."""
    g = image(607, 110, 4300, 1).copy()
    tpl = g[30:94, 60:4260].copy()
    t, m = cvm.match_u8(g, tpl, 1)
    to, mo = oracle.match_u8(g, tpl, 1, threads=16)
    assert np.array_equal(bits(m), bits(mo)) and same_tuple(t, to)
    assert (t[4], t[5]) == (60, 30)


# ------------------------------------------------------------ frame streams


def test_stream_equals_find_all_per_frame():
    """A frame stream (colour fleet + gray fleet on the gray conversion,
    replayed as a CUDA graph, two frames in flight) gives exactly the
    results of Fleet.FindAll on each frame."""
    rng = np.random.default_rng(55)
    H, W = 300, 420
    frames = []
    base = rgba(61, H, W)
    for i in range(5):
        f = base.copy()
        y, x = int(rng.integers(0, H - 40)), int(rng.integers(0, W - 60))
        f[y:y + 40, x:x + 60, :3] = rng.integers(0, 256, (40, 60, 3), dtype=np.uint8)
        frames.append(f)
    tc = [base[10:34, 20:60].copy(), base[100:150, 200:230].copy(), rgba(62, 24, 24), base[200:296, 300:400].copy()]
    tg = [cvm.rgba_to_gray(base[50:80, 50:90]), cvm.rgba_to_gray(base[150:180, 250:310])]
    cf = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tc])
    gf = cvm.NewFleet(*[cvm.NewGrayMatcher(t) for t in tg])
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
        want_c = cf.FindAll(f)
        want_g = gf.FindAll(cvm.rgba_to_gray(f))
        assert [tuple(r) for r in rc] == [tuple(r) for r in want_c]
        assert [tuple(r) for r in rg] == [tuple(r) for r in want_g]
        assert ms > 0


# ------------------------------------------------------- every occurrence


def _recipe(m, thresh, rx, ry):
    """The MatchMap recipe of cvmatch_test.go:324-381, in numpy."""
    h, w = m.shape
    out = []
    for y, x in np.argwhere(~(m < thresh)):
        win = m[max(0, y - ry):min(h, y + ry + 1), max(0, x - rx):min(w, x + rx + 1)]
        if not np.any(win > m[y, x]):
            out.append((int(x), int(y)))
    return out


def test_find_all_occurrences_on_device():
    """TestFindAllOccurrences (cvmatch_test.go:324-381) with the recipe run
    on the device: the five planted copies, nothing else, raster order."""
    rng = np.random.default_rng(101)
    parent = np.empty((300, 400, 4), np.uint8)
    parent[..., :3] = rng.integers(0, 64, (300, 400, 3))
    parent[..., 3] = 255
    tpl = rgba(102, 24, 32)
    spots = [(10, 12), (200, 40), (350, 260), (60, 240), (180, 150)]
    for x, y in spots:
        parent[y:y + 24, x:x + 32] = tpl
    hits, n = cvm.MatchMapPeaks(parent, tpl, 0.999, 16, 12)
    assert n == 5
    assert hits == sorted(spots, key=lambda p: (p[1], p[0]))


@pytest.mark.parametrize("thresh,rx,ry", [(0.2, 3, 2), (0.0, 1, 1), (0.5, 16, 12)])
def test_occurrences_equal_recipe_and_truncate_in_raster_order(thresh, rx, ry):
    img = rgba(71, 180, 260)
    tpl = img[40:60, 100:130].copy()
    m, _, _ = cvm.MatchMap(img, tpl)
    want = _recipe(m, thresh, rx, ry)
    hits, n = cvm.MatchMapPeaks(img, tpl, thresh, rx, ry, max_peaks=len(want) + 5)
    assert n == len(want) and hits == want
    k = max(1, len(want) // 3)
    hits, n = cvm.MatchMapPeaks(img, tpl, thresh, rx, ry, max_peaks=k)
    assert n == len(want) and hits == want[:k]


def test_peaks_device_on_a_device_map():
    torch = pytest.importorskip("torch")
    L = cvm.lib()
    rng = np.random.default_rng(9)
    m = rng.random((70, 300)).astype(np.float32)
    m[5, 7] = 2.0
    d = torch.from_numpy(m).cuda()
    xy = torch.zeros(2 * 64, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.cvm_peaks_device(d.data_ptr(), 300, 70, 0.9, 4, 3, xy.data_ptr(), 64, cnt.data_ptr(),
                              torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    want = _recipe(m, 0.9, 4, 3)
    n = int(cnt.item())
    assert n == len(want)
    got = [tuple(int(v) for v in p) for p in xy.cpu().numpy().reshape(-1, 2)[:min(n, 64)]]
    assert got == want[:64]


# ----------------------------------------------------- regions of interest


def _roi_expect(res, m, roi, tw, th):
    """First-occurrence extrema of a member's FindAll map over the positions
    whose window lies inside roi = (x, y, w, h), in frame coordinates."""
    x, y, w, h = roi
    rh, rw = m.shape if m is not None else (None, None)
    if m is None:  # flat member: 1 everywhere
        return None
    x0, y0 = max(x, 0), max(y, 0)
    x1, y1 = min(x + w - tw + 1, rw), min(y + h - th + 1, rh)
    if x1 <= x0 or y1 <= y0:
        return "empty"
    sub = m[y0:y1, x0:x1]
    iy, ix = np.unravel_index(int(np.argmin(sub)), sub.shape)
    jy, jx = np.unravel_index(int(np.argmax(sub)), sub.shape)
    return (float(sub[iy, ix]), x0 + int(ix), y0 + int(iy), float(sub[jy, jx]), x0 + int(jx), y0 + int(jy))


def test_fleet_roi_members_equal_restricted_maps():
    parent = rgba(81, 240, 360)
    tpls = [parent[30:54, 40:72].copy(), parent[150:190, 200:250].copy(), rgba(82, 30, 40),
            parent[100:120, 300:340].copy(), np.full((16, 16, 4), 90, np.uint8)]
    tpls[4][..., 3] = 255
    rois = {0: (20, 10, 120, 90), 1: (0, 0, 150, 120), 2: (5, 5, 20, 20), 4: (60, 70, 50, 40)}
    res, maps = oracle.fleet_find_all(tpls, parent, want_maps=True)
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    for i, r in rois.items():
        fleet.SetROI(i, *r)
    got = fleet.FindAll(parent)
    for i, t in enumerate(tpls):
        th, tw = t.shape[:2]
        if i not in rois:
            assert same_tuple(tuple(got[i]), res[i])
            continue
        want = _roi_expect(res[i], maps[i], rois[i], tw, th)
        if want == "empty":
            assert np.isnan(got[i][0]) and np.isnan(got[i][3]) and tuple(got[i])[1:3] == (-1, -1)
        elif want is None:  # flat with an ROI: its first position
            x, y = rois[i][0], rois[i][1]
            assert tuple(got[i]) == (1.0, x, y, 1.0, x, y)
        else:
            assert same_tuple(tuple(got[i]), want), (i, tuple(got[i]), want)
    # clearing the regions restores FindAll's results
    for i in rois:
        fleet.SetROI(i, 0, 0, 0, 0)
    again = fleet.FindAll(parent)
    for i in range(len(tpls)):
        assert same_tuple(tuple(again[i]), res[i])


# ------------------------------------------- frames of 2^20 pixels or more
# One-shot matches on frames this large (statistics not queued late) run the
# frame's row transform beside k_prep and the alpha plane's transform in a
# second launch that only does work when the alpha scans choose four
# channels; the bar stays bit identity with the oracle.

def test_large_frame_constant_alpha_bit_exact():
    img = rgba(61, 1024, 1024)  # 2^20 pixels, alpha 255: cn = 3
    sub = img[300:330, 500:540].copy()
    m, _, _ = cvm.MatchMap(img, sub)
    t = cvm.Match(img, sub)
    to, mo = oracle.match_u8(img, sub, 3, threads=16)
    assert np.array_equal(bits(m), bits(mo))
    assert same_tuple(t, to) and (t[4], t[5]) == (500, 300)


def test_large_frame_varying_alpha_bit_exact():
    img = rgba(62, 1024, 1024, None)  # varying alpha: the fourth channel's launch transforms it
    sub = img[600:628, 100:136].copy()
    m, _, _ = cvm.MatchMap(img, sub)
    t = cvm.Match(img, sub)
    to, mo = oracle.match_u8(img, sub, 4, threads=16)
    assert np.array_equal(bits(m), bits(mo))
    assert same_tuple(t, to) and (t[4], t[5]) == (100, 600)


def test_large_gray_frame_tall_template_bit_exact():
    g = np.ascontiguousarray(image(63, 1000, 1100, 4)[..., 1])  # 1.1 Mpx; 70 rows: block sums too
    sub = g[400:470, 700:770].copy()
    t, m = cvm.match_u8(g, sub, 1)
    to, mo = oracle.match_u8(g, sub, 1, threads=16)
    assert np.array_equal(bits(m), bits(mo))
    assert same_tuple(t, to) and same_tuple(cvm.MatchGray(g, sub), to) and (t[4], t[5]) == (700, 400)


def test_large_frame_fast_form_tall_template_vs_fp64():
    # fast form, a 66-row colour template: statistics above the caller's
    # priority, the frame's rows beside k_prep; within 1e-4 of the FP64
    # definition of the score (cvmatch_test.go:118)
    img = rgba(61, 1024, 1024)
    sub = img[200:266, 300:324].copy()
    prev = cvm.SetForm(cvm.FORM_FAST)
    try:
        m, _, _ = cvm.MatchMap(img, sub)
        t = cvm.Match(img, sub)
    finally:
        cvm.SetForm(prev)
    m64 = oracle.ref_match_f64(img, sub, 3, threads=16)
    assert float(np.abs(m.astype(np.float64) - m64).max()) <= 1e-4
    assert (t[4], t[5]) == (300, 200) and t[3] >= 0.999


@pytest.mark.parametrize("alpha", ["const", "parent"])
def test_large_device_resident_match_bit_exact(alpha):
    """cvm_match_device (the frame already on the device: the template
    spectrum starts at once, the frame's rows beside k_prep) on 2^20
    pixels, bit for bit against the oracle with cn 3 and cn 4."""
    torch = pytest.importorskip("torch")
    L = cvm.lib()
    img = rgba(64, 1024, 1024)
    if alpha == "parent":
        img[517, 3, 3] = 7
    t = img[400:432, 256:304].copy()
    cn = 3 if alpha == "const" else 4
    th, tw = t.shape[:2]
    rw, rh = img.shape[1] - tw + 1, img.shape[0] - th + 1
    d_img, d_tpl = torch.from_numpy(img).cuda(), torch.from_numpy(t).cuda()
    d_map = torch.empty((rh, rw), dtype=torch.float32, device="cuda")
    d_out = torch.zeros(6, dtype=torch.int32, device="cuda")
    to, mo = oracle.match_u8(img, t, cn, threads=16)
    for _ in range(2):  # the second call reuses the pooled buffers
        rc = L.cvm_match_device(d_img.data_ptr(), img.strides[0], img.shape[1], img.shape[0], d_tpl.data_ptr(),
                                t.strides[0], tw, th, d_map.data_ptr(), d_out.data_ptr(),
                                torch.cuda.current_stream().cuda_stream)
        assert rc == 0
        torch.cuda.synchronize()
        assert np.array_equal(bits(d_map.cpu().numpy()), bits(mo))
        o = d_out.cpu().numpy()
        f = o.view(np.float32)
        got = (float(f[0]), int(o[1]), int(o[2]), float(f[3]), int(o[4]), int(o[5]))
        assert same_tuple(got, to) and (got[4], got[5]) == (256, 400)
