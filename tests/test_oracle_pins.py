"""Pins the CPU oracle to the reference before it is trusted as the checker.

Every pin here is one the reference's own test-suite holds for this path
and that reproduces without Go:
  - golden case 110's recorded output hash (impl_golden_test.go:75-87,
    golden_hashes_test.go:21), threads 1 and 4;
  - the 15 planner pins (plan_test.go:12-28);
  - the exact-statistics caps (statscap_test.go:16-35);
  - the bucketing pins (fleet_internal_test.go:27-51);
  - the FFT engine's accuracy and round trip (radix4_test.go:40-81) and the
    column engine's bit identity with the row engine (radix4cols_test.go:16-68);
  - <= 1e-4 against the FP64 definition on the reference's seven shapes
    (cvmatch_test.go:91-139) and the semantic tests around alpha.
The reference's other golden cases draw inputs from Go's math/rand, whose
generator table is not part of the reference tree; those are unpinned.
"""
import json
import os
import sys

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402
from synth import image  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))


@pytest.mark.parametrize("threads", [1, 4])
def test_golden_case_110_reference_hash(threads):
    img, tpl = make_golden.canary110()
    t, res = oracle.match_u8(img, tpl, 1, threads=threads)
    assert hex(oracle.fnv_golden_hash(res, t)) == GOLDEN["reference_pins"]["case110_fnv"]


PLAN_PINS = [
    (128, 128, 1793, 953, 1024, 512, 897, 385),
    (96, 32, 1505, 969, 512, 1024, 417, 969),
    (32, 32, 1889, 1049, 512, 256, 481, 225),
    (256, 256, 3585, 1905, 2048, 1024, 1793, 769),
    (24, 24, 1577, 977, 256, 512, 233, 489),
    (80, 80, 433, 401, 512, 512, 433, 401),
    (64, 64, 449, 449, 512, 512, 449, 449),
    (100, 100, 769, 501, 512, 256, 413, 157),
    (128, 128, 625, 473, 512, 512, 385, 385),
    (64, 64, 1, 1, 64, 64, 1, 1),
    (1, 1, 50, 40, 4, 2, 4, 2),
    (33, 257, 8, 44, 64, 512, 8, 44),
    (17, 13, 81, 49, 64, 64, 48, 49),
    (1, 400, 2000, 1, 32, 512, 32, 1),
    (400, 1, 1, 2000, 512, 2, 1, 2),
]


@pytest.mark.parametrize("pin", PLAN_PINS)
def test_plan_pins(pin):
    p = oracle.plan(*pin[:4])
    assert (p.dft_w, p.dft_h, p.block_w, p.block_h) == pin[4:]


def test_stats_caps():
    limit = (1 << 63) - 1
    for cn in range(1, 5):
        a = oracle.stats_cap(cn)
        v = cn * 65025
        assert a * a <= limit // v
        assert (a + 1) * (a + 1) > limit // v
    assert 3000 * 2000 <= oracle.stats_cap(1)
    big = np.zeros((2500, 2500, 4), np.uint8)
    with pytest.raises(oracle.OraclePanic, match="exceeds the exact-statistics bound for cn=4"):
        oracle.match_u8(big, big, 4)


def _mk(w, h, flat):
    i = np.arange(w * h * 4, dtype=np.int64)
    pix = np.full(w * h * 4, 100, np.int64) if flat else (i * 13 + i // 7)
    pix = (pix & 0xFF).astype(np.uint8).reshape(h, w, 4)
    pix[..., 3] = 255
    return pix


def test_bucketize_pins():
    wide, tall = _mk(300, 8, False), _mk(8, 300, False)
    small, mid = _mk(24, 24, False), _mk(200, 100, False)
    flat = _mk(400, 300, True)
    bs = oracle.bucketize([wide, tall])
    assert len(bs) == 2
    for tw, th, _ in bs:
        assert tw <= 300 and th <= 300 and not (tw == 300 and th == 300)
    assert oracle.bucketize([mid, small]) == [(200, 100, [0, 1])]
    assert oracle.bucketize([flat, small]) == [(24, 24, [1])]


def _randslab(n, seed):
    rng = np.random.default_rng(seed)
    return (rng.random(n, np.float32) * 2 - 1 + 1j * (rng.random(n, np.float32) * 2 - 1)).astype(np.complex64)


def test_fft_r4_matches_dft():
    n = 1
    while n <= 4096:
        for inverse in (False, True):
            x = _randslab(n, n + 7)
            got = oracle.fft_r4(x, inverse)
            want = np.fft.ifft(x.astype(np.complex128)) * n if inverse else np.fft.fft(x.astype(np.complex128))
            norm = np.sum(np.abs(want) ** 2)
            tol = 3e-7 * np.sqrt(norm) * np.sqrt(np.log2(n) + 1) * 4
            assert np.max(np.abs(got.astype(np.complex128) - want)) <= tol
        n *= 2


def test_fft_r4_round_trip():
    for n in (2, 4, 8, 64, 512, 1024):
        x = _randslab(n, n + 3)
        a = oracle.fft_r4(oracle.fft_r4(x, False), True)
        a = (a.real.astype(np.float32) * np.float32(1 / n)) + 1j * (a.imag.astype(np.float32) * np.float32(1 / n))
        assert np.max(np.abs(a - x)) <= 2e-5


def _brev(n):
    bits = int(np.log2(n))
    return np.array([int(format(i, f"0{bits}b")[::-1], 2) if bits else 0 for i in range(n)])


@pytest.mark.parametrize("n", [2, 4, 8, 16, 64, 128, 512])
def test_cols_match_row_engine_bitwise(n):
    br = _brev(n)
    for width in (1, 7, 8, 24, 33):
        src = _randslab(n * width, n * width).reshape(n, width)
        for inverse in (False, True):
            want = np.stack([oracle.fft_r4(src[:, c], inverse) for c in range(width)], axis=1)
            placed = np.empty_like(src)
            placed[br] = src
            got = oracle.cols_r4(placed, inverse, False)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
            got2 = oracle.cols_r4(src, inverse, True)
            assert np.array_equal(got2[br].view(np.uint32), want.view(np.uint32))


REF_SHAPES = [
    (97, 61, 17, 13, 1, 0, 0), (97, 61, 17, 13, 4, 0, 0), (64, 64, 64, 64, 1, 0, 0),
    (50, 40, 1, 1, 4, 0, 0), (300, 200, 31, 29, 1, 7, 3), (40, 300, 33, 257, 1, 0, 0),
    (128, 96, 5, 4, 3, 0, 0),
]


@pytest.mark.parametrize("shape", REF_SHAPES)
def test_against_fp64_definition(shape):
    iw, ih, tw, th, cn, ipad, tpad = shape
    img = image(42 + iw, ih, iw, cn, ipad)
    tpl = image(43 + tw, th, tw, cn, tpad)
    t, res = oracle.match_u8(img, tpl, cn, threads=4)
    ref = oracle.ref_match_f64(img, tpl, cn)
    assert np.max(np.abs(res.astype(np.float64) - ref)) <= 1e-4
    flat = res.ravel()
    # first-occurrence scan over our own values (cvmatch_test.go:121-137)
    assert t[0] == flat.min() and t[3] == flat.max()
    assert t[2] * res.shape[1] + t[1] == int(np.argmin(flat))
    assert t[5] * res.shape[1] + t[4] == int(np.argmax(flat))


def test_constant_alpha_skip():
    iw, ih, tw, th = 120, 90, 24, 18
    img = image(21, ih, iw, 4).copy()
    tpl = image(22, th, tw, 4).copy()
    for a_img, a_tpl in ((200, 55), (0, 255), (255, 0), (128, 128)):
        img[..., 3] = a_img
        tpl[..., 3] = a_tpl
        _, m3 = oracle.match_u8(img, tpl, 3)
        _, m4 = oracle.match_u8(img, tpl, 4)
        assert np.max(np.abs(m3 - m4)) <= 1e-5


def test_alpha_matters():
    img = image(91, 120, 160, 4)
    tpl = image(92, 24, 32, 4)
    _, m3 = oracle.match_u8(img, tpl, 3)
    _, m4 = oracle.match_u8(img, tpl, 4)
    assert np.max(np.abs(m3 - m4)) >= 1e-3


def test_threads_bit_identical():
    img = image(77, 500, 700, 4)
    tpl = image(78, 64, 96, 4)
    t1, r1 = oracle.match_u8(img, tpl, 3, threads=1)
    for n in (2, 3, 4, 8):
        tn, rn = oracle.match_u8(img, tpl, 3, threads=n)
        assert tn == t1 and np.array_equal(rn.view(np.uint32), r1.view(np.uint32))


def test_gray_formula_known_answers():
    for w, h, pad in ((1, 1, 0), (7, 3, 0), (8, 2, 4), (33, 5, 8), (256, 4, 0), (641, 2, 12)):
        pix = image(8 + w, h, w, 4, pad // 4 + 1).copy()
        pix.reshape(-1, 4)[:16, :3] = 255 if pix.size >= 64 else pix.reshape(-1, 4)[:16, :3]
        got = oracle.rgba_to_gray(pix)
        p = pix.astype(np.uint32)
        want = ((4899 * p[..., 0] + 9617 * p[..., 1] + 1868 * p[..., 2] + 8192) >> 14).astype(np.uint8)
        assert np.array_equal(got, want)


def test_bad_arguments_text():
    a = np.zeros((10, 10, 4), np.uint8)
    b = np.zeros((20, 20, 4), np.uint8)
    with pytest.raises(oracle.OraclePanic, match=r"cvmatch: bad match arguments \(20x20 in 10x10, cn=3 step=4\)"):
        oracle.match_u8(a, b, 3)


def test_flat_template_answer():
    img = image(5, 100, 100, 4)
    tpl = np.zeros((10, 10, 4), np.uint8)
    t, res = oracle.match_u8(img, tpl, 4)
    assert t == (1.0, 0, 0, 1.0, 0, 0) and np.all(res == 1.0)


@pytest.mark.parametrize("idx", range(len(make_golden.SOLO_CASES)))
def test_oracle_reproduces_solo_fixture(idx):
    c = make_golden.SOLO_CASES[idx]
    fx = GOLDEN["solo"][idx]
    assert fx["case"] == list(c)
    img, tpl = make_golden.solo_inputs(c)
    t, res = oracle.match_u8(img, tpl, c[5], threads=2)
    assert make_golden.digest(res, t) == fx["digest"]


@pytest.mark.parametrize("idx", range(len(make_golden.FLEET_CASES)))
def test_oracle_reproduces_fleet_fixture(idx):
    c = make_golden.FLEET_CASES[idx]
    parent, tpls = make_golden.fleet_inputs(c)
    rs = oracle.fleet_find_all(tpls, parent, threads=3)
    want = GOLDEN["fleet"][idx]["results"]
    assert [[float(r[0]), r[1], r[2], float(r[3]), r[4], r[5]] for r in rs] == want


def test_single_member_fleet_is_solo():
    parent = image(301, 200, 320, 4).copy()
    parent[..., 3] = 255
    tpl = parent[50:82, 60:108].copy()
    t, _ = oracle.match_u8(parent, tpl, 3)
    (r,) = oracle.fleet_find_all([tpl], parent)
    assert r == t


# ------------------------------------------- the FP64 oracle at full sizes


@pytest.mark.parametrize("shape", REF_SHAPES)
def test_fft_fp64_definition_equals_direct_form(shape):
    """oracle/fp64.py (numerator by a float64 FFT, exact window sums) against
    the direct spatial sum of refMatch (cvmatch_test.go:13-81) on the
    reference's shapes: the same map within 1e-9."""
    from oracle import fp64
    iw, ih, tw, th, cn, ipad, tpad = shape
    img = image(42 + iw, ih, iw, cn, ipad)
    tpl = image(43 + tw, th, tw, cn, tpad)
    direct = oracle.ref_match_f64(img, tpl, cn)
    by_fft = fp64.ref_match_f64(img, tpl, cn)
    assert by_fft.shape == direct.shape
    assert np.max(np.abs(by_fft - direct)) <= 1e-9


def test_fft_fp64_flat_template_and_planted_copy():
    from oracle import fp64
    img = image(501, 90, 140, 4).copy()
    img[..., 3] = 255
    flat = np.full((10, 12, 4), 9, np.uint8)
    assert (fp64.ref_match_f64(img, flat, 3) == 1.0).all()
    t = img[30:52, 40:75].copy()
    m = fp64.ref_match_f64(img, t, 3)
    assert fp64.first_argmax(m) == (40, 30) and abs(m[30, 40] - 1.0) < 1e-12


def test_check_extrema_locations():
    """The location rule: enforced only where the top-2 margin exceeds the
    tolerance."""
    from oracle import fp64
    m = np.zeros((4, 5))
    m[1, 2], m[3, 4], m[0, 0] = 0.9, 0.89995, -0.5
    fp64.check_extrema((-0.5, 0, 0, 0.9, 2, 1), m, 1e-4)
    fp64.check_extrema((-0.5, 0, 0, 0.89995, 4, 3), m, 1e-4)  # margin 5e-5: either place
    m[3, 4] = 0.8
    with pytest.raises(AssertionError):
        fp64.check_extrema((-0.5, 0, 0, 0.8, 4, 3), m, 1e-4)


def test_fleet_subset_equals_full_find_all():
    """oracle.fleet_find_all_sel: the whole fleet's buckets and plans, tails
    of the selected members only -- bit-identical results and maps."""
    parent = image(311, 180, 260, 4).copy()
    parent[..., 3] = 255
    tpls = [parent[y:y + h, x:x + w].copy() for (x, y, w, h) in
            [(10, 12, 20, 16), (40, 30, 33, 40), (100, 90, 17, 9), (150, 20, 60, 50), (5, 120, 8, 30)]]
    full, full_maps = oracle.fleet_find_all(tpls, parent, threads=3, want_maps=True)
    res, maps, phase = oracle.fleet_find_all_sel(tpls, parent, [1, 3], threads=3, want_maps=True)
    assert set(res) == {1, 3} and res[1] == full[1] and res[3] == full[3]
    assert np.array_equal(maps[1], full_maps[1]) and np.array_equal(maps[3], full_maps[3])
    assert phase[0] >= 0 and phase[1] >= 0
