"""Seeded random one-shot matches at odd sizes, colour and gray: the exact
form's full score map and result bit-identical to the oracle's matchU8
(impl.go:1126-1155), the fast form's (with the autotuner choosing its tile
plan) within 1e-4 of the FP64 definition (cvmatch_test.go:13-81) with the
extremum locations the FP64 map and the reference's map determine.
"""
import numpy as np
import pytest

import cvmatch_gb300 as cvm
import oracle
from oracle import fp64

pytestmark = pytest.mark.gpu

TOL = 1e-4

_g = np.random.default_rng(4242)
CASES = []
for _s in range(16):
    _h, _w = int(_g.integers(4, 700)), int(_g.integers(4, 900))
    _th, _tw = int(_g.integers(1, _h + 1)), int(_g.integers(1, _w + 1))
    CASES.append((200 + _s, _h, _w, _th, _tw, int(_g.integers(0, 3))))  # kind: 0 gray, 1 colour, 2 colour + varying alpha


def _scene(seed, h, w, kind):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    for _ in range(10):
        rw, rh = int(rng.integers(1, max(2, w // 2))), int(rng.integers(1, max(2, h // 2)))
        x, y = int(rng.integers(0, w - rw + 1)), int(rng.integers(0, h - rh + 1))
        img[y:y + rh, x:x + rw, :3] = rng.integers(0, 256, 3)
    if kind != 2:
        img[..., 3] = 255
    return img, rng


@pytest.mark.parametrize("case", CASES, ids=[f"seed{c[0]}" for c in CASES])
def test_random_match_exact_and_fast(case):
    seed, h, w, th, tw, kind = case
    img, rng = _scene(seed, h, w, kind)
    x, y = int(rng.integers(0, w - tw + 1)), int(rng.integers(0, h - th + 1))
    if kind == 0:
        src, cn = cvm.rgba_to_gray(img), 1
    else:
        src, cn = img, (4 if kind == 2 else 3)
    tpl = src[y:y + th, x:x + tw].copy()
    prev = cvm.SetForm(cvm.FORM_EXACT)
    try:
        got, m = cvm.match_u8(src, tpl, cn)
        want, wm = oracle.match_u8(src, tpl, cn, threads=16)
        assert np.array_equal(m.view(np.uint32), wm.view(np.uint32))
        assert np.float32(got[0]).view(np.uint32) == np.float32(want[0]).view(np.uint32) and got[1:3] == want[1:3]
        assert np.float32(got[3]).view(np.uint32) == np.float32(want[3]).view(np.uint32) and got[4:6] == want[4:6]
        cvm.SetForm(cvm.FORM_FAST)
        fast, fm = cvm.match_u8(src, tpl, cn)
    finally:
        cvm.SetForm(prev)
    m64 = fp64.ref_match_f64(src, tpl, cn)
    err = float(np.abs(fm.astype(np.float64) - m64).max())
    assert err <= TOL, (case, err)
    fp64.check_extrema(tuple(fast), m64, TOL, ref_map=wm, name=f"seed {seed}")
