"""Score error of the full GPU maps against the FP64 TM_CCOEFF_NORMED
definition (refMatch, cvmatch_test.go:13-81) on the benchmark
configurations, and agreement of the extremum locations.

- The fast form (the reported one) is held to the metric's bar: every score
  of the full map within 1e-4 of FP64, and each extremum located where the
  FP64 map puts it whenever that map's top-2 margin exceeds 1e-4, and where
  the reference's own map puts it whenever the reference map's margin does
  (identical max/min locations wherever the reference's top-2 margin
  exceeds the tolerance).
- The exact form reproduces the reference's float32 pipeline bit for bit
  (test_gpu_parity.py), so its errors here are the reference's own: on
  UI-like scenes with near-flat windows they exceed 1e-4 (the reference's
  worst recorded drift against FP64 is 5.5e-4, CLAUDE.md:61-75); that is
  the bound it is held to, with the same location rules.

The FP64 maps come from oracle/fp64.py (the definition with its numerator
taken by a float64 FFT; pinned to the direct form in test_oracle_pins.py).
Measured errors are printed (pytest -s).
"""
import numpy as np
import pytest

import cvmatch_gb300 as cvm
import oracle
from oracle import fp64

pytestmark = pytest.mark.gpu

TOL = {"fast": 1e-4, "exact": 5.5e-4}   # the metric's bar; the reference's own worst drift
FORMS = {"exact": cvm.FORM_EXACT, "fast": cvm.FORM_FAST}


@pytest.fixture(params=["exact", "fast"])
def form(request):
    prev = cvm.SetForm(FORMS[request.param])
    yield request.param
    cvm.SetForm(prev)


def _check(name, form, m32, m64, ref_map):
    err = np.abs(m32.astype(np.float64) - m64)
    print(f"\n{name} ({form}): max|err| {err.max():.3e}  mean {err.mean():.3e}  >1e-4: "
          f"{int((err > 1e-4).sum())} of {err.size}")
    assert err.max() <= TOL[form]
    (mnx, mny), (mxx, mxy) = fp64.first_argmin(m32), fp64.first_argmax(m32)
    fp64.check_extrema((m32[mny, mnx], mnx, mny, m32[mxy, mxx], mxx, mxy), m64, TOL[form], ref_map=ref_map,
                       name=name)
    if form == "exact":
        assert np.array_equal(m32, ref_map)  # the reference's bits


def test_gray_640x480_vs_fp64(form):
    import bench
    rgba, tpl, at = bench.scene_gray_640x480()
    g, t = cvm.rgba_to_gray(rgba), cvm.rgba_to_gray(tpl)
    _, m = cvm.match_u8(g, t, 1)
    ref_map = oracle.match_u8(g, t, 1, threads=16)[1]
    _check("MatchGray 640x480 / 64x48", form, m, fp64.ref_match_f64(g, t, 1), ref_map)
    assert fp64.first_argmax(m) == at


def test_rgba_1920x1080_vs_fp64(form):
    import bench
    frame, tpl, at = bench.scene_ui_1920x1080()
    m, _, _ = cvm.MatchMap(frame, tpl)
    ref_map = oracle.match_u8(frame, tpl, 3, threads=16)[1]
    _check("Match RGBA 1920x1080 / 96x32", form, m, fp64.ref_match_f64(frame, tpl, 3), ref_map)
    assert fp64.first_argmax(m) == at


def test_gray_3840x2160_full_map_vs_fp64(form):
    """The full 3585 x 1905 MatchMap of a 256 x 256 template (C3)."""
    import bench
    g, tpl, at = bench.scene_gray_3840x2160()
    _, m = cvm.match_u8(g, tpl, 1)
    assert m.shape == (1905, 3585)
    ref_map = oracle.match_u8(g, tpl, 1, threads=16)[1]
    _check("MatchMap gray 3840x2160 / 256x256", form, m, fp64.ref_match_f64(g, tpl, 1), ref_map)
    assert fp64.first_argmax(m) == at
