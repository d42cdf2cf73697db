"""Score error of the GPU maps against the FP64 direct spatial correlation
(the refMatch definition of cvmatch_test.go:13-81) on the benchmark
configurations, and agreement of the peak locations.

The GPU path reproduces the reference's FP32 pipeline bit for bit (checked
in test_gpu_parity.py), so these errors are the reference's own: on natural
images they stay near 1e-5, on UI-like scenes with near-flat windows the
reference's float32 tail drifts further (its own worst recorded drift is
5.5e-4, CLAUDE.md:61-75).  The bound asserted here is that one; the measured
values are printed (pytest -s) for the results table.
"""
import numpy as np
import pytest

import cvmatch_gb300 as cvm
import oracle

pytestmark = pytest.mark.gpu

TOL_REF_DRIFT = 5.5e-4   # the reference's own worst drift against FP64


def _report(name, m32, m64):
    err = np.abs(m32.astype(np.float64) - m64)
    gi, ri = np.unravel_index(np.argmax(m32), m32.shape), np.unravel_index(np.argmax(m64), m64.shape)
    top = np.sort(m64.ravel())[-2:]
    print(f"\n{name}: max|err| {err.max():.3e}  mean {err.mean():.3e}  >1e-4: {int((err > 1e-4).sum())} of {err.size}"
          f"  argmax gpu {gi[::-1]} fp64 {ri[::-1]}  fp64 top-2 margin {top[1] - top[0]:.3e}")
    return err.max(), gi, ri, top[1] - top[0]


FORMS = {"exact": cvm.FORM_EXACT, "fast": cvm.FORM_FAST}


@pytest.fixture(params=["exact", "fast"])
def form(request):
    prev = cvm.SetForm(FORMS[request.param])
    yield request.param
    cvm.SetForm(prev)


def test_gray_640x480_vs_fp64(form):
    import bench
    rgba, tpl, _ = bench.scene_gray_640x480()
    g, t = cvm.rgba_to_gray(rgba), cvm.rgba_to_gray(tpl)
    _, m = cvm.match_u8(g, t, 1)
    m64 = oracle.ref_match_f64(g, t, 1, threads=16)
    e, gi, ri, margin = _report(f"MatchGray 640x480 / 64x48 ({form})", m, m64)
    assert e <= TOL_REF_DRIFT
    if margin > 1e-4:
        assert gi == ri


def test_rgba_1920x1080_vs_fp64(form):
    import bench
    frame, tpl, _ = bench.scene_ui_1920x1080()
    m, _, _ = cvm.MatchMap(frame, tpl)
    m64 = oracle.ref_match_f64(frame, tpl, 3, threads=16)
    e, gi, ri, margin = _report(f"Match RGBA 1920x1080 / 96x32 ({form})", m, m64)
    assert e <= TOL_REF_DRIFT
    if margin > 1e-4:
        assert gi == ri
