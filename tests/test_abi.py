"""The C ABI library builds, loads, and exports every symbol include/cvmatch_gpu.h
declares; argument errors carry the reference's panic text.  No compute
call is made here (these run without a GPU)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import cvmatch_gb300 as cvm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cvmatch_gpu.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(cvm_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = cvm.lib()
    path = cvm.library_path()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (cvm_[a-z0-9_]+)", out))
    decl = declared_symbols()
    assert len(decl) >= 20
    missing = [s for s in decl if s not in exported]
    assert not missing, missing
    for s in decl:
        assert hasattr(L, s)


def test_header_compiles_as_c():
    src = '#include "cvmatch_gpu.h"\nint main(void){cvm_result r; (void)r; return CVM_OK;}\n'
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.dirname(HEADER), "-x", "c", "-",
                        "-o", "/dev/null"], input=src, text=True, capture_output=True)
    assert r.returncode == 0, r.stderr


def _err(rc):
    buf = C.create_string_buffer(512)
    cvm.lib().cvm_last_error(buf, 512)
    return rc, buf.value.decode()


def test_bad_arguments_rejected_before_any_device_work():
    L = cvm.lib()
    a = np.zeros((10, 10, 4), np.uint8)
    b = np.zeros((20, 20, 4), np.uint8)
    r = cvm._CResult()
    rc, msg = _err(L.cvm_match(a.ctypes.data, 40, 10, 10, b.ctypes.data, 80, 20, 20, C.byref(r)))
    assert rc == 1 and msg == "cvmatch: bad match arguments (20x20 in 10x10, cn=3 step=4)"
    a[0, 1, 3] = 7  # parent alpha varies: the reference picks cn=4 before it panics
    rc, msg = _err(L.cvm_match(a.ctypes.data, 40, 10, 10, b.ctypes.data, 80, 20, 20, C.byref(r)))
    assert rc == 1 and msg == "cvmatch: bad match arguments (20x20 in 10x10, cn=4 step=4)"
    rc, msg = _err(L.cvm_match(None, 40, 10, 10, b.ctypes.data, 80, 20, 20, C.byref(r)))
    assert rc == 5 and msg == "cvmatch: nil image"
    rc, msg = _err(L.cvm_match(a.ctypes.data, 40, 0, 10, b.ctypes.data, 80, 20, 20, C.byref(r)))
    assert rc == 6 and msg == "cvmatch: empty image"
    rc, msg = _err(L.cvm_match_u8(a.ctypes.data, 40, 10, 10, a.ctypes.data, 40, 5, 5, 5, 4, None,
                                  C.byref(r)))
    assert rc == 1 and msg == "cvmatch: bad match arguments (5x5 in 10x10, cn=5 step=4)"


def test_stats_cap_rejected():
    L = cvm.lib()
    r = cvm._CResult()
    big = np.zeros((2500, 2500, 4), np.uint8)
    big[0, 1, 3] = 1  # varying alpha: cn=4, whose cap 5954902 < 2500*2500
    rc, msg = _err(L.cvm_match(big.ctypes.data, 10000, 2500, 2500, big.ctypes.data, 10000, 2500, 2500,
                               C.byref(r)))
    assert rc == 2 and msg == "cvmatch: template area 2500x2500 exceeds the exact-statistics bound for cn=4"
    m = C.c_void_p()
    rc, msg = _err(L.cvm_matcher_new(big.ctypes.data, 10000, 2500, 2500, 4, C.byref(m)))
    assert rc == 2 and msg == "cvmatch: template area 2500x2500 exceeds the exact-statistics bound"


def test_python_mirror_errors():
    with pytest.raises(cvm.CvmatchError, match="cvmatch: nil image"):
        cvm.Match(None, np.zeros((2, 2, 4), np.uint8))
    with pytest.raises(cvm.CvmatchError, match="cvmatch: empty image"):
        cvm.Match(np.zeros((0, 2, 4), np.uint8), np.zeros((2, 2, 4), np.uint8))
    with pytest.raises(cvm.CvmatchError, match="cvmatch: empty fleet"):
        cvm.NewFleet()


def test_version_string():
    assert b"sm_103a" in cvm.lib().cvm_version()


def test_product_planner_matches_reference_pins():
    """The library's own planner (not the oracle's) against plan_test.go:12-28."""
    from test_oracle_pins import PLAN_PINS
    L = cvm.lib()
    for pin in PLAN_PINS:
        out = (C.c_int32 * 6)()
        assert L.cvm_plan(*pin[:4], out) == 0
        assert tuple(out[:4]) == pin[4:]


def test_product_planner_matches_oracle_shrink():
    import oracle
    L = cvm.lib()
    for (tw, th, iw, ih) in [(31, 29, 316, 330), (24, 18, 316, 359), (9, 33, 40, 533), (96, 32, 1920, 1080),
                             (256, 256, 3840, 2160), (64, 48, 640, 480)]:
        rw, rh = iw - tw + 1, ih - th + 1
        out = (C.c_int32 * 6)()
        assert L.cvm_plan(tw, th, rw, rh, out) == 0
        p = oracle.plan(tw, th, rw, rh)
        assert out[4] == oracle.shrink_dh(p, rh, th)


def test_product_planner_matches_oracle_random_shapes():
    """The library's planner (band sums in closed form) picks the oracle's
    plan (the band-by-band loop of newGoPlan, impl.go:246-295) on random
    shapes, including tall results with many short bands."""
    import numpy as np
    import oracle
    L = cvm.lib()
    rng = np.random.default_rng(7)
    for _ in range(400):
        tw, th = (int(v) for v in rng.integers(1, 300, 2))
        rw, rh = (int(v) for v in rng.integers(1, 4000, 2))
        out = (C.c_int32 * 6)()
        assert L.cvm_plan(tw, th, rw, rh, out) == 0
        p = oracle.plan(tw, th, rw, rh)
        assert (out[0], out[1], out[2], out[3]) == (p.dft_w, p.dft_h, p.block_w, p.block_h), (tw, th, rw, rh)


def test_form_setters_validate_without_device_work():
    """cvm_set_form / cvm_get_form: the process-wide form of one-shot
    matches; an unknown form is refused and leaves the form unchanged."""
    L = cvm.lib()
    assert L.cvm_get_form() == cvm.FORM_EXACT
    rc, msg = _err(L.cvm_set_form(7))
    assert rc == 1 and "unknown form 7" in msg
    assert L.cvm_get_form() == cvm.FORM_EXACT
    assert L.cvm_set_form(cvm.FORM_FAST) == 0 and L.cvm_get_form() == cvm.FORM_FAST
    assert cvm.SetForm(cvm.FORM_EXACT) == cvm.FORM_FAST and L.cvm_get_form() == cvm.FORM_EXACT
    rc, msg = _err(L.cvm_fleet_set_form(None, cvm.FORM_FAST))
    assert rc == 3 and msg == "cvmatch: empty fleet"


def test_no_device_fails_loudly():
    """Without an sm_103 device every compute entry raises: there is no CPU
    fallback behind the C ABI.  (Skipped where a device is present.)"""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    img = np.zeros((40, 60, 4), np.uint8)
    img[5:20, 7:30] = 200
    sub = img[5:15, 10:25].copy()
    for call in (lambda: cvm.Match(img, sub), lambda: cvm.MatchMap(img, sub),
                 lambda: cvm.MatchGray(img[..., 0].copy(), sub[..., 0].copy()),
                 lambda: cvm.NewFleet(cvm.NewMatcher(sub)).FindAll(img)):
        with pytest.raises(cvm.CvmatchError, match="no CUDA device"):
            call()
