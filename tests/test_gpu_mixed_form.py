"""The mixed form (CVM_FORM_MIXED): the fast form with its 1024-point
inverse row transforms -- the inverse DFT of inverseRowPair,
impl.go:394-444 -- run as two 32-point DFT stages on the tensor cores
(tcgen05 kind::f16 matrix products on hi + lo split FP16 operands with
per-transform power-of-two scaling, FP32 accumulation).

First the path's own check (cvm_tc_selftest: the kernel's stages against a
double-precision DFT on the host); then the form held to the metric's bar
like the fast form: scores within 1e-4 of the FP64 definition
(cvmatch_test.go:13-81), extremum locations equal to the FP64 map's and the
reference's wherever their top-2 margins exceed 1e-4; and no tensor-core
wait ever gave up (cvm_device_status).
"""
import numpy as np
import pytest

import cvmatch_gb300 as cvm
import oracle
from oracle import fp64

pytestmark = pytest.mark.gpu

TOL = 1e-4


def test_tensor_core_dft_selftest():
    dft, gemm = cvm.tc_selftest()
    print(f"\ntensor-core DFT error relative to the line norm: 1024-point {dft:.2e}, first stage {gemm:.2e}")
    assert gemm < 1e-5 and dft < 1e-5
    assert cvm.device_status() == 0


@pytest.fixture
def mixed_form():
    prev = cvm.SetForm(cvm.FORM_MIXED)
    prev_t = cvm.SetAutotune(False)  # newGoPlan's 1024-wide tiles: the tensor-core rows
    yield
    cvm.SetForm(prev)
    cvm.SetAutotune(prev_t)
    assert cvm.device_status() == 0


@pytest.fixture
def no_autotune():
    prev_t = cvm.SetAutotune(False)
    yield
    cvm.SetAutotune(prev_t)


def test_mixed_match_rgba_1920x1080_vs_fp64(mixed_form):
    """C2's plan has 1024-wide tiles: every inverse row on the tensor cores."""
    import bench
    frame, tpl, at = bench.scene_ui_1920x1080()
    m, _, _ = cvm.MatchMap(frame, tpl)
    m64 = fp64.ref_match_f64(frame, tpl, 3)
    err = np.abs(m.astype(np.float64) - m64)
    print(f"\nMatch RGBA 1920x1080 / 96x32 (mixed): map max|err| {err.max():.2e}")
    assert err.max() <= TOL
    ref_map = oracle.match_u8(frame, tpl, 3, threads=16)[1]
    (mnx, mny), (mxx, mxy) = fp64.first_argmin(m), fp64.first_argmax(m)
    fp64.check_extrema((m[mny, mnx], mnx, mny, m[mxy, mxx], mxx, mxy), m64, TOL, ref_map=ref_map, name="C2 mixed")
    assert (mxx, mxy) == at
    r = tuple(cvm.Match(frame, tpl))
    assert r == (float(m[mny, mnx]), mnx, mny, float(m[mxy, mxx]), mxx, mxy)


def test_mixed_equals_fast_where_rows_are_not_1024():
    """Other row widths run the fast form unchanged: identical results."""
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, (300, 420, 4), dtype=np.uint8)
    img[..., 3] = 255
    t = img[100:140, 150:214].copy()
    p = oracle.plan(64, 40, 420 - 63, 300 - 39)
    assert p.dft_w != 1024
    prev = cvm.SetForm(cvm.FORM_FAST)
    prev_t = cvm.SetAutotune(False)  # both forms on newGoPlan's plan
    try:
        fast, _, _ = cvm.MatchMap(img, t)
        cvm.SetForm(cvm.FORM_MIXED)
        mixed, _, _ = cvm.MatchMap(img, t)
    finally:
        cvm.SetForm(prev)
        cvm.SetAutotune(prev_t)
    assert np.array_equal(fast.view(np.uint32), mixed.view(np.uint32))


def test_mixed_fleet_vs_fp64_and_fast(no_autotune):
    """A fleet whose bucket plans 1024-wide tiles, in the mixed form: every
    member against FP64 and against the fast form."""
    import bench
    frame, tpls, where = bench.scene_fleet_2560x1440(count=24)
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    assert any(b[2] == 1024 for b in fleet.buckets(2560, 1440))
    fleet.SetForm(cvm.FORM_FAST)
    fast = fleet.FindAll(frame)
    fleet.SetForm(cvm.FORM_MIXED)
    mixed = fleet.FindAll(frame)
    assert cvm.device_status() == 0
    _, ref_maps = oracle.fleet_find_all(tpls, frame, threads=16, want_maps=True)
    F = fp64.Frame(frame, 3)
    worst, worst_fast = 0.0, 0.0
    for i, t in enumerate(tpls):
        worst = max(worst, fp64.check_extrema(tuple(mixed[i]), F.match(t), TOL, ref_map=ref_maps[i],
                                              name=f"mixed member {i} {t.shape[1]}x{t.shape[0]}"))
        worst_fast = max(worst_fast, abs(mixed[i].MaxV - fast[i].MaxV), abs(mixed[i].MinV - fast[i].MinV))
        if where[i] is not None:
            assert (mixed[i].MaxX, mixed[i].MaxY) == where[i]
    print(f"\nmixed fleet: worst extremum error against FP64 {worst:.2e}, against the fast form {worst_fast:.2e}")


def test_mixed_stream_equals_mixed_find_all(no_autotune):
    """The CUDA-graph frame stream replays the tensor-core kernels: the same
    results as FindAll."""
    import bench
    frames, color, gray = bench.scene_stream_1920x1080(frames=2, ncolor=6, ngray=2)
    H, W = frames[0].shape[:2]
    cf = cvm.NewFleet(*[cvm.NewMatcher(t) for t in color])
    gf = cvm.NewFleet(*[cvm.NewGrayMatcher(t) for t in gray])
    cf.SetForm(cvm.FORM_MIXED)
    gf.SetForm(cvm.FORM_MIXED)
    st = cvm.NewStream(cf, gf, W, H)
    st.push(frames[0])
    st.push(frames[1])
    got = [st.pull(), st.pull()]
    for f, (rc, rg, _) in zip(frames, got):
        assert [tuple(r) for r in rc] == [tuple(r) for r in cf.FindAll(f)]
        assert [tuple(r) for r in rg] == [tuple(r) for r in gf.FindAll(oracle.rgba_to_gray(f))]
    assert cvm.device_status() == 0
