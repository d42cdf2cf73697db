"""cvm_match_u8_device_noalloc: the entry point for callers that cannot
allocate device memory (their device memory belongs to another allocator,
or a driver allocation's latency is not acceptable in their loop).  Its
workspace is a fixed array inside the library, shared by every call, so
these tests check that two different calls in a row each give exactly the
result of the allocating entry point (cvm_match_u8_device, pinned to the
exact form, which is the form the fixed-scratch entry always computes) and
of the oracle (the reference's float32 path restated on the CPU), i.e.
nothing from the previous call leaks into the next, and that matches too
large for the fixed array or too wide for its shared-memory staging are
refused with a clear error instead of running.

This file is collected last on purpose: it must pass alone in a fresh
process (the first call performs the one-time set-up) and after every
other test.
"""
import ctypes as C

import numpy as np
import pytest

import cvmatch_gb300 as cvm
import oracle

pytestmark = pytest.mark.gpu

ARGS = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int,
        C.c_void_p, C.c_void_p, C.c_void_p]


def _lib():
    L = cvm.lib()
    L.cvm_match_u8_device_noalloc.argtypes = ARGS
    L.cvm_match_u8_device.argtypes = ARGS
    return L


def _run(fn, img, tpl, cn, want_map):
    torch = pytest.importorskip("torch")
    img = np.ascontiguousarray(img)
    tpl = np.ascontiguousarray(tpl)
    step = 1 if img.ndim == 2 else img.shape[2]
    ih, iw = img.shape[:2]
    th, tw = tpl.shape[:2]
    rw, rh = iw - tw + 1, ih - th + 1
    d_img = torch.from_numpy(img).cuda()
    d_tpl = torch.from_numpy(tpl).cuda()
    d_map = torch.full((rh, rw), float("nan"), dtype=torch.float32, device="cuda") if want_map else None
    d_out = torch.zeros(6, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = fn(d_img.data_ptr(), img.strides[0], iw, ih, d_tpl.data_ptr(), tpl.strides[0], tw, th, cn, step,
            d_map.data_ptr() if want_map else None, d_out.data_ptr(), stream)
    torch.cuda.synchronize()
    out = d_out.cpu().numpy()
    return rc, (d_map.cpu().numpy() if want_map else None), out


def _err():
    buf = C.create_string_buffer(512)
    cvm.lib().cvm_last_error(buf, 512)
    return buf.value.decode()


def _case_colour():
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, (400, 640, 4), dtype=np.uint8)
    img[..., 3] = 255
    tpl = img[100:132, 200:296].copy()
    return img, tpl, 3


def _case_gray():
    rng = np.random.default_rng(6)
    img = rng.integers(0, 256, (200, 300), dtype=np.uint8)
    tpl = rng.integers(0, 256, (29, 31), dtype=np.uint8)
    return img, tpl, 1


@pytest.fixture
def exact_form():
    """The allocating entry point reads the process-wide form: pin it to the
    exact form (the fixed-scratch entry's) whatever earlier tests left."""
    prev = cvm.SetForm(cvm.FORM_EXACT)
    yield
    cvm.SetForm(prev)


def _tuple(out):
    return (float(out[:1].view(np.float32)[0]), int(out[1]), int(out[2]), float(out[3:4].view(np.float32)[0]),
            int(out[4]), int(out[5]))


def test_two_calls_in_a_row_match_the_allocating_entry_point(exact_form):
    L = _lib()
    for img, tpl, cn in (_case_colour(), _case_gray(), _case_colour()):
        want_t, want_map = oracle.match_u8(img, tpl, cn, threads=8)
        for map_wanted in (True, False):
            rc0, m0, o0 = _run(L.cvm_match_u8_device, img, tpl, cn, map_wanted)
            assert rc0 == 0, _err()
            rc1, m1, o1 = _run(L.cvm_match_u8_device_noalloc, img, tpl, cn, map_wanted)
            assert rc1 == 0, _err()
            # the tests' tolerance is bit identity: with the allocating entry
            # point and with the reference's own result (the oracle)
            assert np.array_equal(o1, o0)
            assert _tuple(o1) == want_t
            if map_wanted:
                assert np.array_equal(m1.view(np.uint32), m0.view(np.uint32))
                assert np.array_equal(m1.view(np.uint32), want_map.view(np.uint32))


def test_fast_form_setting_does_not_change_the_fixed_scratch_result():
    L = _lib()
    img, tpl, cn = _case_colour()
    want_t, _ = oracle.match_u8(img, tpl, cn, threads=8)
    prev = cvm.SetForm(cvm.FORM_FAST)
    try:
        rc, _, out = _run(L.cvm_match_u8_device_noalloc, img, tpl, cn, False)
    finally:
        cvm.SetForm(prev)
    assert rc == 0, _err()
    assert _tuple(out) == want_t


def test_oversized_match_is_refused():
    L = _lib()
    rng = np.random.default_rng(7)
    img = rng.integers(0, 256, (2160, 3840), dtype=np.uint8)
    tpl = img[:256, :256].copy()
    rc, _, _ = _run(L.cvm_match_u8_device_noalloc, img, tpl, 1, False)
    assert rc == 11  # CVM_ERR_UNSUPPORTED
    assert "fixed device scratch" in _err()


def test_template_too_wide_for_shared_memory_is_refused():
    """A 6000-pixel-wide RGBA template would need ~245 KB of shared memory
    per block in the normalisation; refused before anything is queued."""
    L = _lib()
    rng = np.random.default_rng(8)
    img = rng.integers(0, 256, (200, 6000, 4), dtype=np.uint8)
    img[..., 3] = 255
    tpl = img[50:54, :].copy()
    rc, _, _ = _run(L.cvm_match_u8_device_noalloc, img, tpl, 3, False)
    assert rc == 11  # CVM_ERR_UNSUPPORTED
    assert "shared memory" in _err()
