"""TMA-staged frame rows in the forward row transform (forwardRowPair,
impl.go:301-344): frames whose address and row pitch are 16-byte aligned
are copied into shared memory by cp.async.bulk.tensor boxes (the profile
labels those launches k_fwd_rows_tma); other frames take plain loads.
Either way the exact form's results are the reference's bits."""
import ctypes as C

import numpy as np
import pytest

import cvmatch_gb300 as cvm
import oracle

pytestmark = pytest.mark.gpu


def _profiled(fn):
    L = cvm.lib()
    L.cvm_profile_enable.argtypes = [C.c_int]
    L.cvm_profile_enable.restype = None
    L.cvm_profile_read.argtypes = [C.c_int, C.c_char_p, C.c_size_t, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
    L.cvm_profile_enable(1)
    try:
        out = fn()
    finally:
        L.cvm_profile_enable(0)
    names, i = [], 0
    buf, ms, n = C.create_string_buffer(64), C.c_double(), C.c_uint64()
    while L.cvm_profile_read(i, buf, 64, C.byref(ms), C.byref(n)) == 0:
        names.append(buf.value.decode())
        i += 1
    return out, names


def _scene(seed, h, w):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    img[..., 3] = 255
    for _ in range(20):
        rw, rh = int(rng.integers(10, w // 3)), int(rng.integers(10, h // 3))
        x, y = int(rng.integers(0, w - rw)), int(rng.integers(0, h - rh))
        img[y:y + rh, x:x + rw, :3] = rng.integers(0, 256, 3)
    return img


@pytest.fixture
def exact():
    prev = cvm.SetForm(cvm.FORM_EXACT)
    yield
    cvm.SetForm(prev)


def test_host_frame_rows_staged_by_tma_bit_exact(exact):
    img = _scene(301, 700, 1500)
    t = img[200:248, 333:413].copy()          # x0 offsets of the tiles are not 16-byte multiples
    (r, m), names = _profiled(lambda: cvm.match_u8(img, t, 3))
    assert "k_fwd_rows_tma" in names, names
    want, wm = oracle.match_u8(img, t, 3, threads=16)
    assert r == want and np.array_equal(m.view(np.uint32), wm.view(np.uint32))
    assert cvm.device_status() == 0


def test_gray_frame_rows_staged_by_tma_bit_exact(exact):
    g = oracle.rgba_to_gray(_scene(303, 640, 1400))
    t = g[100:160, 511:600].copy()
    (r, m), names = _profiled(lambda: cvm.match_u8(g, t, 1))
    assert "k_fwd_rows_tma" in names, names
    want, wm = oracle.match_u8(g, t, 1, threads=16)
    assert r == want and np.array_equal(m.view(np.uint32), wm.view(np.uint32))


def test_unaligned_device_frame_takes_plain_loads(exact):
    """A device frame 4 bytes past a 16-byte boundary (row pitch a multiple
    of 4 but not of 16): no tensor map, plain loads, the same bits."""
    torch = pytest.importorskip("torch")
    img = _scene(307, 500, 1300)
    t = img[120:160, 400:470].copy()
    H, W = img.shape[:2]
    pitch = W * 4 + 4
    raw = torch.zeros(H * pitch + 16, dtype=torch.uint8, device="cuda")
    view = raw[4:4 + H * pitch].view(H, pitch)[:, :W * 4]
    view.copy_(torch.from_numpy(img.reshape(H, W * 4)))
    d_tpl = torch.from_numpy(t).cuda()
    rh, rw = H - t.shape[0] + 1, W - t.shape[1] + 1
    d_map = torch.empty((rh, rw), dtype=torch.float32, device="cuda")
    d_out = torch.zeros(6, dtype=torch.int32, device="cuda")
    L = cvm.lib()

    def run():
        rc = L.cvm_match_u8_device(view.data_ptr(), pitch, W, H, d_tpl.data_ptr(), t.strides[0], t.shape[1],
                                   t.shape[0], 3, 4, d_map.data_ptr(), d_out.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        return rc

    rc, names = _profiled(run)
    assert rc == 0
    assert "k_fwd_rows_tma" not in names and "k_fwd_rows" in names, names
    want, wm = oracle.match_u8(img, t, 3, threads=16)
    assert np.array_equal(d_map.cpu().numpy().view(np.uint32), wm.view(np.uint32))
