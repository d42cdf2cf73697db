"""A fast-form fleet's window statistics formed inside the inverse-rows
epilogue from the frame's summed-area table (CVM_STATS_EPILOGUE) against
the statistics kernel (CVM_STATS_KERNEL, the default): the epilogue restores
each window's squared sum from its residue modulo 2^32 and runs the
kernel's den sequence on the same integers, so every result must be the
same bits.  normalizeBandGo (impl.go:708-805) computes these statistics
once per band in the reference; here they are checked on the benchmark's
256-template fleet, on random fleets (odd sizes, varying alpha: the
table's alpha block), on gray fleets, and at the largest member area the
table serves for a four-channel member (257 x 257 on windows of
alternating 127/128 bytes, where U - q is within 0.1 % of 2^32) and just
beyond it (the statistics kernel then runs for that bucket).

The restoration itself, q = U - ((U - q_mod) mod 2^32) with U = 255 x
(sum of the channel sums), is checked on the CPU against exact window
sums of extreme windows.
"""
import numpy as np
import pytest

import cvmatch_gb300 as cvm

TWO32 = 1 << 32


def _restore(sums, q):
    """The epilogue's restoration from residues modulo 2^32."""
    U = 255 * sum(int(s) % TWO32 for s in sums)
    return U - ((U - q % TWO32) % TWO32)


@pytest.mark.parametrize("area,cn,fill", [
    (66052, 4, "alt"),     # the largest four-channel area served, worst case U - q
    (66052, 4, "max"),     # every byte 255: q = U
    (88069, 3, "alt"),     # three channels
    (264208, 1, "alt"),    # gray
    (264208, 1, "zero"),
    (24576, 3, "rand"),
])
def test_squared_sum_restored_from_residue(area, cn, fill):
    rng = np.random.default_rng(area + cn)
    if fill == "alt":
        v = np.where(np.arange(area * cn) % 2 == 0, 127, 128)
    elif fill == "max":
        v = np.full(area * cn, 255)
    elif fill == "zero":
        v = np.zeros(area * cn, np.int64)
    else:
        v = rng.integers(0, 256, area * cn)
    v = v.astype(np.int64).reshape(area, cn)
    sums = v.sum(axis=0)
    q = int((v * v).sum())
    assert 255 * int(sums.sum()) - q < TWO32          # the bound the host checks
    assert area * cn * 16256 < TWO32
    assert _restore(sums, q) == q


@pytest.mark.parametrize("cn,area", [(4, 66052), (3, 88069), (1, 264208)])
def test_restoration_bound_is_tight(cn, area):
    """One pixel more than the largest area served and the worst window
    (alternating 127/128 bytes) reaches 2^32: the residue no longer
    determines q, so the host must send that bucket to the kernel."""
    assert area * cn * 16256 < TWO32 <= (area + 1) * cn * 16256
    v = np.where(np.arange((area + 1) * cn) % 2 == 0, 127, 128).astype(np.int64)
    q = int((v * v).sum())
    assert 255 * int(v.sum()) - q >= TWO32
    assert _restore(v.reshape(area + 1, cn).sum(axis=0), q) != q


def _same(a, b):
    for i, (g, r) in enumerate(zip(a, b)):
        g, r = tuple(g), tuple(r)
        assert np.float32(g[0]).view(np.uint32) == np.float32(r[0]).view(np.uint32) and g[1:3] == r[1:3], (i, g, r)
        assert np.float32(g[3]).view(np.uint32) == np.float32(r[3]).view(np.uint32) and g[4:6] == r[4:6], (i, g, r)


def _both(fleet, img):
    """FindAll in the fast form with the statistics in the epilogue and
    with the statistics kernel, and the launches each took."""
    L = cvm.lib()
    fleet.SetForm(cvm.FORM_FAST)
    try:
        fleet.SetStats(cvm.STATS_KERNEL)
        fleet.FindAll(img)  # geometry, plans and template spectra
        n0 = L.cvm_launch_count()
        ker = [tuple(r) for r in fleet.FindAll(img)]
        n1 = L.cvm_launch_count()
        fleet.SetStats(cvm.STATS_EPILOGUE)
        epi = [tuple(r) for r in fleet.FindAll(img)]
        n2 = L.cvm_launch_count()
    finally:
        fleet.SetStats(cvm.STATS_KERNEL)
        fleet.SetForm(cvm.FORM_EXACT)
    return epi, ker, n2 - n1, n1 - n0


@pytest.mark.gpu
def test_c4_fleet_epilogue_statistics_equal_kernel():
    import bench
    frame, tpls, _ = bench.scene_fleet_2560x1440()
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    epi, ker, na, nk = _both(fleet, frame)
    assert len(epi) == 256
    _same(epi, ker)
    # a different set of launches: per wave no statistics kernel, per frame
    # the table's builds instead of the prefix's block sums
    assert na != nk, (na, nk)
    assert cvm.device_status() == 0


def _frame(rng, h, w, alpha_varies):
    img = np.empty((h, w, 4), np.uint8)
    img[..., :3] = rng.integers(0, 256, (h, w, 3))
    for _ in range(10):
        rw, rh = int(rng.integers(2, max(3, w // 2))), int(rng.integers(2, max(3, h // 2)))
        x, y = int(rng.integers(0, w - rw + 1)), int(rng.integers(0, h - rh + 1))
        img[y:y + rh, x:x + rw, :3] = rng.integers(0, 256, 3)
    img[..., 3] = rng.integers(0, 256, (h, w)) if alpha_varies else 255
    return img


@pytest.mark.gpu
@pytest.mark.parametrize("seed,h,w,n,alpha,gray", [
    (11, 300, 517, 9, False, False),
    (12, 200, 260, 7, True, False),    # four-channel members
    (13, 97, 641, 12, False, False),
    (14, 400, 300, 5, True, False),
    (15, 333, 517, 8, False, True),    # gray fleet
    (16, 40, 900, 6, False, True),
])
def test_random_fleet_epilogue_statistics_equal_kernel(seed, h, w, n, alpha, gray):
    rng = np.random.default_rng(seed)
    img = _frame(rng, h, w, alpha)
    tpls = []
    for _ in range(n):
        tw, th = int(rng.integers(1, min(150, w) + 1)), int(rng.integers(1, min(120, h) + 1))
        x, y = int(rng.integers(0, w - tw + 1)), int(rng.integers(0, h - th + 1))
        tpls.append(img[y:y + th, x:x + tw].copy())
    mk = cvm.NewGrayMatcher if gray else cvm.NewMatcher
    fleet = cvm.NewFleet(*[mk(t) for t in tpls])
    epi, ker, na, nk = _both(fleet, img)
    _same(epi, ker)
    assert cvm.device_status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("tw", [257, 258])
def test_area_bound_four_channels(tw):
    """A four-channel member of 257 x 257 (area 66049, inside the bound) and
    of 258 x 257 (beyond it: its bucket runs the statistics kernel) on a
    frame of alternating 127/128 bytes in every channel, alpha included --
    windows whose U - q is the largest the table must restore -- with a
    textured strip so that the scores are not all near-flat."""
    rng = np.random.default_rng(tw)
    h, w = 420, 700
    img = np.where((np.arange(h)[:, None, None] + np.arange(w)[None, :, None] + np.arange(4)) % 2 == 0,
                   127, 128).astype(np.uint8)
    img[300:, :, :3] = rng.integers(0, 256, (h - 300, w, 3))
    img = np.ascontiguousarray(img)
    tpls = [img[10:267, 40:40 + tw].copy(), img[150:407, 300:300 + tw].copy(), img[5:60, 5:90].copy()]
    fleet = cvm.NewFleet(*[cvm.NewMatcher(t) for t in tpls])
    epi, ker, na, nk = _both(fleet, img)
    _same(epi, ker)
    assert cvm.device_status() == 0
