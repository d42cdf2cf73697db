"""FP64 TM_CCOEFF_NORMED by FFT: the refMatch definition at full frame sizes.

TEST INFRASTRUCTURE ONLY (the checker; the product never imports it).

`cvo_ref_match_f64` (cvm_oracle.c) restates refMatch (cvmatch_test.go:13-81)
as the direct spatial sum: O(rw * rh * tw * th) multiply-adds, minutes for
a 256 x 256 template on a 3840 x 2160 frame and hours for a 256-member
fleet on 2560 x 1440.  This module computes the same definition with the
correlation numerator taken by a float64 FFT, so full-size maps take
seconds:

- window sums of every channel and of the squared pixels come from exact
  int64 summed-area tables, and the denominator is then formed with the
  same float64 operations, in the same order, as refMatch's
  (`wm2 = sum_k wsum_k^2`, `* 1/area`, `diff2 = wsum2 - wm2` clamped at 0,
  `lim = min(10*FLT_EPSILON * wsum2, 0.5)`, `den = sqrt(diff2) * templNorm`),
  so `den` is bit-identical to the direct form's;
- the numerator `sum(I*T) - sum_k wsum_k*mean_k` is the correlation of the
  frame offset by 128 with the exact-integer zero-sum template
  `area*T - sum(T)` per channel, divided by `area` at the end (both
  rewrites are exact in real arithmetic: the template sums to zero, so the
  offset drops out); the channels are summed in the frequency domain.
  Its float64 rounding is ~1e-16 of the product of the operands' norms,
  far below every tolerance it is used against (the CPU test pins it to
  the direct form within 1e-9 on the reference's shapes);
- the guard ladder is refMatch's (|num| < den: num/den; < 1.125 den: +-1;
  else 0) and a flat template gives a map of ones.
"""
from __future__ import annotations

import os

import numpy as np

try:
    import scipy.fft as _fft
    _next_fast = _fft.next_fast_len
except ImportError:  # numpy only
    _fft = None

    def _next_fast(n, real=True):
        m = 1
        while m < n:
            m *= 2
        return m

FLT_EPS10 = 1.1920929e-06   # Go folds the constant 10*fltEps exactly (cvmatch_test.go)
_WORKERS = max(1, min(16, os.cpu_count() or 1))


def _rfft2(a, shape):
    if _fft is not None:
        return _fft.rfft2(a, s=shape, workers=_WORKERS)
    return np.fft.rfft2(a, s=shape)


def _irfft2(a, shape):
    if _fft is not None:
        return _fft.irfft2(a, s=shape, workers=_WORKERS)
    return np.fft.irfft2(a, s=shape)


def _planes(img: np.ndarray, cn: int):
    """uint8 H x W (x C) view -> list of cn int64 planes."""
    if img.ndim == 2:
        assert cn == 1
        return [img.astype(np.int64)]
    return [img[..., k].astype(np.int64) for k in range(cn)]


def _sat(a: np.ndarray) -> np.ndarray:
    """Exclusive 2-D prefix sums, (H+1) x (W+1), int64."""
    s = np.zeros((a.shape[0] + 1, a.shape[1] + 1), np.int64)
    np.cumsum(np.cumsum(a, axis=0, dtype=np.int64), axis=1, dtype=np.int64, out=s[1:, 1:])
    return s


def _window(s: np.ndarray, th: int, tw: int, rh: int, rw: int) -> np.ndarray:
    return s[th:th + rh, tw:tw + rw] - s[0:rh, tw:tw + rw] - s[th:th + rh, 0:rw] + s[0:rh, 0:rw]


class Frame:
    """One frame's FP64 state: its per-channel spectra (offset by 128) and
    exact window-sum tables, shared by every template matched against it."""

    def __init__(self, img: np.ndarray, cn: int, pad=(0, 0)):
        planes = _planes(img, cn)
        self.cn = cn
        self.ih, self.iw = planes[0].shape
        # the FFT size only has to cover the frame (valid outputs never wrap)
        self.shape = (_next_fast(self.ih + pad[0], True), _next_fast(self.iw + pad[1], True))
        self.spec = [_rfft2((p - 128).astype(np.float64), self.shape) for p in planes]
        self.sat = [_sat(p) for p in planes]
        self.sat2 = _sat(sum(p * p for p in planes))

    def match(self, tpl: np.ndarray) -> np.ndarray:
        tp = _planes(tpl, self.cn)
        th, tw = tp[0].shape
        rh, rw = self.ih - th + 1, self.iw - tw + 1
        area = th * tw
        inv_area = 1.0 / float(area)
        # template statistics exactly as refMatch forms them
        templ_norm = 0.0
        sums = []
        for p in tp:
            s, s2 = float(p.sum()), float((p * p).sum())
            mean = s * inv_area
            templ_norm += s2 * inv_area - mean * mean
            sums.append(int(p.sum()))
        if templ_norm < 2.220446049250313e-16:
            return np.ones((rh, rw), np.float64)
        templ_norm = np.sqrt(templ_norm * area)
        # numerator: frame - 128 correlated with area*T - sum(T), channels summed in frequency
        acc = None
        for k, p in enumerate(tp):
            z = (p * area - sums[k]).astype(np.float64)
            prod = self.spec[k] * np.conj(_rfft2(z, self.shape))
            acc = prod if acc is None else acc + prod
        corr = _irfft2(acc, self.shape)[:rh, :rw]
        num = corr * inv_area
        # denominator: exact window sums, refMatch's float64 sequence
        wm2 = np.zeros((rh, rw), np.float64)
        for k in range(self.cn):
            ws = _window(self.sat[k], th, tw, rh, rw).astype(np.float64)
            wm2 += ws * ws
        wsum2 = _window(self.sat2, th, tw, rh, rw).astype(np.float64)
        wm2 *= inv_area
        diff2 = np.maximum(wsum2 - wm2, 0.0)
        lim = np.minimum(FLT_EPS10 * wsum2, 0.5)
        den = np.where(diff2 > lim, np.sqrt(diff2) * templ_norm, 0.0)
        a = np.abs(num)
        with np.errstate(divide="ignore", invalid="ignore"):
            q = num / den
        return np.where(a < den, q, np.where(a < den * 1.125, np.copysign(1.0, num), 0.0))


def ref_match_f64(img: np.ndarray, tpl: np.ndarray, cn: int) -> np.ndarray:
    """The FP64 TM_CCOEFF_NORMED map of tpl over img (refMatch's definition)."""
    return Frame(img, cn).match(tpl)


def top2_margin(m: np.ndarray, which: str = "max") -> float:
    """Distance from the map's extremum to its next-best value (over every
    other position): the margin above which the extremum's location is
    determined at a given tolerance."""
    flat = np.asarray(m, np.float64).ravel()
    if flat.size < 2:
        return float("inf")
    if which == "max":
        i = int(np.argmax(flat))
        return float(flat[i] - np.max(np.delete(flat, i)))
    i = int(np.argmin(flat))
    return float(np.min(np.delete(flat, i)) - flat[i])


def first_argmax(m: np.ndarray):
    """(x, y) of the first maximum in raster order."""
    y, x = np.unravel_index(int(np.argmax(m)), m.shape)
    return int(x), int(y)


def first_argmin(m: np.ndarray):
    y, x = np.unravel_index(int(np.argmin(m)), m.shape)
    return int(x), int(y)


def check_extrema(got, m64: np.ndarray, tol: float, ref_map=None, name: str = "", off=(0, 0)):
    """A result six-tuple (minV, minX, minY, maxV, maxX, maxY) against the
    FP64 map m64 of the same positions: both extrema within tol of the FP64
    extrema, and each location equal to the FP64 map's first-occurrence
    location wherever that map's top-2 margin exceeds tol -- and equal to
    the reference's (ref_map, the reference's own float32 map, when given)
    wherever the reference map's margin does.  off: the map's origin in the
    result's coordinates (a region of interest).  Returns the larger value
    error."""
    min_v, min_x, min_y, max_v, max_x, max_y = (float(got[0]), int(got[1]), int(got[2]), float(got[3]),
                                                int(got[4]), int(got[5]))
    mx, mn = float(m64.max()), float(m64.min())
    e_max, e_min = abs(max_v - mx), abs(min_v - mn)
    at_max, at_min = (max_x - off[0], max_y - off[1]), (min_x - off[0], min_y - off[1])
    print(f"\n{name}: |max err| {e_max:.2e}  |min err| {e_min:.2e}  margins fp64 "
          f"{top2_margin(m64, 'max'):.1e}/{top2_margin(m64, 'min'):.1e}")
    assert e_max <= tol and e_min <= tol, (name, e_max, e_min)
    for m, what in ((m64, "fp64"), (ref_map, "reference")):
        if m is None:
            continue
        if top2_margin(m, "max") > tol:
            assert at_max == first_argmax(m), (name, what, "max", at_max, first_argmax(m))
        if top2_margin(m, "min") > tol:
            assert at_min == first_argmin(m), (name, what, "min", at_min, first_argmin(m))
    return max(e_max, e_min)
