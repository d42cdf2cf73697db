"""cvmatch_gb300 -- GB300 (sm_103a) TM_CCOEFF_NORMED template matching.

The host-side mirror of cvmatch's public Go API over the C ABI in
include/cvmatch_gpu.h (library: cvmatch_gb300/_build/libcvmatch_gpu.so):

    Match(parent, sub)          -> (minV, minX, minY, maxV, maxX, maxY)   cvmatch.go:75
    MatchMap(parent, sub)       -> (res, w, h)                            cvmatch.go:100
    MatchGray(parent, sub)      -> six-tuple                              cvmatch.go:128
    NewMatcher(sub) / NewGrayMatcher(sub) -> Matcher; Matcher.Find(parent) matcher.go:45-130
    NewFleet(*matchers) -> Fleet; Fleet.FindAll(parent) -> [Result]        fleet.go:85-332

Images are numpy uint8 arrays: H x W x 4 for RGBA (the *image.RGBA case),
H x W for 8-bit gray (the *image.Gray / YCbCr Y-plane case).  Row strides
are honoured, so a numpy slice is a sub-image exactly like
image.RGBA.SubImage.  Argument errors raise CvmatchError carrying the
reference's panic text.  There is no CPU path: every call runs the CUDA
library, and a missing library or device raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from collections import namedtuple

import numpy as np

__all__ = ["Match", "MatchMap", "MatchGray", "NewMatcher", "NewGrayMatcher", "NewFleet", "Matcher",
           "Fleet", "NewStream", "Stream", "MatchMapPeaks", "Result", "CvmatchError", "Threads", "Impl", "rgba_to_gray", "alpha_const",
           "match_u8", "library_path", "lib"]

# The Go package's knobs, kept for API compatibility.  The GPU path has no
# worker count: Threads is accepted and ignored (results never depended on
# it, threads_test.go:62-81).
Threads = 0
Impl = "gb300"

Result = namedtuple("Result", ["MinV", "MinX", "MinY", "MaxV", "MaxX", "MaxY"])


class CvmatchError(ValueError):
    """A call the reference would answer with a panic (the message is the
    reference's panic text), or a CUDA failure (code CVM_ERR_CUDA)."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class _CResult(C.Structure):
    _fields_ = [("min_v", C.c_float), ("min_x", C.c_int32), ("min_y", C.c_int32),
                ("max_v", C.c_float), ("max_x", C.c_int32), ("max_y", C.c_int32)]

    def tuple(self):
        return (self.min_v, self.min_x, self.min_y, self.max_v, self.max_x, self.max_y)


_HERE = os.path.dirname(os.path.abspath(__file__))
_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return os.path.join(_HERE, "_build", "libcvmatch_gpu.so")


def lib():
    """Loads the CUDA library, compiling it first when it is missing or
    older than its sources (the same nvcc build __graft_entry__.build runs)."""
    global _lib
    with _lock:
        if _lib is None:
            from . import build as _build
            path = _build.build()
            L = C.CDLL(path)
            vp, i32, i64, u8p = C.c_void_p, C.c_int, C.c_int64, C.c_void_p
            R = C.POINTER(_CResult)
            L.cvm_last_error.argtypes = [C.c_char_p, C.c_size_t]
            L.cvm_last_error.restype = C.c_size_t
            img_args = [u8p, i64, i32, i32, u8p, i64, i32, i32]
            L.cvm_match.argtypes = img_args + [R]
            L.cvm_match_map.argtypes = img_args + [vp]
            L.cvm_match_gray.argtypes = img_args + [R]
            L.cvm_match_gray_rgba.argtypes = img_args + [R]
            L.cvm_match_u8.argtypes = img_args + [i32, i32, vp, R]
            L.cvm_match_u8_device.argtypes = img_args + [i32, i32, vp, vp, vp]
            L.cvm_match_map_peaks.argtypes = img_args + [C.c_float, i32, i32, vp, i32, C.POINTER(C.c_int32)]
            L.cvm_match_u8_peaks.argtypes = img_args + [i32, i32, C.c_float, i32, i32, vp, i32, C.POINTER(C.c_int32)]
            L.cvm_peaks_device.argtypes = [vp, i32, i32, C.c_float, i32, i32, vp, i32, vp, vp]
            L.cvm_match_device.argtypes = img_args + [vp, vp, vp]
            L.cvm_rgba_to_gray.argtypes = [u8p, i64, i32, i32, vp]
            L.cvm_rgba_to_gray_device.argtypes = [u8p, i64, i32, i32, vp, i64, vp]
            L.cvm_alpha_const.argtypes = [u8p, i64, i32, i32, C.POINTER(C.c_int)]
            L.cvm_matcher_new.argtypes = [u8p, i64, i32, i32, i32, C.POINTER(vp)]
            L.cvm_matcher_find.argtypes = [vp, u8p, i64, i32, i32, R]
            L.cvm_matcher_find_device.argtypes = [vp, u8p, i64, i32, i32, vp, vp]
            L.cvm_matcher_free.argtypes = [vp]
            L.cvm_matcher_free.restype = None
            L.cvm_fleet_new.argtypes = [C.POINTER(vp), i32, C.POINTER(vp)]
            L.cvm_fleet_find_all.argtypes = [vp, u8p, i64, i32, i32, vp]
            L.cvm_fleet_find_all_device.argtypes = [vp, u8p, i64, i32, i32, vp, vp]
            L.cvm_fleet_free.argtypes = [vp]
            L.cvm_fleet_free.restype = None
            L.cvm_fleet_set_roi.argtypes = [vp, i32, i32, i32, i32, i32]
            L.cvm_fleet_set_form.argtypes = [vp, i32]
            L.cvm_fleet_buckets.argtypes = [vp, i32, i32, vp, i32]
            L.cvm_fleet_set_wave.argtypes = [vp, i32]
            L.cvm_fleet_set_overlap.argtypes = [vp, i32]
            L.cvm_fleet_set_stats.argtypes = [vp, i32]
            L.cvm_fleet_bucket_members.argtypes = [vp, i32, vp, i32]
            L.cvm_set_form.argtypes = [i32]
            L.cvm_get_form.argtypes = []
            L.cvm_set_autotune.argtypes = [i32]
            L.cvm_autotune_report.argtypes = [C.c_char_p, C.c_size_t]
            L.cvm_autotune_report.restype = C.c_size_t
            L.cvm_tc_selftest.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.cvm_device_status.argtypes = [C.POINTER(C.c_int)]
            L.cvm_stream_new.argtypes = [vp, vp, i32, i32, C.POINTER(vp)]
            L.cvm_stream_push.argtypes = [vp, u8p, i64]
            L.cvm_stream_pull.argtypes = [vp, vp, vp, C.POINTER(C.c_double)]
            L.cvm_stream_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
            L.cvm_stream_free.argtypes = [vp]
            L.cvm_stream_free.restype = None
            L.cvm_host_alloc.argtypes = [C.c_size_t]
            L.cvm_host_alloc.restype = vp
            L.cvm_host_free.argtypes = [vp]
            L.cvm_host_free.restype = None
            L.cvm_launch_count.restype = C.c_uint64
            L.cvm_version.restype = C.c_char_p
            _lib = L
    return _lib


def _check(rc: int):
    if rc != 0:
        buf = C.create_string_buffer(1024)
        lib().cvm_last_error(buf, len(buf))
        raise CvmatchError(rc, buf.value.decode(errors="replace"))


def _view(img, channels: int):
    """(pointer, byte stride, width, height) of an image array."""
    if img is None:
        raise CvmatchError(5, "cvmatch: nil image")
    a = np.asarray(img)
    if a.dtype != np.uint8:
        raise TypeError("cvmatch_gb300: images are uint8 arrays")
    if channels == 4:
        if a.ndim != 3 or a.shape[2] != 4:
            raise TypeError("cvmatch_gb300: RGBA images are H x W x 4 arrays")
        ok = a.strides[2] == 1 and a.strides[1] == 4
    else:
        if a.ndim != 2:
            raise TypeError("cvmatch_gb300: gray images are H x W arrays")
        ok = a.strides[1] == 1
    h, w = a.shape[0], a.shape[1]
    if h == 0 or w == 0:
        raise CvmatchError(6, "cvmatch: empty image")
    if not ok or a.strides[0] < w * channels:
        a = np.ascontiguousarray(a)
    return a, a.ctypes.data, a.strides[0], w, h


def _is_rgba(img) -> bool:
    a = np.asarray(img)
    return a.ndim == 3 and a.shape[2] == 4


def Match(parent, sub):
    """Match (cvmatch.go:75-94): RGBA TM_CCOEFF_NORMED min/max locations."""
    pa, pp, ps, pw, ph = _view(parent, 4)
    sa, sp, ss, sw, sh = _view(sub, 4)
    r = _CResult()
    _check(lib().cvm_match(pp, ps, pw, ph, sp, ss, sw, sh, C.byref(r)))
    return r.tuple()


def MatchMap(parent, sub):
    """MatchMap (cvmatch.go:100-117): the full response map (rows x cols)."""
    pa, pp, ps, pw, ph = _view(parent, 4)
    sa, sp, ss, sw, sh = _view(sub, 4)
    w, h = pw - sw + 1, ph - sh + 1
    res = np.empty((max(h, 1), max(w, 1)), np.float32)
    _check(lib().cvm_match_map(pp, ps, pw, ph, sp, ss, sw, sh, res.ctypes.data))
    return res, w, h


def MatchMapPeaks(parent, sub, thresh: float, rx: int, ry: int, max_peaks: int = 4096):
    """Every occurrence by the MatchMap recipe (cvmatch_test.go:324-381):
    scores >= thresh that no neighbour within +-rx columns / +-ry rows
    exceeds, in raster order, computed on the device.  Returns (list of
    (x, y) up to max_peaks, total count)."""
    pa, pp, ps, pw, ph = _view(parent, 4)
    sa, sp, ss, sw, sh = _view(sub, 4)
    xy = np.empty((max(max_peaks, 1), 2), np.int32)
    cnt = C.c_int32()
    _check(lib().cvm_match_map_peaks(pp, ps, pw, ph, sp, ss, sw, sh, float(thresh), rx, ry, xy.ctypes.data,
                                     max_peaks, C.byref(cnt)))
    n = min(cnt.value, max_peaks)
    return [(int(x), int(y)) for x, y in xy[:n]], cnt.value


def rgba_to_gray(img) -> np.ndarray:
    """rgbToGray (cvmatch.go:222-240) on the device."""
    a, p, s, w, h = _view(img, 4)
    out = np.empty((h, w), np.uint8)
    _check(lib().cvm_rgba_to_gray(p, s, w, h, out.ctypes.data))
    return out


def alpha_const(img) -> bool:
    """alphaConst (cvmatch.go:146-168) on the device."""
    a, p, s, w, h = _view(img, 4)
    v = C.c_int()
    _check(lib().cvm_alpha_const(p, s, w, h, C.byref(v)))
    return bool(v.value)


def _gray(img):
    return rgba_to_gray(img) if _is_rgba(img) else img


def MatchGray(parent, sub):
    """MatchGray (cvmatch.go:128-139): gray planes are used as they are,
    RGBA inputs are converted with OpenCV's fixed-point weights."""
    r = _CResult()
    if _is_rgba(parent) and _is_rgba(sub):
        pa, pp, ps, pw, ph = _view(parent, 4)
        sa, sp, ss, sw, sh = _view(sub, 4)
        _check(lib().cvm_match_gray_rgba(pp, ps, pw, ph, sp, ss, sw, sh, C.byref(r)))
        return r.tuple()
    pa, pp, ps, pw, ph = _view(_gray(parent), 1)
    sa, sp, ss, sw, sh = _view(_gray(sub), 1)
    _check(lib().cvm_match_gray(pp, ps, pw, ph, sp, ss, sw, sh, C.byref(r)))
    return r.tuple()


def match_u8(img, tpl, cn: int, want_map: bool = True):
    """matchU8 (impl.go:1126-1155) on raw views: img/tpl are H x W (step 1)
    or H x W x step arrays; returns (six-tuple, map or None)."""
    img = np.asarray(img)
    tpl = np.asarray(tpl)
    step = 1 if img.ndim == 2 else img.shape[2]
    tstep = 1 if tpl.ndim == 2 else tpl.shape[2]
    if step != tstep:
        raise CvmatchError(1, "cvmatch_gb300: image and template steps differ")
    ia = np.ascontiguousarray(img) if (img.ndim == 3 and img.strides[1] != step) or img.strides[-1] != 1 else img
    ta = np.ascontiguousarray(tpl) if (tpl.ndim == 3 and tpl.strides[1] != step) or tpl.strides[-1] != 1 else tpl
    ih, iw = ia.shape[0], ia.shape[1]
    th, tw = ta.shape[0], ta.shape[1]
    rw, rh = iw - tw + 1, ih - th + 1
    res = np.empty((rh, rw), np.float32) if want_map and rw > 0 and rh > 0 else None
    r = _CResult()
    _check(lib().cvm_match_u8(ia.ctypes.data, ia.strides[0], iw, ih, ta.ctypes.data, ta.strides[0], tw, th,
                              cn, step, res.ctypes.data if res is not None else None, C.byref(r)))
    return r.tuple(), res


class Matcher:
    """A prepared template (matcher.go:25-40).  Find is bit-identical to
    Match (colour) or MatchGray (gray) on the same parent."""

    def __init__(self, sub, step: int):
        self._step = step
        a, p, s, w, h = _view(sub, step)
        h_ = C.c_void_p()
        _check(lib().cvm_matcher_new(p, s, w, h, step, C.byref(h_)))
        self._h = h_
        self.w, self.h = w, h

    def Find(self, parent):
        if self._step == 1:
            parent = _gray(parent)
        a, p, s, w, h = _view(parent, self._step)
        r = _CResult()
        _check(lib().cvm_matcher_find(self._h, p, s, w, h, C.byref(r)))
        return r.tuple()

    def find_device(self, d_parent: int, pstride: int, pw: int, ph: int, d_out: int, stream: int = 0):
        """Queues Find on a device-resident parent; writes one result struct
        (24 bytes) at d_out.  Pointers are raw device addresses."""
        _check(lib().cvm_matcher_find_device(self._h, d_parent, pstride, pw, ph, d_out, stream or None))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.cvm_matcher_free(h)
            self._h = None


def NewMatcher(sub) -> Matcher:
    """NewMatcher (matcher.go:45-53): colour, Match semantics."""
    return Matcher(sub, 4)


def NewGrayMatcher(sub) -> Matcher:
    """NewGrayMatcher (matcher.go:57-64): MatchGray semantics."""
    return Matcher(_gray(sub), 1)


FORM_EXACT = 0
FORM_FAST = 1
FORM_MIXED = 2
STATS_KERNEL = 0
STATS_EPILOGUE = 1


def SetAutotune(on: bool) -> bool:
    """The fast forms' tile-plan autotuner on or off (cvm_set_autotune);
    returns the previous setting."""
    return bool(lib().cvm_set_autotune(1 if on else 0))


def autotune_report():
    """The tuned shapes and their measured candidate plans (list of dicts)."""
    import json
    n = lib().cvm_autotune_report(None, 0)
    buf = C.create_string_buffer(n + 1)
    lib().cvm_autotune_report(buf, n + 1)
    return json.loads(buf.value.decode())


def tc_selftest():
    """(dft error, first-stage GEMM error) of the tensor-core DFT path on
    this device, relative to each line's norm (cvm_tc_selftest)."""
    a, b = C.c_double(), C.c_double()
    _check(lib().cvm_tc_selftest(C.byref(a), C.byref(b)))
    return a.value, b.value


def device_status() -> int:
    """1 when a tensor-core kernel gave up waiting since the last call."""
    v = C.c_int()
    _check(lib().cvm_device_status(C.byref(v)))
    return v.value


def SetForm(form: int) -> int:
    """Arithmetic of one-shot matches and Matcher.Find, process-wide
    (cvm_set_form): FORM_EXACT (default, the reference's bits), FORM_FAST,
    or FORM_MIXED (the fast form with its 1024-point inverse row transforms
    on the tensor cores).  Returns the previous form."""
    prev = lib().cvm_get_form()
    _check(lib().cvm_set_form(form))
    return prev


class Fleet:
    """Many prepared matchers against one frame (fleet.go:19-50)."""

    def __init__(self, ms):
        if len(ms) == 0:
            raise CvmatchError(3, "cvmatch: empty fleet")
        self._ms = list(ms)  # keeps the member handles alive (fleet.go:89-92)
        arr = (C.c_void_p * len(ms))(*[m._h.value for m in ms])
        h_ = C.c_void_p()
        _check(lib().cvm_fleet_new(arr, len(ms), C.byref(h_)))
        self._h = h_
        self._step = ms[0]._step

    def FindAll(self, parent):
        if self._step == 1:
            parent = _gray(parent)
        a, p, s, w, h = _view(parent, self._step)
        out = (_CResult * len(self._ms))()
        _check(lib().cvm_fleet_find_all(self._h, p, s, w, h, out))
        return [Result(*o.tuple()) for o in out]

    def find_all_device(self, d_parent: int, pstride: int, pw: int, ph: int, d_out: int, stream: int = 0):
        _check(lib().cvm_fleet_find_all_device(self._h, d_parent, pstride, pw, ph, d_out, stream or None))

    def SetROI(self, member: int, x: int, y: int, w: int, h: int):
        """Restrict member (construction order) to a region of interest in
        frame pixels; w or h <= 0 clears it (see cvm_fleet_set_roi)."""
        _check(lib().cvm_fleet_set_roi(self._h, member, x, y, w, h))

    def SetForm(self, form: int):
        """FORM_EXACT (default: the reference's float32 arithmetic, bit for
        bit), FORM_MIXED (FORM_FAST with its 1024-point inverse rows on the
        tensor cores) or FORM_FAST (zero-mean templates, channels summed in the
        frequency domain; see cvm_fleet_set_form)."""
        _check(lib().cvm_fleet_set_form(self._h, form))

    def SetWave(self, members: int):
        """At most `members` member tails per wave (0: by the workspace
        budget); see cvm_fleet_set_wave."""
        _check(lib().cvm_fleet_set_wave(self._h, members))

    def SetOverlap(self, on: bool):
        """Overlapped waves of member tails (on, the default) or every wave
        in sequence; see cvm_fleet_set_overlap."""
        _check(lib().cvm_fleet_set_overlap(self._h, 1 if on else 0))

    def SetStats(self, mode: int):
        """STATS_KERNEL (the default: the statistics kernel) or
        STATS_EPILOGUE (window statistics inside the inverse-rows epilogue
        from the frame's summed-area table, where it applies); the results
        are the same bits.  See cvm_fleet_set_stats."""
        _check(lib().cvm_fleet_set_stats(self._h, mode))

    def buckets(self, pw: int, ph: int):
        """[(tw, th, dftW, dftH, blockW, blockH, dh2, tiles, members)] per
        bucket on a pw x ph frame (bucketize + the bucket plans)."""
        n = lib().cvm_fleet_buckets(self._h, pw, ph, None, 0)
        if n < 0:
            _check(-n)
        out = (C.c_int32 * (9 * max(n, 1)))()
        lib().cvm_fleet_buckets(self._h, pw, ph, out, n)
        return [tuple(out[9 * b:9 * b + 9]) for b in range(n)]

    def bucket_members(self, b: int):
        """Construction-order indices of bucket b's members."""
        n = lib().cvm_fleet_bucket_members(self._h, b, None, 0)
        if n < 0:
            _check(-n)
        out = (C.c_int32 * max(n, 1))()
        lib().cvm_fleet_bucket_members(self._h, b, out, n)
        return list(out[:n])

    def __len__(self):
        return len(self._ms)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.cvm_fleet_free(h)
            self._h = None


def NewFleet(*ms) -> Fleet:
    """NewFleet (fleet.go:85-101)."""
    if len(ms) == 1 and isinstance(ms[0], (list, tuple)):
        ms = tuple(ms[0])
    return Fleet(ms)


class Stream:
    """A stream of equal-size RGBA frames matched against a colour fleet and
    optionally a gray fleet on each frame's gray conversion; the per-frame
    pipeline replays as a CUDA graph, and two frames may be in flight.
    Results equal Fleet.FindAll per frame."""

    def __init__(self, color: Fleet, gray, pw: int, ph: int):
        self._color, self._gray = color, gray  # the fleets must outlive the stream
        h_ = C.c_void_p()
        _check(lib().cvm_stream_new(color._h, gray._h if gray is not None else None, pw, ph, C.byref(h_)))
        self._h = h_
        self._pw, self._ph = pw, ph

    def push(self, frame):
        a, p, s, w, h = _view(frame, 4)
        if (w, h) != (self._pw, self._ph):
            raise CvmatchError(1, "cvmatch_gpu: frame size differs from the stream's")
        _check(lib().cvm_stream_push(self._h, p, s))

    def pull(self):
        """(colour results, gray results, device ms) of the oldest frame."""
        nc, ng = len(self._color), len(self._gray) if self._gray is not None else 0
        oc, og = (_CResult * nc)(), (_CResult * max(ng, 1))()
        ms = C.c_double()
        _check(lib().cvm_stream_pull(self._h, oc, og if ng else None, C.byref(ms)))
        return [Result(*o.tuple()) for o in oc], [Result(*o.tuple()) for o in og[:ng]], ms.value

    def info(self):
        """(graphed, kernel launches per frame)."""
        g, n = C.c_int(), C.c_int()
        _check(lib().cvm_stream_info(self._h, C.byref(g), C.byref(n)))
        return bool(g.value), n.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.cvm_stream_free(h)
            self._h = None


def NewStream(color: Fleet, gray, pw: int, ph: int) -> Stream:
    return Stream(color, gray, pw, ph)
