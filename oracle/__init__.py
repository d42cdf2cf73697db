"""ctypes binding of the CPU oracle (oracle/cvm_oracle.c).

TEST INFRASTRUCTURE ONLY: the oracle is the checker.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module;
the product package (cvmatch_gb300) never does.

The C file restates the reference's scalar Go path op for op; every
function here maps one-to-one onto an exported C function and names the
reference code it follows in that C function's comment.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libcvm_oracle.so")
_lock = threading.Lock()
_lib = None


class Result(C.Structure):
    _fields_ = [("min_v", C.c_float), ("min_x", C.c_int32), ("min_y", C.c_int32),
                ("max_v", C.c_float), ("max_x", C.c_int32), ("max_y", C.c_int32)]

    def tuple(self):
        return (self.min_v, self.min_x, self.min_y, self.max_v, self.max_x, self.max_y)


class Plan(C.Structure):
    _fields_ = [("dft_w", C.c_int32), ("dft_h", C.c_int32), ("hw", C.c_int32),
                ("block_w", C.c_int32), ("block_h", C.c_int32), ("cost", C.c_int64)]


class Member(C.Structure):
    _fields_ = [("pix", C.c_void_p), ("stride", C.c_int64), ("w", C.c_int32), ("h", C.c_int32)]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    src = os.path.join(_HERE, "cvm_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB_PATH)
            vp, i32, i64 = C.c_void_p, C.c_int, C.c_int64
            L.cvo_plan_make.argtypes = [i32, i32, i32, i32, C.POINTER(Plan)]
            L.cvo_shrink_dh.argtypes = [C.POINTER(Plan), i32, i32]
            L.cvo_stats_cap.argtypes = [i32]
            L.cvo_stats_cap.restype = i64
            L.cvo_sincospi.argtypes = [i32, i32, C.POINTER(C.c_float), C.POINTER(C.c_float)]
            L.cvo_tri_twiddles.argtypes = [i32, vp]
            L.cvo_fft_r4.argtypes = [vp, i32, i32]
            L.cvo_cols_r4.argtypes = [vp, i32, i32, i32, i32]
            L.cvo_rgba_to_gray.argtypes = [vp, i64, i32, i32, vp]
            L.cvo_alpha_const.argtypes = [vp, i64, i32, i32]
            L.cvo_templ_stats.argtypes = [vp, i64, i32, i32, i32, i32, vp, C.POINTER(C.c_int64)]
            L.cvo_match_u8.argtypes = [vp, i64, i32, i32, vp, i64, i32, i32, i32, i32, i32, vp,
                                       C.POINTER(Result), C.c_char_p]
            L.cvo_cross_corr.argtypes = [vp, i64, i32, i32, vp, i64, i32, i32, i32, i32, i32, vp]
            L.cvo_normalize.argtypes = [vp, i64, i32, i32, i32, i32, i32, i32, vp, i64, i32, vp, vp,
                                        C.POINTER(Result)]
            L.cvo_bucketize.argtypes = [C.POINTER(Member), i32, i32, vp, vp, vp, vp]
            L.cvo_fleet_find_all.argtypes = [C.POINTER(Member), i32, i32, vp, i64, i32, i32, i32,
                                             C.POINTER(Result), C.c_char_p]
            L.cvo_fleet_find_all_maps.argtypes = [C.POINTER(Member), i32, i32, vp, i64, i32, i32, i32,
                                                  C.POINTER(Result), vp, C.c_char_p]
            L.cvo_fleet_find_all_sel.argtypes = [C.POINTER(Member), i32, i32, vp, i64, i32, i32, i32, vp,
                                                 C.POINTER(Result), vp, vp, C.c_char_p]
            L.cvo_ref_match_f64.argtypes = [vp, i64, i32, i32, vp, i64, i32, i32, i32, i32, i32, vp]
            _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class OraclePanic(ValueError):
    """The reference would panic with this message."""


def plan(tw, th, rw, rh):
    p = Plan()
    lib().cvo_plan_make(tw, th, rw, rh, C.byref(p))
    return p


def shrink_dh(p: Plan, rh: int, th: int) -> int:
    return lib().cvo_shrink_dh(C.byref(p), rh, th)


def stats_cap(cn: int) -> int:
    return lib().cvo_stats_cap(cn)


def tri_twiddles(n: int) -> np.ndarray:
    cnt = lib().cvo_tri_twiddles(n, None)
    out = np.zeros(max(cnt, 1) * 2, np.float32)
    lib().cvo_tri_twiddles(n, _ptr(out))
    return out[: 2 * cnt].view(np.complex64)


def fft_r4(a: np.ndarray, inverse: bool) -> np.ndarray:
    a = np.ascontiguousarray(a, np.complex64).copy()
    lib().cvo_fft_r4(_ptr(a), a.size, int(inverse))
    return a


def cols_r4(d: np.ndarray, inverse: bool, use_rmap: bool) -> np.ndarray:
    d = np.ascontiguousarray(d, np.complex64).copy()
    lib().cvo_cols_r4(_ptr(d), d.shape[0], d.shape[1], int(inverse), int(use_rmap))
    return d


def _view(img: np.ndarray):
    """(base array, byte stride, width, height, step) of an HxW or HxWxC uint8 view."""
    if img.dtype != np.uint8:
        raise TypeError("uint8 image expected")
    if img.ndim == 2:
        step = 1
    else:
        step = img.shape[2]
    if img.strides[-1] != 1 or (img.ndim == 3 and img.strides[1] != step):
        raise ValueError("pixels of a row must be contiguous")
    return img, img.strides[0], img.shape[1], img.shape[0], step


def rgba_to_gray(img: np.ndarray) -> np.ndarray:
    a, stride, w, h, step = _view(img)
    assert step == 4
    out = np.empty((h, w), np.uint8)
    lib().cvo_rgba_to_gray(_ptr(a), stride, w, h, _ptr(out))
    return out


def alpha_const(img: np.ndarray) -> bool:
    a, stride, w, h, step = _view(img)
    assert step == 4
    return bool(lib().cvo_alpha_const(_ptr(a), stride, w, h))


def templ_stats(tpl: np.ndarray, cn: int):
    a, stride, w, h, step = _view(tpl)
    ts = np.zeros(4, np.int64)
    vs = C.c_int64()
    lib().cvo_templ_stats(_ptr(a), stride, w, h, cn, step, _ptr(ts), C.byref(vs))
    return ts, vs.value


def match_u8(img: np.ndarray, tpl: np.ndarray, cn: int, threads: int = 1, want_map: bool = True):
    """matchU8 on two uint8 views sharing one step; returns (tuple, map or None)."""
    a, istride, iw, ih, step = _view(img)
    b, tstride, tw, th, tstep = _view(tpl)
    if step != tstep:
        raise ValueError("image and template steps differ")
    rw, rh = iw - tw + 1, ih - th + 1
    res = np.empty((max(rh, 0), max(rw, 0)), np.float32) if want_map and rw > 0 and rh > 0 else None
    out = Result()
    err = C.create_string_buffer(256)
    rc = lib().cvo_match_u8(_ptr(a), istride, iw, ih, _ptr(b), tstride, tw, th, cn, step, threads,
                            _ptr(res) if res is not None else None, C.byref(out), err)
    if rc != 0:
        raise OraclePanic(err.value.decode())
    return out.tuple(), res


def cross_corr(img: np.ndarray, tpl: np.ndarray, cn: int, threads: int = 1) -> np.ndarray:
    a, istride, iw, ih, step = _view(img)
    b, tstride, tw, th, _ = _view(tpl)
    res = np.empty((ih - th + 1, iw - tw + 1), np.float32)
    rc = lib().cvo_cross_corr(_ptr(a), istride, iw, ih, _ptr(b), tstride, tw, th, cn, step, threads, _ptr(res))
    if rc != 0:
        raise OraclePanic("bad arguments")
    return res


def normalize(img: np.ndarray, tw: int, th: int, cn: int, tsum, var_sum: int, corr: np.ndarray,
              threads: int = 1):
    a, istride, iw, ih, step = _view(img)
    ts = np.ascontiguousarray(tsum, np.int64)
    corr = np.ascontiguousarray(corr, np.float32)
    res = np.empty_like(corr)
    out = Result()
    lib().cvo_normalize(_ptr(a), istride, iw, ih, tw, th, cn, step, _ptr(ts), var_sum, threads,
                        _ptr(corr), _ptr(res), C.byref(out))
    return out.tuple(), res


def _members(tpls):
    ms = (Member * len(tpls))()
    step = None
    for i, t in enumerate(tpls):
        a, stride, w, h, s = _view(t)
        step = s if step is None else step
        ms[i].pix, ms[i].stride, ms[i].w, ms[i].h = _ptr(a), stride, w, h
    return ms, step


def bucketize(tpls):
    """bucketize over templates; returns [(tw, th, [member indices]), ...]."""
    ms, step = _members(tpls)
    n = len(tpls)
    tw = np.zeros(max(n, 1), np.int32)
    th = np.zeros(max(n, 1), np.int32)
    offs = np.zeros(n + 1, np.int32)
    mem = np.zeros(max(n, 1), np.int32)
    nb = lib().cvo_bucketize(ms, n, step or 4, _ptr(tw), _ptr(th), _ptr(offs), _ptr(mem))
    return [(int(tw[b]), int(th[b]), [int(m) for m in mem[offs[b]:offs[b + 1]]]) for b in range(nb)]


def fleet_find_all(tpls, parent: np.ndarray, threads: int = 1, want_maps: bool = False):
    """Fleet.FindAll; with want_maps also every member's score map on its
    bucket's plan (None for flat members): (results, maps)."""
    ms, step = _members(tpls)
    a, pstride, pw, ph, pstep = _view(parent)
    if len(tpls) and pstep != step:
        raise ValueError("parent step differs from the members'")
    out = (Result * max(len(tpls), 1))()
    err = C.create_string_buffer(256)
    maps = None
    mp = None
    if want_maps:
        maps = []
        for t in tpls:
            th, tw = np.asarray(t).shape[:2]
            maps.append(np.full((ph - th + 1, pw - tw + 1), np.nan, np.float32) if tw <= pw and th <= ph else None)
        mp = (C.c_void_p * max(len(tpls), 1))(*[m.ctypes.data if m is not None else None for m in maps])
    rc = lib().cvo_fleet_find_all_maps(ms, len(tpls), step or pstep, _ptr(a), pstride, pw, ph, threads, out, mp, err)
    if rc != 0:
        raise OraclePanic(err.value.decode())
    res = [out[i].tuple() for i in range(len(tpls))]
    if not want_maps:
        return res
    for i, r in enumerate(res):
        if maps[i] is not None and np.isnan(maps[i]).all():
            maps[i] = None  # flat member: no map (impl.go:1137-1144)
    return res, maps


def fleet_find_all_sel(tpls, parent: np.ndarray, want, threads: int = 1, want_maps: bool = False):
    """Fleet.FindAll of the whole fleet's buckets and plans, with the member
    tails run only for the members in `want` (indices, construction order):
    those members' results are bit-identical to the full FindAll's.
    Returns (results: {index: six-tuple}, maps: {index: map or None} or
    None, (phase-1 seconds, phase-2 seconds))."""
    ms, step = _members(tpls)
    a, pstride, pw, ph, pstep = _view(parent)
    if len(tpls) and pstep != step:
        raise ValueError("parent step differs from the members'")
    n = len(tpls)
    mask = np.zeros(max(n, 1), np.uint8)
    want = sorted(set(int(i) for i in want))
    mask[want] = 1
    out = (Result * max(n, 1))()
    err = C.create_string_buffer(256)
    maps, mp = None, None
    if want_maps:
        maps = {}
        for i in want:
            th, tw = np.asarray(tpls[i]).shape[:2]
            maps[i] = np.full((ph - th + 1, pw - tw + 1), np.nan, np.float32) if tw <= pw and th <= ph else None
        mp = (C.c_void_p * max(n, 1))(*[maps[i].ctypes.data if (i in maps and maps[i] is not None) else None
                                        for i in range(n)])
    phase = np.zeros(2, np.float64)
    rc = lib().cvo_fleet_find_all_sel(ms, n, step or pstep, _ptr(a), pstride, pw, ph, threads, _ptr(mask), out,
                                      mp, _ptr(phase), err)
    if rc != 0:
        raise OraclePanic(err.value.decode())
    res = {i: out[i].tuple() for i in want}
    if maps is not None:
        for i in want:
            if maps[i] is not None and np.isnan(maps[i]).all():
                maps[i] = None  # flat member: no map (impl.go:1137-1144)
    return res, maps, (float(phase[0]), float(phase[1]))


def ref_match_f64(img: np.ndarray, tpl: np.ndarray, cn: int, threads: int = 8) -> np.ndarray:
    a, istride, iw, ih, step = _view(img)
    b, tstride, tw, th, _ = _view(tpl)
    out = np.empty((ih - th + 1, iw - tw + 1), np.float64)
    lib().cvo_ref_match_f64(_ptr(a), istride, iw, ih, _ptr(b), tstride, tw, th, cn, step, threads, _ptr(out))
    return out


def fnv_golden_hash(res: np.ndarray, t) -> int:
    """goldenHash (impl_golden_test.go:27-44): FNV-1a 64 over the map's
    float32 bits (little-endian) then the six extrema fields."""
    min_v, min_x, min_y, max_v, max_x, max_y = t
    tail = np.array([np.float32(min_v).view(np.uint32), min_x & 0xFFFFFFFF, min_y & 0xFFFFFFFF,
                     np.float32(max_v).view(np.uint32), max_x & 0xFFFFFFFF, max_y & 0xFFFFFFFF],
                    dtype="<u4")
    data = np.ascontiguousarray(res, "<f4").tobytes() + tail.tobytes()
    h = 0xcbf29ce484222325
    prime = 0x100000001b3
    mask = 0xFFFFFFFFFFFFFFFF
    for byte in data:
        h ^= byte
        h = (h * prime) & mask
    return h
