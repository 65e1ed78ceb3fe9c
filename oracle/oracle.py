"""ctypes wrapper of the C oracle (amdat_oracle.c): TEST INFRASTRUCTURE ONLY.

Used by tests, the smoke check and the benchmark's CPU-baseline leg as the
checker; the engine never imports this module.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_oracle

REF32, F64 = 0, 1
LINEAR, EXPONENTIAL, SNAPSHOT = 0, 1, 2

_lib = None


class Scheme(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n_exponentials", C.c_int32),
                ("n_exponential_steps", C.c_int32), ("exp_base", C.c_float),
                ("frt", C.c_int32), ("first_exponent", C.c_int32),
                ("time_unit", C.c_float), ("limit", C.c_int32)]


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_oracle.build_lib())
        _lib.orc_pairs_list.restype = C.c_int64
        _lib.orc_pairs_loop.restype = C.c_int64
        _lib.orc_n_timesteps.restype = C.c_int32
        _lib.orc_n_timegaps.restype = C.c_int32
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def scheme(ts, limit: int = 0) -> Scheme:
    """Oracle scheme from an amdat_gb300.synth.TimeScheme."""
    s = Scheme()
    if ts.kind == "linear":
        lib().orc_scheme_init(C.byref(s), LINEAR, ts.n_timesteps, 1, C.c_float(1.0), 0, 0,
                              C.c_float(ts.time_unit))
    elif ts.kind == "exponential":
        lib().orc_scheme_init(C.byref(s), EXPONENTIAL, ts.n_exponentials, ts.n_exponential_steps,
                              C.c_float(ts.exp_base), ts.frt, ts.first_exponent,
                              C.c_float(ts.time_unit))
    else:
        lib().orc_scheme_init(C.byref(s), SNAPSHOT, 1, 0, C.c_float(1.0), 0, 0, C.c_float(1.0))
    s.limit = limit
    return s


def n_timegaps(s):
    return lib().orc_n_timegaps(C.byref(s))


def n_timesteps(s):
    return lib().orc_n_timesteps(C.byref(s))


def timelist(s):
    out = np.zeros(n_timesteps(s), np.float32)
    lib().orc_timelist(C.byref(s), _p(out))
    return out


def displacement_times(s):
    out = np.zeros(n_timegaps(s), np.float32)
    lib().orc_displacement_times(C.byref(s), _p(out))
    return out


def timegap_weighting(s, fullblock=0):
    out = np.zeros(n_timegaps(s), np.int32)
    lib().orc_timegap_weighting(C.byref(s), int(fullblock), _p(out))
    return out


def pairs(s, fullblock=0, loop_order=False):
    fn = lib().orc_pairs_loop if loop_order else lib().orc_pairs_list
    n = fn(C.byref(s), int(fullblock), None, None, None)
    g = np.zeros(max(n, 1), np.int32)
    a = np.zeros(max(n, 1), np.int32)
    b = np.zeros(max(n, 1), np.int32)
    fn(C.byref(s), int(fullblock), _p(g), _p(a), _p(b))
    return g[:n], a[:n], b[:n]


def _f32(x):
    return np.ascontiguousarray(x, dtype=np.float32)


def _i32(x):
    return np.ascontiguousarray(x, dtype=np.int32)


def msd(s, unwrapped, lst, mode=F64):
    u = _f32(unwrapped)
    lst = _i32(lst)
    out = np.zeros(n_timegaps(s))
    w = np.zeros(n_timegaps(s))
    lib().orc_msd(C.byref(s), _p(u), u.shape[1], _p(lst), len(lst), mode, _p(out), _p(w))
    return out


def ngp(s, unwrapped, lst, mode=F64):
    u = _f32(unwrapped)
    lst = _i32(lst)
    out = np.zeros(n_timegaps(s))
    lib().orc_ngp(C.byref(s), _p(u), u.shape[1], _p(lst), len(lst), mode, _p(out))
    return out


def disp_moments(s, unwrapped, lst=None, fullblock=0):
    u = _f32(unwrapped)
    G = n_timegaps(s)
    d2, d4, cnt = np.zeros(G), np.zeros(G), np.zeros(G, np.int64)
    if lst is None:
        lst = np.arange(u.shape[1], dtype=np.int32)
    lst = _i32(lst)
    lib().orc_disp_moments(C.byref(s), int(fullblock), _p(u), u.shape[1], _p(lst), len(lst),
                           _p(d2), _p(d4), _p(cnt))
    return d2, d4, cnt


def isfs(s, unwrapped, lst, kvec_n, shell_off, spacing, box_len, fullblock=0, mode=F64):
    u = _f32(unwrapped)
    lst = _i32(lst)
    kv = _i32(kvec_n).reshape(-1)
    off = _i32(shell_off)
    ns = len(off) - 1
    out = np.zeros((n_timegaps(s), ns))
    lib().orc_isfs(C.byref(s), int(fullblock), _p(u), u.shape[1], _p(lst), len(lst), _p(kv),
                   _p(off), ns, C.c_float(spacing), C.c_double(box_len), mode, _p(out))
    return out


def boxify(wrapped, lo, hi):
    """System::boxify on a copy of the wrapped coordinates [frames][atoms][3]."""
    w = np.array(wrapped, dtype=np.float32, order="C", copy=True)
    lo, hi = _f32(np.asarray(lo)), _f32(np.asarray(hi))
    lib().orc_boxify(_p(w), w.shape[0], w.shape[1], _p(lo), _p(hi))
    return w


def assign_bins(wrapped, nbins, lo, hi):
    """Trajectory_List_Bins::assign_bins: flat bin [frames][atoms] or -1."""
    w = _f32(wrapped)
    lo, hi = _f32(np.asarray(lo)), _f32(np.asarray(hi))
    out = np.empty(w.shape[:2], np.int32)
    lib().orc_assign_bins(_p(w), w.shape[0], w.shape[1], int(nbins[0]), int(nbins[1]), int(nbins[2]),
                          _p(lo), _p(hi), _p(out))
    return out


def msd_bins(s, unwrapped, lst, bins, n_bins, persistent=0, mode=F64):
    """Per-bin MSD: (msd [bins][gaps], weighting [bins][gaps])."""
    u = _f32(unwrapped)
    lst = _i32(lst)
    b = _i32(bins)
    G = n_timegaps(s)
    out = np.zeros((n_bins, G))
    w = np.zeros((n_bins, G))
    lib().orc_msd_bins(C.byref(s), _p(u), u.shape[1], _p(lst), len(lst), _p(b), int(n_bins),
                       int(persistent), mode, _p(out), _p(w))
    return out, w


def isfs_bins(s, unwrapped, lst, kvec_n, shell_off, spacing, box_len, bins, n_bins, fullblock=0,
              persistent=0, mode=F64):
    """Per-bin self-intermediate scattering function [bins][gaps][shells]."""
    u = _f32(unwrapped)
    lst = _i32(lst)
    kv = _i32(kvec_n).reshape(-1)
    off = _i32(shell_off)
    b = _i32(bins)
    ns = len(off) - 1
    out = np.zeros((n_bins, n_timegaps(s), ns))
    lib().orc_isfs_bins(C.byref(s), int(fullblock), _p(u), u.shape[1], _p(lst), len(lst), _p(kv), _p(off), ns,
                        C.c_float(spacing), C.c_double(box_len), _p(b), int(n_bins), int(persistent), mode,
                        _p(out))
    return out


def ngp_bins(s, unwrapped, lst, bins, n_bins, persistent=0, mode=F64):
    """Per-bin NGP (its MSD pass over the same members) [bins][gaps]."""
    u = _f32(unwrapped)
    lst = _i32(lst)
    b = _i32(bins)
    out = np.zeros((n_bins, n_timegaps(s)))
    lib().orc_ngp_bins(C.byref(s), _p(u), u.shape[1], _p(lst), len(lst), _p(b), int(n_bins), int(persistent),
                       mode, _p(out))
    return out


def msd2d_bins(s, unwrapped, lst, plane, bins, n_bins, persistent=0, mode=F64):
    """Per-bin Mean_Square_Displacement_2D [bins][gaps] (plane 0 = xy, 1 = xz, 2 = yz)."""
    u = _f32(unwrapped)
    lst = _i32(lst)
    b = _i32(bins)
    out = np.zeros((n_bins, n_timegaps(s)))
    lib().orc_msd2d_bins(C.byref(s), _p(u), u.shape[1], _p(lst), len(lst), int(plane), _p(b), int(n_bins),
                         int(persistent), mode, _p(out))
    return out


def mean_disp_bins(s, unwrapped, lst, bins, n_bins, persistent=0, mode=F64):
    """Per-bin Mean_Displacement [bins][gaps][3]."""
    u = _f32(unwrapped)
    lst = _i32(lst)
    b = _i32(bins)
    out = np.zeros((n_bins, n_timegaps(s), 3))
    lib().orc_mean_disp_bins(C.byref(s), _p(u), u.shape[1], _p(lst), len(lst), _p(b), int(n_bins),
                             int(persistent), mode, _p(out))
    return out


def fast_particles(s, unwrapped, lst, gap, min_u2):
    """Fast_Particles: (fast [blocks][atoms] 0/1, membership map [frames][atoms] 0/-1)."""
    u = _f32(unwrapped)
    lst = _i32(lst)
    fast = np.zeros((s.n_exponentials, u.shape[1]), np.int32)
    bins = np.zeros(u.shape[:2], np.int32)
    lib().orc_fast_particles(C.byref(s), _p(u), u.shape[1], _p(lst), len(lst), int(gap), C.c_float(min_u2),
                             _p(fast), _p(bins))
    return fast, bins


def vhs(s, unwrapped, lst, max_value, n_bins):
    u = _f32(unwrapped)
    lst = _i32(lst)
    G = n_timegaps(s)
    counts = np.zeros((G, n_bins), np.int64)
    w = np.zeros(G, np.int64)
    corr = np.zeros((G, n_bins))
    lib().orc_vhs(C.byref(s), _p(u), u.shape[1], _p(lst), len(lst), C.c_float(max_value),
                  n_bins, _p(counts), _p(w), _p(corr))
    return counts, w, corr


def rhok(wrapped, lst, frames, kvec_n, spacing, box_len, mode=F64):
    r = _f32(wrapped)
    lst = _i32(lst)
    fr = _i32(frames)
    kv = _i32(kvec_n).reshape(-1)
    nk = len(kv) // 3
    out = np.zeros((len(fr), nk, 2))
    lib().orc_rhok(_p(r), r.shape[1], _p(lst), len(lst), _p(fr), len(fr), _p(kv), nk,
                   C.c_float(spacing), C.c_double(box_len), mode, _p(out))
    return out


def isf(s, rho1, rho2, shell_off, n_list, fullblock=0, mode=F64):
    r1 = np.ascontiguousarray(rho1, np.float64)
    r2 = np.ascontiguousarray(rho2, np.float64)
    off = _i32(shell_off)
    ns = len(off) - 1
    out = np.zeros((n_timegaps(s), ns))
    lib().orc_isf(C.byref(s), int(fullblock), _p(r1), _p(r2), r1.shape[1], _p(off), ns, n_list,
                  mode, _p(out))
    return out


def structure_factor(s, timescheme, wrapped, lst, kvec_n, shell_off, spacing, box_len, mode=F64):
    r = _f32(wrapped)
    lst = _i32(lst)
    kv = _i32(kvec_n).reshape(-1)
    off = _i32(shell_off)
    ns = len(off) - 1
    out = np.zeros(ns)
    lib().orc_structure_factor(C.byref(s), int(timescheme), _p(r), r.shape[1], _p(lst), len(lst),
                               _p(kv), _p(off), ns, C.c_float(spacing), C.c_double(box_len), mode,
                               _p(out))
    return out


def onetime_frames(s, timescheme):
    T = n_timesteps(s)
    if timescheme == -1:
        return list(range(T))
    if timescheme < -1:
        return [-timescheme - 2]
    return list(range(timescheme, s.n_exponentials, s.n_exponential_steps))


def rdf(s, timescheme, wrapped, box, lst, n_bins, max_distance):
    r = _f32(wrapped)
    lst = _i32(lst)
    bx = _f32(box)
    nf = len(onetime_frames(s, timescheme))
    counts = np.zeros((nf, n_bins), np.int64)
    mean = np.zeros(n_bins)
    lib().orc_rdf(C.byref(s), int(timescheme), _p(r), r.shape[1], _p(bx), _p(lst), len(lst),
                  n_bins, C.c_float(max_distance), _p(counts), _p(mean))
    return counts, mean


def vhd(s, wrapped, box, lst, max_value, n_bins, fullblock=0):
    r = _f32(wrapped)
    lst = _i32(lst)
    bx = _f32(box)
    G = n_timegaps(s)
    counts = np.zeros((G, n_bins), np.int64)
    w = np.zeros(G, np.int64)
    lib().orc_vhd(C.byref(s), int(fullblock), _p(r), r.shape[1], _p(bx), _p(lst), len(lst),
                  C.c_float(max_value), n_bins, _p(counts), _p(w))
    return counts, w


def disp_fs_parallel(s, unwrapped, kvec_n, box_len, n_threads, fullblock=0):
    u = _f32(unwrapped)
    kv = _i32(kvec_n).reshape(-1)
    G = n_timegaps(s)
    d2, fs = np.zeros(G), np.zeros(G)
    lib().orc_disp_fs_parallel(C.byref(s), int(fullblock), _p(u), u.shape[1], _p(kv),
                               len(kv) // 3, C.c_double(box_len), int(n_threads), _p(d2), _p(fs))
    return d2, fs


def rhok_parallel(wrapped, frames, kvec_n, box_len, n_threads):
    r = _f32(wrapped)
    fr = _i32(frames)
    kv = _i32(kvec_n).reshape(-1)
    nk = len(kv) // 3
    out = np.zeros((len(fr), nk, 2))
    lib().orc_rhok_parallel(_p(r), r.shape[1], _p(fr), len(fr), _p(kv), nk, C.c_double(box_len),
                            int(n_threads), _p(out))
    return out


def structure_factor_bins(s, timescheme, wrapped, lst, bins, n_bins, kvec_n, shell_off, spacing, box_len,
                          mode=F64):
    """Per-bin S(k) [bins][shells] of the time-dependent lists (list && bin)."""
    r = _f32(wrapped)
    lst = _i32(lst)
    b = _i32(bins)
    kv = _i32(kvec_n).reshape(-1)
    off = _i32(shell_off)
    ns = len(off) - 1
    out = np.zeros((n_bins, ns))
    lib().orc_structure_factor_bins(C.byref(s), int(timescheme), _p(r), r.shape[1], _p(lst), len(lst), _p(b),
                                    int(n_bins), _p(kv), _p(off), ns, C.c_float(spacing), C.c_double(box_len),
                                    mode, _p(out))
    return out


def bins_distance(wrapped, box, kind, binned, from_list=None, point=(0, 0, 0), axis=0, direction=0,
                  position=0.0, thickness=1.0, n_bins=1):
    """Distance bin map [frames][atoms] (-1 = none): kind 0 to the nearest member
    of from_list, 1 to a point, 2 to a plane (direction 0 average, 1 above, 2 below)."""
    r = _f32(wrapped)
    bx = _f32(box)
    bl = _i32(binned)
    fl = _i32(from_list if from_list is not None else [])
    pt = _f32(point)
    out = np.zeros((r.shape[0], r.shape[1]), np.int32)
    lib().orc_bins_distance(_p(r), r.shape[0], r.shape[1], _p(bx), int(kind), _p(bl), len(bl), _p(fl), len(fl),
                            _p(pt), int(axis), int(direction), C.c_float(position), C.c_float(thickness),
                            int(n_bins), _p(out))
    return out


def rhok_lattice(wrapped, frames, kvec_n, box_len, n_threads):
    """FP64 rho(k) of integer-lattice vectors from per-axis phasor tables (every
    atom of the trajectory); agrees with rhok_parallel to FP64 rounding."""
    r = _f32(wrapped)
    fr = _i32(frames)
    kv = _i32(kvec_n).reshape(-1)
    nk = len(kv) // 3
    out = np.zeros((len(fr), nk, 2))
    lib().orc_rhok_lattice(_p(r), r.shape[1], _p(fr), len(fr), _p(kv), nk, C.c_double(box_len),
                           int(n_threads), _p(out))
    return out


def gsmooth(wrapped, box, lst, frames, sigma, r_max, n_bins):
    """FP64 Gaussian-smoothed pair histogram (the engine's amdat_gsmooth_run)."""
    r = _f32(wrapped)
    bx = _f32(box)
    lst, fr = _i32(lst), _i32(frames)
    h = np.zeros(n_bins)
    lib().orc_gsmooth(_p(r), r.shape[1], _p(bx), _p(lst), len(lst), _p(fr), len(fr),
                      C.c_double(sigma), C.c_double(r_max), int(n_bins), _p(h))
    return h


def gsmooth_grad(wrapped, box, lst, frames, sigma, r_max, n_bins, w):
    """FP64 gradient of sum_b w[b] h[b] with respect to the list's positions."""
    r = _f32(wrapped)
    bx = _f32(box)
    lst, fr = _i32(lst), _i32(frames)
    ww = np.ascontiguousarray(w, np.float64)
    g = np.zeros((len(fr), len(lst), 3))
    lib().orc_gsmooth_grad(_p(r), r.shape[1], _p(bx), _p(lst), len(lst), _p(fr), len(fr),
                           C.c_double(sigma), C.c_double(r_max), int(n_bins), _p(ww), _p(g))
    return g


def sk_grad(wrapped, lst, frames, kvec_n, shell_off, box_len, w, n_threads=1):
    """FP64 gradient of sum_s w[s] S_raw[s], S_raw[s] = sum_f sum_{k in s} |rho_k|^2 / H_s."""
    r = _f32(wrapped)
    lst, fr = _i32(lst), _i32(frames)
    kv = _i32(kvec_n).reshape(-1)
    off = _i32(shell_off)
    ww = np.ascontiguousarray(w, np.float64)
    g = np.zeros((len(fr), len(lst), 3))
    lib().orc_sk_grad(_p(r), r.shape[1], _p(lst), len(lst), _p(fr), len(fr), _p(kv), len(kv) // 3,
                      _p(off), len(off) - 1, C.c_double(box_len), _p(ww), int(n_threads), _p(g))
    return g


def msd2d(s, unwrapped, lst, plane, mode=F64):
    """Mean_Square_Displacement_2D: plane 0 = xy, 1 = xz, 2 = yz."""
    u = _f32(unwrapped)
    lst = _i32(lst)
    out = np.zeros(n_timegaps(s))
    lib().orc_msd2d(C.byref(s), _p(u), u.shape[1], _p(lst), len(lst), int(plane), mode, _p(out))
    return out


def mean_disp(s, unwrapped, lst, mode=F64):
    """Mean_Displacement: [G][3]."""
    u = _f32(unwrapped)
    lst = _i32(lst)
    out = np.zeros((n_timegaps(s), 3))
    lib().orc_mean_disp(C.byref(s), _p(u), u.shape[1], _p(lst), len(lst), mode, _p(out))
    return out


def u2dist(s, unwrapped, lst, gap, bins, maxvalue, mode=F64):
    """DebyeWaller_Dist / Displacement_Distribution at one gap: (mean, variance, dist[bins+1])."""
    u = _f32(unwrapped)
    lst = _i32(lst)
    m, v = C.c_double(), C.c_double()
    dist = np.zeros(bins + 1)
    lib().orc_u2dist(C.byref(s), _p(u), u.shape[1], _p(lst), len(lst), int(gap), int(bins),
                     C.c_float(maxvalue), mode, C.byref(m), C.byref(v), _p(dist))
    return m.value, v.value, dist
