"""Python binding of the amdat_gb300 C ABI (include/amdat_gb300.h) via ctypes.

This is a thin convenience layer for tests, benchmarks and scripting: every
call goes straight to libamdat_gb300.so, which runs the CUDA kernels.  There
is no CPU fallback: if the library is missing or no GPU is present, calls
raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libamdat_gb300.so")

LINEAR, EXPONENTIAL, SNAPSHOT = 0, 1, 2
MIXED, PLAIN_FP64 = 0, 1
OUT_HOST, OUT_DEVICE = 0, 1

STATUS = {0: "OK", 1: "ARGUMENT", 2: "STATE", 3: "CUDA", 4: "NO_DEVICE", 5: "MEMORY", 6: "TIMEOUT"}


class AmdatError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"amdat_gb300 error {STATUS.get(status, status)}: {msg}")
        self.status = status


class Scheme(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n_exponentials", C.c_int32),
                ("n_exponential_steps", C.c_int32), ("exp_base", C.c_float),
                ("frt", C.c_int32), ("first_exponent", C.c_int32),
                ("time_unit", C.c_float), ("limit", C.c_int32)]


class DispRequest(C.Structure):
    _fields_ = [("list", C.c_int32), ("fullblock", C.c_int32), ("precision", C.c_int32),
                ("n_shells", C.c_int32), ("shell_offsets", C.c_void_p), ("kvec_n", C.c_void_p),
                ("kvec_period", C.c_float), ("n_bins", C.c_int32), ("bin_max", C.c_float)]


EXPORTED = [
    "amdat_version", "amdat_last_error", "amdat_scheme_init", "amdat_scheme_counts",
    "amdat_scheme_times", "amdat_scheme_weighting", "amdat_scheme_pairs", "amdat_create",
    "amdat_destroy", "amdat_set_stream", "amdat_synchronize", "amdat_launch_count",
    "amdat_traj_upload", "amdat_traj_upload_f64", "amdat_traj_upload_device",
    "amdat_list_create", "amdat_list_size", "amdat_disp_run", "amdat_disp_run_lists",
    "amdat_set_scheme", "amdat_wave_density", "amdat_wave_density_lattice",
    "amdat_wave_density_vectors", "amdat_wave_density_read", "amdat_wave_density_free",
    "amdat_isf_run", "amdat_structure_factor_run", "amdat_rdf_run", "amdat_vhd_run",
    "amdat_profile_reset", "amdat_profile_kernel", "amdat_run_script", "amdat_script_error",
    "amdat_disp_plan_create", "amdat_disp_plan_run", "amdat_disp_plan_read", "amdat_disp_plan_info",
    "amdat_disp_plan_destroy", "amdat_disp_plan_sharing", "amdat_disp_moments_noalloc",
    "amdat_gsmooth_run", "amdat_disp_axes_run",
    "amdat_gsmooth_adjoint", "amdat_structure_factor_adjoint",
    "amdat_boxify", "amdat_bins_create", "amdat_bins_read", "amdat_bins_free",
    "amdat_disp_bins_run", "amdat_disp_bins_axes_run", "amdat_fast_particles", "amdat_timelist_create",
    "amdat_bins_distance", "amdat_structure_factor_bins",
]

PLAN_AUTOTUNE, PLAN_GRAPH, PLAN_NO_SHARING = 1, 2, 4

_lib = None


def lib():
    """Load libamdat_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} not built: run amdat_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        L.amdat_version.restype = C.c_char_p
        L.amdat_last_error.restype = C.c_char_p
        L.amdat_script_error.restype = C.c_char_p
        for name in EXPORTED:
            fn = getattr(L, name)
            if name not in ("amdat_version", "amdat_last_error", "amdat_script_error"):
                fn.restype = C.c_int
        _lib = L
    return _lib


def _check(status: int):
    if status != 0:
        raise AmdatError(status, lib().amdat_last_error().decode())


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _i32(x):
    return np.ascontiguousarray(x, dtype=np.int32)


def _f32(x):
    return np.ascontiguousarray(x, dtype=np.float32)


def make_scheme(ts, limit: int = 0) -> Scheme:
    """C scheme from an amdat_gb300.synth.TimeScheme (or anything with the same fields)."""
    s = Scheme()
    if ts.kind == "linear":
        _check(lib().amdat_scheme_init(C.byref(s), LINEAR, ts.n_timesteps, 1, C.c_float(1.0), 0,
                                       0, C.c_float(ts.time_unit)))
    elif ts.kind == "exponential":
        _check(lib().amdat_scheme_init(C.byref(s), EXPONENTIAL, ts.n_exponentials,
                                       ts.n_exponential_steps, C.c_float(ts.exp_base), ts.frt,
                                       ts.first_exponent, C.c_float(ts.time_unit)))
    else:
        _check(lib().amdat_scheme_init(C.byref(s), SNAPSHOT, 1, 0, C.c_float(1.0), 0, 0,
                                       C.c_float(1.0)))
    s.limit = limit
    return s


def run_script(path: str, device: int = 0):
    """Run an AMDAT input script (hot-path commands) through amdat_run_script."""
    st = lib().amdat_run_script(path.encode(), int(device))
    if st != 0:
        raise AmdatError(st, lib().amdat_script_error().decode())


def scheme_counts(s: Scheme, fullblock=0, loop_order=0):
    T, G, P = C.c_int32(), C.c_int32(), C.c_int64()
    _check(lib().amdat_scheme_counts(C.byref(s), int(fullblock), int(loop_order), C.byref(T),
                                     C.byref(G), C.byref(P)))
    return T.value, G.value, P.value


def scheme_times(s: Scheme):
    T, G, _ = scheme_counts(s)
    tl, gt = np.zeros(T, np.float32), np.zeros(G, np.float32)
    _check(lib().amdat_scheme_times(C.byref(s), _p(tl), _p(gt)))
    return tl, gt


def scheme_pairs(s: Scheme, fullblock=0, loop_order=0):
    _, _, P = scheme_counts(s, fullblock, loop_order)
    g, a, b = (np.zeros(max(P, 1), np.int32) for _ in range(3))
    _check(lib().amdat_scheme_pairs(C.byref(s), int(fullblock), int(loop_order), _p(g), _p(a), _p(b)))
    return g[:P], a[:P], b[:P]


def scheme_weighting(s: Scheme, fullblock=0):
    _, G, _ = scheme_counts(s)
    w = np.zeros(G, np.int32)
    _check(lib().amdat_scheme_weighting(C.byref(s), int(fullblock), _p(w)))
    return w


class Engine:
    """One context on one GPU (amdat_create)."""

    def __init__(self, device: int = 0):
        self._ctx = C.c_void_p()
        _check(lib().amdat_create(int(device), C.byref(self._ctx)))
        self.n_frames = self.n_atoms = 0
        self.n_timegaps = 0
        self.scheme = None

    def close(self):
        if self._ctx:
            lib().amdat_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._ctx

    def set_stream(self, stream_ptr: int | None):
        _check(lib().amdat_set_stream(self._ctx, C.c_void_p(stream_ptr or 0)))

    def synchronize(self):
        _check(lib().amdat_synchronize(self._ctx))

    def launch_count(self) -> int:
        n = C.c_int64()
        _check(lib().amdat_launch_count(self._ctx, C.byref(n)))
        return n.value

    def profile_reset(self, enable: bool = True):
        _check(lib().amdat_profile_reset(self._ctx, int(enable)))

    def profile_kernel(self, name: str):
        """(launches, total device ms) of a kernel since the last profile_reset."""
        n, ms = C.c_int64(), C.c_double()
        _check(lib().amdat_profile_kernel(self._ctx, name.encode(), C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def upload_ptr(self, host_ptr: int, n_frames: int, n_atoms: int, box, box_lo=None):
        """Upload FP32 [T][N][3] coordinates from a raw host pointer (e.g. pinned memory)."""
        box = np.ascontiguousarray(box, np.float32)
        lo = None if box_lo is None else np.ascontiguousarray(box_lo, np.float32)
        _check(lib().amdat_traj_upload(self._ctx, n_frames, n_atoms, C.c_void_p(host_ptr), None,
                                       _p(box), _p(lo)))
        self.n_frames, self.n_atoms = n_frames, n_atoms

    def upload(self, unwrapped, box, box_lo=None, wrapped=None):
        u = np.ascontiguousarray(unwrapped)
        T, N, _ = u.shape
        box = np.ascontiguousarray(box, np.float32)
        lo = None if box_lo is None else np.ascontiguousarray(box_lo, np.float32)
        if u.dtype == np.float64:
            w = None if wrapped is None else np.ascontiguousarray(wrapped, np.float64)
            _check(lib().amdat_traj_upload_f64(self._ctx, T, N, _p(u), _p(w), _p(box), _p(lo)))
        else:
            u = np.ascontiguousarray(u, np.float32)
            w = None if wrapped is None else np.ascontiguousarray(wrapped, np.float32)
            _check(lib().amdat_traj_upload(self._ctx, T, N, _p(u), _p(w), _p(box), _p(lo)))
        self.n_frames, self.n_atoms = T, N

    def upload_device(self, dev_ptr: int, n_frames: int, n_atoms: int, box, box_lo=None):
        box = np.ascontiguousarray(box, np.float32)
        lo = None if box_lo is None else np.ascontiguousarray(box_lo, np.float32)
        _check(lib().amdat_traj_upload_device(self._ctx, n_frames, n_atoms, C.c_void_p(dev_ptr),
                                              _p(box), _p(lo)))
        self.n_frames, self.n_atoms = n_frames, n_atoms

    def set_scheme(self, ts, limit: int = 0):
        s = ts if isinstance(ts, Scheme) else make_scheme(ts, limit)
        _check(lib().amdat_set_scheme(self._ctx, C.byref(s)))
        self.scheme = s
        self.n_timegaps = scheme_counts(s)[1]

    def list(self, atoms) -> int:
        a = _i32(atoms)
        h = C.c_int32()
        _check(lib().amdat_list_create(self._ctx, _p(a), len(a), C.byref(h)))
        return h.value

    def _disp_req(self, list_h, fullblock, precision, shells, period, n_bins, bin_max):
        req = DispRequest()
        req.list, req.fullblock, req.precision = int(list_h), int(fullblock), int(precision)
        keep = []
        if shells is not None:
            kv, off = shells
            kv = _i32(kv).reshape(-1)
            off = _i32(off)
            keep += [kv, off]
            req.n_shells = len(off) - 1
            req.shell_offsets = off.ctypes.data
            req.kvec_n = kv.ctypes.data
            req.kvec_period = float(period)
        req.n_bins = int(n_bins)
        req.bin_max = float(bin_max)
        return req, keep

    def disp(self, list_h=0, fullblock=0, shells=None, period=1.0, n_bins=0, bin_max=0.0,
             precision=MIXED):
        """Fused displacement pass; returns dict of per-gap arrays."""
        req, keep = self._disp_req(list_h, fullblock, precision, shells, period, n_bins, bin_max)
        G = self.n_timegaps
        S = req.n_shells
        d2, d4 = np.zeros(G), np.zeros(G)
        cnt = np.zeros(G, np.int64)
        fs = np.zeros((G, max(S, 1)))
        gs = np.zeros((G, max(n_bins, 1)), np.int64)
        _check(lib().amdat_disp_run(self._ctx, C.byref(req), OUT_HOST, _p(d2), _p(d4), _p(cnt),
                                    _p(fs) if S else None, _p(gs) if n_bins else None))
        del keep
        return dict(sum_d2=d2, sum_d4=d4, atom_pairs=cnt, fs_sum=fs[:, :S], gs_counts=gs[:, :n_bins])

    def disp_lists(self, lists, fullblock=0, shells=None, period=1.0, n_bins=0, bin_max=0.0,
                   out_device=None):
        req, keep = self._disp_req(0, fullblock, MIXED, shells, period, n_bins, bin_max)
        ls = _i32(lists)
        G, S, L = self.n_timegaps, req.n_shells, len(ls)
        if out_device is not None:
            d2, d4, cnt, fs, gs = out_device
            _check(lib().amdat_disp_run_lists(self._ctx, C.byref(req), _p(ls), L, OUT_DEVICE,
                                              C.c_void_p(d2), C.c_void_p(d4), C.c_void_p(cnt),
                                              C.c_void_p(fs) if S else None,
                                              C.c_void_p(gs) if n_bins else None))
            return None
        d2, d4 = np.zeros((L, G)), np.zeros((L, G))
        cnt = np.zeros((L, G), np.int64)
        fs = np.zeros((L, G, max(S, 1)))
        gs = np.zeros((L, G, max(n_bins, 1)), np.int64)
        _check(lib().amdat_disp_run_lists(self._ctx, C.byref(req), _p(ls), L, OUT_HOST, _p(d2),
                                          _p(d4), _p(cnt), _p(fs) if S else None,
                                          _p(gs) if n_bins else None))
        del keep
        return dict(sum_d2=d2, sum_d4=d4, atom_pairs=cnt, fs_sum=fs[..., :S],
                    gs_counts=gs[..., :n_bins])

    def disp_device(self, out_ptrs, list_h=0, fullblock=0, shells=None, period=1.0, n_bins=0,
                    bin_max=0.0, precision=MIXED):
        """Fused displacement pass writing to device pointers (d2, d4, cnt, fs, gs)."""
        req, keep = self._disp_req(list_h, fullblock, precision, shells, period, n_bins, bin_max)
        d2, d4, cnt, fs, gs = out_ptrs
        _check(lib().amdat_disp_run(self._ctx, C.byref(req), OUT_DEVICE, C.c_void_p(d2),
                                    C.c_void_p(d4), C.c_void_p(cnt),
                                    C.c_void_p(fs) if req.n_shells else None,
                                    C.c_void_p(gs) if n_bins else None))
        del keep

    def disp_axes(self, list_h=0, fullblock=0, gap=-1, n_bins=0, bin_size=1.0):
        """Per-axis sums [G][6] (dx, dy, dz, dx^2, dy^2, dz^2), sum |dr|^4, atom-pair
        counts and the |dr|^2 histogram (top bin = overflow) (amdat_disp_axes_run)."""
        G = self.n_timegaps
        ax, d4 = np.zeros((G, 6)), np.zeros(G)
        cnt = np.zeros(G, np.int64)
        h = np.zeros((G, max(n_bins, 1)), np.int64)
        _check(lib().amdat_disp_axes_run(self._ctx, int(list_h), int(fullblock), int(gap), int(n_bins),
                                         C.c_float(bin_size), OUT_HOST, _p(ax), _p(d4), _p(cnt),
                                         _p(h) if n_bins else None))
        return dict(axis_sums=ax, sum_d4=d4, atom_pairs=cnt, d2_counts=h[:, :n_bins])

    # ---- spatial bins
    def boxify(self, lo, hi):
        """System::boxify of the wrapped coordinates (amdat_boxify)."""
        lo, hi = _f32(lo), _f32(hi)
        _check(lib().amdat_boxify(self._ctx, _p(lo), _p(hi)))

    def bins_create(self, nbins, lo, hi) -> int:
        """Bin map of the wrapped coordinates (amdat_bins_create)."""
        lo, hi = _f32(lo), _f32(hi)
        h = C.c_int32()
        _check(lib().amdat_bins_create(self._ctx, int(nbins[0]), int(nbins[1]), int(nbins[2]), _p(lo), _p(hi),
                                       C.byref(h)))
        return h.value

    def bins_read(self, handle, n_frames, n_atoms, n_bins):
        """(map [frames][atoms], members per frame and bin [frames][bins])."""
        m = np.empty((n_frames, n_atoms), np.int32)
        c = np.zeros((n_frames, n_bins), np.int64)
        _check(lib().amdat_bins_read(self._ctx, int(handle), OUT_HOST, _p(m), _p(c)))
        return m, c

    def disp_bins_axes(self, list_h, bins_h, n_bins, persistent=0):
        """Per-bin axis sums [B][G][6] (dx, dy, dz, dx^2, dy^2, dz^2) and counts [B][G]."""
        G = self.n_timegaps
        ax = np.zeros((n_bins, G, 6))
        cnt = np.zeros((n_bins, G), np.int64)
        _check(lib().amdat_disp_bins_axes_run(self._ctx, int(list_h), int(bins_h), int(persistent), OUT_HOST,
                                              _p(ax), _p(cnt)))
        return dict(axis_sums=ax, count=cnt)

    def fast_particles(self, list_h, gap, min_u2) -> int:
        """Block-wise fast-particle membership as a one-bin map (amdat_fast_particles)."""
        h = C.c_int32()
        _check(lib().amdat_fast_particles(self._ctx, int(list_h), int(gap), C.c_float(min_u2), C.byref(h)))
        return h.value

    def timelist(self, members_per_frame) -> int:
        """Time-dependent list from the members of each frame (amdat_timelist_create)."""
        off = np.concatenate([[0], np.cumsum([len(m) for m in members_per_frame])]).astype(np.int32)
        idx = (np.concatenate([np.asarray(m, np.int32) for m in members_per_frame])
               if off[-1] else np.zeros(1, np.int32)).astype(np.int32)
        h = C.c_int32()
        _check(lib().amdat_timelist_create(self._ctx, _p(off), _p(idx), C.byref(h)))
        return h.value

    def bins_distance(self, kind, binned, from_list=0, point=(0.0, 0.0, 0.0), axis=0, direction=0,
                      position=0.0, thickness=1.0, n_bins=1) -> int:
        """Distance bin map (create_bin_list distance ...): kind 0 trajectory, 1 point, 2 plane."""
        pt = np.ascontiguousarray(point, np.float32)
        h = C.c_int32()
        _check(lib().amdat_bins_distance(self._ctx, int(kind), int(binned), int(from_list), _p(pt), int(axis),
                                         int(direction), C.c_float(position), C.c_float(thickness), int(n_bins),
                                         C.byref(h)))
        return h.value

    def structure_factor_bins(self, list_h, bins_h, n_bins, kvec_n, shell_off, period, frames):
        """Per-bin (sum over frames and shell of |rho|^2 / H, member-frame count)."""
        kv = _i32(kvec_n).reshape(-1)
        off = _i32(shell_off)
        fr = _i32(frames)
        S = len(off) - 1
        s = np.zeros((n_bins, S))
        n = np.zeros(n_bins, np.int64)
        _check(lib().amdat_structure_factor_bins(self._ctx, int(list_h), int(bins_h), _p(kv), len(kv) // 3, _p(off),
                                                 S, C.c_float(period), _p(fr), len(fr), _p(s), _p(n)))
        return s, n

    def bins_free(self, handle):
        _check(lib().amdat_bins_free(self._ctx, int(handle)))

    def disp_bins(self, list_h, bins_h, n_bins, persistent=0, fullblock=0, shells=None, period=1.0, d4=True):
        """Per-bin sums (amdat_disp_bins_run): sum_d2, sum_d4, count [B][G], fs_sum [B][G][S]."""
        G = self.n_timegaps
        d2 = np.zeros((n_bins, G))
        d4s = np.zeros((n_bins, G))
        cnt = np.zeros((n_bins, G), np.int64)
        kv = off = None
        S = 0
        if shells is not None:
            kv, off = _i32(shells[0]).reshape(-1), _i32(shells[1])
            S = len(off) - 1
        fs = np.zeros((n_bins, G, max(S, 1)))
        _check(lib().amdat_disp_bins_run(self._ctx, int(list_h), int(bins_h), int(persistent), int(fullblock), S,
                                         _p(off), _p(kv), C.c_float(period), OUT_HOST, _p(d2),
                                         _p(d4s) if d4 else None, _p(cnt),
                                         _p(fs) if S else None))
        return dict(sum_d2=d2, sum_d4=d4s if d4 else None, count=cnt, fs_sum=fs[:, :, :S])

    def plan(self, lists, fullblock=0, shells=None, period=1.0, n_bins=0, bin_max=0.0, flags=0):
        """Prepared many-list displacement run (amdat_disp_plan_*)."""
        return DispPlan(self, lists, fullblock, shells, period, n_bins, bin_max, flags)

    # ---- Fourier densities
    def wave_density(self, list_h, kvec_n, period, frames, precision=MIXED) -> int:
        kv = _i32(kvec_n).reshape(-1)
        fr = _i32(frames)
        h = C.c_int32()
        _check(lib().amdat_wave_density(self._ctx, int(list_h), _p(kv), len(kv) // 3,
                                        C.c_float(period), _p(fr), len(fr), int(precision),
                                        C.byref(h)))
        return h.value

    def wave_density_lattice(self, list_h, kmax, dk, period, frames, precision=MIXED):
        fr = _i32(frames)
        h, nk, ns = C.c_int32(), C.c_int32(), C.c_int32()
        _check(lib().amdat_wave_density_lattice(self._ctx, int(list_h), C.c_float(kmax),
                                                C.c_float(dk), C.c_float(period), _p(fr), len(fr),
                                                int(precision), C.byref(h), C.byref(nk),
                                                C.byref(ns)))
        return h.value, nk.value, ns.value

    def wave_density_vectors(self, handle, n_k, n_shells):
        kv = np.zeros((n_k, 3), np.int32)
        off = np.zeros(n_shells + 1, np.int32)
        _check(lib().amdat_wave_density_vectors(self._ctx, int(handle), _p(kv), _p(off)))
        return kv, off

    def wave_density_read(self, handle, n_frames, n_k, out_device=None):
        """rho[frame][k] as float32 (re, im) pairs; with out_device (a device
        pointer to n_frames * n_k float2) the table is copied on the device."""
        if out_device is not None:
            _check(lib().amdat_wave_density_read(self._ctx, int(handle), OUT_DEVICE,
                                                 C.c_void_p(out_device)))
            return None
        rho = np.zeros((n_frames, n_k, 2), np.float32)
        _check(lib().amdat_wave_density_read(self._ctx, int(handle), OUT_HOST, _p(rho)))
        return rho

    def wave_density_free(self, handle):
        _check(lib().amdat_wave_density_free(self._ctx, int(handle)))

    def isf(self, d1, d2, shell_off, fullblock=0, out_device=None):
        off = _i32(shell_off)
        S = len(off) - 1
        G = self.n_timegaps
        if out_device is not None:
            corr, pc = out_device
            _check(lib().amdat_isf_run(self._ctx, int(d1), int(d2), int(fullblock), _p(off), S,
                                       OUT_DEVICE, C.c_void_p(corr), C.c_void_p(pc)))
            return None
        corr = np.zeros((G, S))
        pc = np.zeros(G, np.int64)
        _check(lib().amdat_isf_run(self._ctx, int(d1), int(d2), int(fullblock), _p(off), S,
                                   OUT_HOST, _p(corr), _p(pc)))
        return corr, pc

    def structure_factor(self, d1, d2, shell_off, out_device=None):
        off = _i32(shell_off)
        S = len(off) - 1
        if out_device is not None:
            _check(lib().amdat_structure_factor_run(self._ctx, int(d1), int(d2), _p(off), S,
                                                    OUT_DEVICE, C.c_void_p(out_device)))
            return None
        out = np.zeros(S)
        _check(lib().amdat_structure_factor_run(self._ctx, int(d1), int(d2), _p(off), S, OUT_HOST,
                                                _p(out)))
        return out

    # ---- pair histograms
    def rdf(self, list1, list2, frames, max_distance, n_bins):
        fr = _i32(frames)
        out = np.zeros((len(fr), n_bins), np.int64)
        _check(lib().amdat_rdf_run(self._ctx, int(list1), int(list2), _p(fr), len(fr),
                                   C.c_float(max_distance), int(n_bins), OUT_HOST, _p(out)))
        return out

    def vhd(self, list1, list2, max_distance, n_bins, fullblock=0):
        out = np.zeros((self.n_timegaps, n_bins), np.int64)
        _check(lib().amdat_vhd_run(self._ctx, int(list1), int(list2), int(fullblock),
                                   C.c_float(max_distance), int(n_bins), OUT_HOST, _p(out)))
        return out


    # ---- differentiable structure
    def gsmooth(self, list_h, frames, sigma, r_max, n_bins, out_device=None):
        """Gaussian-smoothed pair histogram h[n_bins] (FP64), summed over frames."""
        fr = _i32(frames)
        if out_device is not None:
            _check(lib().amdat_gsmooth_run(self._ctx, int(list_h), _p(fr), len(fr), C.c_float(sigma),
                                           C.c_float(r_max), int(n_bins), OUT_DEVICE,
                                           C.c_void_p(out_device)))
            return None
        out = np.zeros(n_bins)
        _check(lib().amdat_gsmooth_run(self._ctx, int(list_h), _p(fr), len(fr), C.c_float(sigma),
                                       C.c_float(r_max), int(n_bins), OUT_HOST, _p(out)))
        return out

    def gsmooth_adjoint(self, list_h, frames, sigma, r_max, n_bins, dl_dh, n_list):
        """dLoss/dr [n_frames][n_list][3] (FP32) for dLoss/dh = dl_dh."""
        fr = _i32(frames)
        w = np.ascontiguousarray(dl_dh, dtype=np.float64)
        g = np.zeros((len(fr), n_list, 3), np.float32)
        _check(lib().amdat_gsmooth_adjoint(self._ctx, int(list_h), _p(fr), len(fr), C.c_float(sigma),
                                           C.c_float(r_max), int(n_bins), _p(w), OUT_HOST, _p(g)))
        return g

    def structure_factor_adjoint(self, density, shell_off, dl_ds, n_frames, n_list):
        """dLoss/dr [n_frames][n_list][3] (FP32) of loss(S_raw) with dLoss/dS_raw = dl_ds,
        S_raw the auto structure factor of the density (structure_factor(d, d, ...))."""
        off = _i32(shell_off)
        w = np.ascontiguousarray(dl_ds, dtype=np.float64)
        g = np.zeros((n_frames, n_list, 3), np.float32)
        _check(lib().amdat_structure_factor_adjoint(self._ctx, int(density), _p(off), len(off) - 1,
                                                    _p(w), OUT_HOST, _p(g)))
        return g


class DispPlan:
    """A prepared displacement run over many lists: run() is stream work only
    (optionally a CUDA-graph replay), read() copies the results out."""

    def __init__(self, eng, lists, fullblock, shells, period, n_bins, bin_max, flags):
        self.eng = eng
        req, self._keep = eng._disp_req(0, fullblock, MIXED, shells, period, n_bins, bin_max)
        self.lists = _i32(lists)
        self.S, self.NB, self.L, self.G = req.n_shells, int(n_bins), len(self.lists), eng.n_timegaps
        self._plan = C.c_void_p()
        _check(lib().amdat_disp_plan_create(eng.handle, C.byref(req), _p(self.lists), self.L,
                                            int(flags), C.byref(self._plan)))

    def run(self):
        _check(lib().amdat_disp_plan_run(self.eng.handle, self._plan))

    def read(self):
        L, G, S, NB = self.L, self.G, self.S, self.NB
        d2, d4 = np.zeros((L, G)), np.zeros((L, G))
        cnt = np.zeros((L, G), np.int64)
        fs = np.zeros((L, G, max(S, 1)))
        gs = np.zeros((L, G, max(NB, 1)), np.int64)
        _check(lib().amdat_disp_plan_read(self.eng.handle, self._plan, OUT_HOST, _p(d2), _p(d4),
                                          _p(cnt), _p(fs) if S else None, _p(gs) if NB else None))
        return dict(sum_d2=d2, sum_d4=d4, atom_pairs=cnt, fs_sum=fs[..., :S], gs_counts=gs[..., :NB])

    def info(self):
        ch, bps, ni, ms = C.c_int32(), C.c_int32(), C.c_int64(), C.c_double()
        _check(lib().amdat_disp_plan_info(self._plan, C.byref(ch), C.byref(bps), C.byref(ni),
                                          C.byref(ms)))
        return dict(chunk=ch.value, blocks_per_sm=bps.value, n_items=ni.value, tuned_ms=ms.value)

    def sharing(self):
        """(work units, atoms streamed per time pair, sum of the list sizes)"""
        nu, ua, la = C.c_int32(), C.c_int64(), C.c_int64()
        _check(lib().amdat_disp_plan_sharing(self._plan, C.byref(nu), C.byref(ua), C.byref(la)))
        return dict(n_units=nu.value, unit_atoms=ua.value, list_atoms=la.value)

    def close(self):
        if self._plan:
            lib().amdat_disp_plan_destroy(self.eng.handle, self._plan)
            self._plan = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
