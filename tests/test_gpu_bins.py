"""GPU parity of the spatial bins (amdat_boxify, amdat_bins_create) and the
binned displacement pass (amdat_disp_bins_run) against the oracle, through the
C ABI.  Bin maps and member counts are bit-exact; per-bin MSD <= 1e-6 relative
and F_s (normalised, F_s(q,0) = 1) <= 1e-6 absolute to the FP64 oracle.  The
reference's own per-bin output files are checked through the command-line
driver (tests/golden/bins, test_gpu_cli.py)."""
import numpy as np
import pytest

from golden.make_golden import load
from oracle import oracle as orc
from oracle import wavevectors as wv

pytestmark = pytest.mark.gpu
f32 = np.float32


def _bounds(traj):
    lo = traj.box_lo.astype(f32)
    hi = (traj.box_lo.astype(np.float64) + traj.box.astype(np.float64)).astype(f32)
    return lo, hi


def _region(lo, hi, user_lo, user_hi):
    # a bound of 0, or one beyond the box, is the box's own
    rlo = np.array([lo[d] if (user_lo[d] == 0 or user_lo[d] < lo[d]) else user_lo[d] for d in range(3)], f32)
    rhi = np.array([hi[d] if (user_hi[d] == 0 or user_hi[d] > hi[d]) else user_hi[d] for d in range(3)], f32)
    return rlo, rhi


def _wrapped_with_strays(traj, seed=5):
    """Wrapped coordinates with some atoms moved one box length out (boxify
    brings them back) and some exactly on a region bound (never in a bin)."""
    w = traj.wrapped().copy()
    rng = np.random.default_rng(seed)
    T, N, _ = w.shape
    L = traj.box.astype(f32)
    for _ in range(40):
        t, a, d = rng.integers(T), rng.integers(N), rng.integers(3)
        w[t, a, d] = f32(w[t, a, d] + (L[d] if rng.random() < 0.5 else -L[d]))
    w[0, 0, 0] = f32(traj.box_lo[0])
    w[1, 1, 1] = f32(2.0)
    return w


CASES = [((1, 1, 3), None), ((2, 1, 2), ([1.0, 0.0, 0.0], [5.0, 0.0, 4.0])), ((4, 3, 5), None),
         ((3, 3, 3), ([2.0, 2.0, -9.0], [0.0, 9.0, 4.5]))]


@pytest.mark.parametrize("nb,region", CASES)
def test_bin_map_matches_oracle(eng, nb, region):
    traj, _, _ = load("bins")
    w = _wrapped_with_strays(traj)
    eng.upload(traj.unwrapped, traj.box, traj.box_lo, wrapped=w)
    lo, hi = _bounds(traj)
    rlo, rhi = (lo, hi) if region is None else _region(lo, hi, np.asarray(region[0], f32),
                                                       np.asarray(region[1], f32))
    eng.boxify(lo, hi)
    B = nb[0] * nb[1] * nb[2]
    h = eng.bins_create(nb, rlo, rhi)
    got, counts = eng.bins_read(h, traj.n_frames, traj.n_atoms, B)
    ref = orc.assign_bins(orc.boxify(w, lo, hi), nb, rlo, rhi)
    np.testing.assert_array_equal(got, ref)
    ref_counts = np.stack([np.bincount(r[r >= 0], minlength=B) for r in ref])
    np.testing.assert_array_equal(counts, ref_counts)
    assert got[0, 0] == -1  # on the lower bound: outside
    eng.bins_free(h)


def _check_bins(eng, traj, lst, lst_h, nb, persistent, fullblock, qvectors, m0=8, m1=9):
    lo, hi = _bounds(traj)
    eng.boxify(lo, hi)
    B = nb[0] * nb[1] * nb[2]
    h = eng.bins_create(nb, lo, hi)
    bins = orc.assign_bins(orc.boxify(traj.wrapped(), lo, hi), nb, lo, hi)
    n, off_all = qvectors
    kv, off = n[off_all[m0]:off_all[m1 + 1]], off_all[m0:m1 + 2] - off_all[m0]
    L = float(f32(traj.box.min()))
    out = eng.disp_bins(lst_h, h, B, persistent=persistent, fullblock=fullblock, shells=(kv, off), period=L)
    # without the |dr|^4 column the other columns are unchanged
    out3 = eng.disp_bins(lst_h, h, B, persistent=persistent, fullblock=fullblock, shells=(kv, off), period=L,
                         d4=False)
    np.testing.assert_array_equal(out3["count"], out["count"])
    np.testing.assert_allclose(out3["sum_d2"], out["sum_d2"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(out3["fs_sum"], out["fs_sum"], rtol=1e-12, atol=1e-12)
    s = orc.scheme(traj.scheme)
    msd, w = orc.msd_bins(s, traj.unwrapped, lst, bins, B, persistent, orc.F64)
    corr = orc.isfs_bins(s, traj.unwrapped, lst, kv, off, float(wv.spacing(L)), L, bins, B, fullblock,
                         persistent, orc.F64)
    cnt = out["count"]
    if fullblock == 0 or persistent:
        # the MSD's own pairs (fullblock 0): counts are its weighting
        np.testing.assert_array_equal(cnt, w.astype(np.int64))
        m = cnt > 0
        np.testing.assert_allclose(out["sum_d2"][m] / cnt[m], msd[m], rtol=1e-6, atol=1e-12)
        assert np.isnan(msd[~m]).all()
    m = cnt > 0
    fs = out["fs_sum"][m] / cnt[m][:, None]
    assert np.abs(fs - corr[m]).max() <= 1e-6
    eng.bins_free(h)
    return cnt


@pytest.mark.parametrize("persistent", [0, 1])
@pytest.mark.parametrize("fullblock", [0, 1])
def test_disp_bins_match_oracle(eng, qvectors, persistent, fullblock):
    traj, _, _ = load("bins")
    eng.upload(traj.unwrapped, traj.box, traj.box_lo, wrapped=traj.wrapped())
    eng.set_scheme(traj.scheme)
    lst = np.arange(traj.n_atoms, dtype=np.int32)
    _check_bins(eng, traj, lst, 0, (2, 2, 3), persistent, fullblock, qvectors)
    # a gathered sub-list
    sub = np.nonzero(traj.types == 1)[0].astype(np.int32)
    _check_bins(eng, traj, sub, eng.list(sub), (1, 3, 2), persistent, fullblock, qvectors)


def test_disp_bins_many_bins_global_path(eng):
    """More bins than the per-block shared accumulators hold (global atomics):
    the per-bin sums against a numpy scatter of the FP64 terms."""
    traj, _, _ = load("bins")
    eng.upload(traj.unwrapped, traj.box, traj.box_lo, wrapped=traj.wrapped())
    eng.set_scheme(traj.scheme)
    lo, hi = _bounds(traj)
    nb = (24, 24, 24)
    B = nb[0] * nb[1] * nb[2]
    eng.boxify(lo, hi)
    h = eng.bins_create(nb, lo, hi)
    out = eng.disp_bins(0, h, B)
    bins = orc.assign_bins(orc.boxify(traj.wrapped(), lo, hi), nb, lo, hi)
    s = orc.scheme(traj.scheme)
    g, t0, t1 = orc.pairs(s, 0)
    G = eng.n_timegaps
    u = traj.unwrapped.astype(np.float64)
    d2 = ((u[t1] - u[t0]) ** 2).sum(-1)  # [pairs][atoms]
    b0 = bins[t0]
    keep = b0 >= 0
    key = (b0 * G + g[:, None])[keep]
    ref = np.zeros(B * G)
    np.add.at(ref, key, d2[keep])
    rc = np.bincount(key, minlength=B * G)
    np.testing.assert_array_equal(out["count"].reshape(-1), rc)
    np.testing.assert_allclose(out["sum_d2"].reshape(-1), ref, rtol=1e-6, atol=1e-9)
    eng.bins_free(h)


def test_bins_errors(eng, engine_mod):
    traj, _, _ = load("bins")
    eng.upload(traj.unwrapped, traj.box, traj.box_lo)
    eng.set_scheme(traj.scheme)
    lo, hi = _bounds(traj)
    with pytest.raises(engine_mod.AmdatError):
        eng.bins_create((0, 1, 1), lo, hi)
    with pytest.raises(engine_mod.AmdatError):
        eng.disp_bins(0, 12345, 1)
    h = eng.bins_create((1, 1, 1), lo, hi)
    # a map is tied to the trajectory it was made for
    eng.upload(traj.unwrapped[:-1], traj.box, traj.box_lo)
    with pytest.raises(engine_mod.AmdatError):
        eng.disp_bins(0, h, 1)
    eng.bins_free(h)


def _referenced(u):
    """The engine's stored coordinates: re-referenced to frame 0 in one FP32 rounding."""
    u = np.asarray(u, np.float32)
    return (u - u[0:1]).astype(np.float32)


@pytest.mark.parametrize("gap,thr", [(3, 0.004), (6, 0.05), (0, 0.0)])
def test_fast_particles_match_oracle(eng, gap, thr):
    """Fast_Particles membership per block, bit-exact against the oracle run on the
    same frame-0-referenced coordinates; NGP and MSD of the time-dependent list."""
    traj, _, _ = load("fast")
    eng.upload(traj.unwrapped, traj.box, traj.box_lo)
    eng.set_scheme(traj.scheme)
    sub = np.nonzero(traj.types == 1)[0].astype(np.int32)
    s = orc.scheme(traj.scheme)
    u = _referenced(traj.unwrapped)
    for lst, h_list in ((np.arange(traj.n_atoms, dtype=np.int32), 0), (sub, eng.list(sub))):
        h = eng.fast_particles(h_list, gap, thr)
        got, counts = eng.bins_read(h, traj.n_frames, traj.n_atoms, 1)
        fast, ref = orc.fast_particles(s, u, lst, gap, thr)
        np.testing.assert_array_equal(got, ref)
        K = traj.scheme.n_exponential_steps
        np.testing.assert_array_equal(counts[::K][:fast.shape[0], 0], fast.sum(1))
        out = eng.disp_bins(0, h, 1)
        allat = np.arange(traj.n_atoms, dtype=np.int32)
        msd, w = orc.msd_bins(s, u, allat, ref, 1, 0, orc.F64)
        ngp = orc.ngp_bins(s, u, allat, ref, 1, 0, orc.F64)
        np.testing.assert_array_equal(out["count"][0], w[0].astype(np.int64))
        m = out["count"][0] > 0
        gm = out["sum_d2"][0][m] / out["count"][0][m]
        np.testing.assert_allclose(gm, msd[0][m], rtol=1e-6, atol=1e-12)
        ok = gm > 0  # gap 0 has no NGP (0/0)
        wq = out["count"][0][m][ok].astype(float)
        gq = out["sum_d4"][0][m][ok] * 3.0 / wq / (5.0 * gm[ok] * gm[ok]) - 1.0
        np.testing.assert_allclose(gq, ngp[0][m][ok], rtol=1e-6, atol=1e-9)
        eng.bins_free(h)


def test_bins_edge_cases(eng):
    """An empty list, a region no atom is in, a single-atom list and a fast-particle
    threshold nothing passes: zero counts (the reference's 0/0 normalisation), no faults."""
    traj, _, _ = load("bins")
    eng.upload(traj.unwrapped, traj.box, traj.box_lo, wrapped=traj.wrapped())
    eng.set_scheme(traj.scheme)
    lo, hi = _bounds(traj)
    G = eng.n_timegaps
    eng.boxify(lo, hi)
    h = eng.bins_create((2, 2, 2), lo, hi)
    empty = eng.list(np.zeros(0, np.int32))
    out = eng.disp_bins(empty, h, 8)
    assert out["count"].sum() == 0 and not out["sum_d2"].any()
    one = eng.list(np.array([7], np.int32))
    out = eng.disp_bins(one, h, 8)
    assert out["count"].sum() == len(orc.pairs(orc.scheme(traj.scheme), 0)[0])  # one member per pair
    eng.bins_free(h)
    # a region thinner than any spacing between atoms and the box edge: no members
    h = eng.bins_create((1, 1, 1), lo, np.array([lo[0], hi[1], hi[2]], np.float32) + np.float32(1e-6))
    m, c = eng.bins_read(h, traj.n_frames, traj.n_atoms, 1)
    assert (m == -1).all() and c.sum() == 0
    out = eng.disp_bins(0, h, 1)
    assert out["count"].sum() == 0
    eng.bins_free(h)
    h = eng.fast_particles(0, 1, 1e30)
    m, c = eng.bins_read(h, traj.n_frames, traj.n_atoms, 1)
    assert (m == -1).all()
    assert eng.disp_bins(0, h, 1)["count"].shape == (1, G)
    eng.bins_free(h)


@pytest.mark.parametrize("persistent", [0, 1])
def test_disp_bins_axes_match_oracle(eng, persistent):
    """Per-bin axis sums (msd_2d, mean_displacement) against the FP64 oracle."""
    traj, _, _ = load("bins_axes")
    eng.upload(traj.unwrapped, traj.box, traj.box_lo, wrapped=traj.wrapped())
    eng.set_scheme(traj.scheme)
    lo, hi = _bounds(traj)
    nb = (1, 2, 2)
    B = 4
    eng.boxify(lo, hi)
    h = eng.bins_create(nb, lo, hi)
    bins = orc.assign_bins(orc.boxify(traj.wrapped(), lo, hi), nb, lo, hi)
    s = orc.scheme(traj.scheme)
    lst = np.arange(traj.n_atoms, dtype=np.int32)
    out = eng.disp_bins_axes(0, h, B, persistent)
    cnt = out["count"]
    m = cnt > 0
    md = orc.mean_disp_bins(s, traj.unwrapped, lst, bins, B, persistent, orc.F64)
    got_md = out["axis_sums"][..., :3][m] / cnt[m][:, None]
    scale = np.abs(md[m]).max()
    assert np.abs(got_md - md[m]).max() <= 1e-6 * scale + 1e-12
    if not persistent:  # the oracle's persistent msd_2d carries the reference's weighting offset
        m2 = orc.msd2d_bins(s, traj.unwrapped, lst, 0, bins, B, 0, orc.F64)
        got2 = (out["axis_sums"][..., 3] + out["axis_sums"][..., 4])[m] / cnt[m]
        np.testing.assert_allclose(got2, m2[m], rtol=1e-6, atol=1e-12)
    eng.bins_free(h)


def test_timelist_matches_oracle(eng):
    """A time-dependent list given as per-frame members (CSR): msd and the member
    counts against the oracle on the same membership, static and persistent."""
    traj, _, _ = load("bins")
    eng.upload(traj.unwrapped, traj.box, traj.box_lo)
    eng.set_scheme(traj.scheme)
    rng = np.random.default_rng(3)
    T, N = traj.n_frames, traj.n_atoms
    members = [np.sort(rng.choice(N, size=rng.integers(0, N // 2), replace=False)) for _ in range(T)]
    members[2] = np.zeros(0, np.int64)  # a frame without members
    h = eng.timelist(members)
    got, counts = eng.bins_read(h, T, N, 1)
    ref = -np.ones((T, N), np.int32)
    for t, m in enumerate(members):
        ref[t, m] = 0
    np.testing.assert_array_equal(got, ref)
    np.testing.assert_array_equal(counts[:, 0], [len(m) for m in members])
    s = orc.scheme(traj.scheme)
    allat = np.arange(N, dtype=np.int32)
    for persistent in (0, 1):
        out = eng.disp_bins(0, h, 1, persistent=persistent)
        msd, w = orc.msd_bins(s, traj.unwrapped, allat, ref, 1, persistent, orc.F64)
        np.testing.assert_array_equal(out["count"][0], w[0].astype(np.int64))
        m = out["count"][0] > 0
        np.testing.assert_allclose(out["sum_d2"][0][m] / out["count"][0][m], msd[0][m], rtol=1e-6, atol=1e-12)
    eng.bins_free(h)


DISTANCE_CASES = [
    dict(kind=0, thickness=0.5, n_bins=4, from_type=1),                       # nearest member of type 2
    dict(kind=0, thickness=0.3, n_bins=9, from_type=1, gathered=True),
    dict(kind=1, thickness=0.75, n_bins=3, point=(3.0, 2.5, 1.0)),
    dict(kind=1, thickness=0.4, n_bins=12, point=(0.0, 5.9, 3.3), gathered=True),
    dict(kind=2, thickness=0.8, n_bins=3, axis=2, direction=0, position=2.0),   # average
    dict(kind=2, thickness=1.0, n_bins=4, axis=0, direction=1, position=1.5),   # above
    dict(kind=2, thickness=1.25, n_bins=3, axis=1, direction=2, position=4.0),  # below
    dict(kind=2, thickness=0.35, n_bins=8, axis=0, direction=0, position=5.5, gathered=True),
]


@pytest.mark.parametrize("c", DISTANCE_CASES, ids=lambda c: "k{kind}_t{thickness}".format(**c))
def test_distance_bin_map_matches_oracle(eng, c):
    """create_bin_list distance trajectory|point|plane: every member's bin in every
    frame, bit-exact against the oracle's restatement of the reference's FP32
    chains (the golden case bins_distance pins the oracle to the reference)."""
    traj, _, _ = load("bins_distance")
    w = _wrapped_with_strays(traj, seed=7)
    eng.upload(traj.unwrapped, traj.box, traj.box_lo, wrapped=w)
    lo, hi = _bounds(traj)
    eng.boxify(lo, hi)
    wb = orc.boxify(w, lo, hi)
    N = traj.n_atoms
    binned = np.arange(N, dtype=np.int32)
    if c.get("gathered"):
        binned = np.sort(np.random.default_rng(3).choice(N, N // 2, replace=False)).astype(np.int32)
    hb = eng.list(binned) if c.get("gathered") else 0
    frm = np.nonzero(traj.types == c.get("from_type", 0))[0].astype(np.int32) if c["kind"] == 0 else None
    hf = eng.list(frm) if frm is not None else 0
    box = (hi - lo).astype(f32)
    kw = dict(point=c.get("point", (0, 0, 0)), axis=c.get("axis", 0), direction=c.get("direction", 0),
              position=c.get("position", 0.0), thickness=c["thickness"], n_bins=c["n_bins"])
    h = eng.bins_distance(c["kind"], hb, hf, **kw)
    nbx = [1, 1, 1]
    nbx[c.get("axis", 2) if c["kind"] == 2 else 2] = c["n_bins"]
    B = nbx[0] * nbx[1] * nbx[2]
    got, counts = eng.bins_read(h, traj.n_frames, N, B)
    ref = orc.bins_distance(wb, box, c["kind"], binned, frm, **kw)
    np.testing.assert_array_equal(got, ref)
    assert (got >= 0).sum() > 0
    for b in range(B):
        np.testing.assert_array_equal(counts[:, b], (ref == b).sum(1))
    eng.bins_free(h)


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_structure_factor_bins_match_oracle(eng, qvectors, kind):
    """S(k) per bin (structure_factor with a bin_list target): the list members in
    the bin at each frame, every reference q-vector shell, <= 1e-5 relative to
    the FP64 oracle (the reference's own per-bin files: tests/golden/bins_distance)."""
    traj, _, _ = load("bins_distance")
    eng.upload(traj.unwrapped, traj.box, traj.box_lo)
    eng.set_scheme(traj.scheme)
    lo, hi = _bounds(traj)
    eng.boxify(lo, hi)
    wb = orc.boxify(traj.wrapped(), lo, hi)
    N = traj.n_atoms
    lst = np.arange(N, dtype=np.int32)
    box = (hi - lo).astype(f32)
    frm = np.nonzero(traj.types == 1)[0].astype(np.int32)
    args = {0: dict(kind=0, thickness=0.5, n_bins=4), 1: dict(kind=1, thickness=0.75, n_bins=3, point=(3.0, 2.5, 1.0)),
            2: dict(kind=2, thickness=1.0, n_bins=3, axis=1, direction=0, position=2.0)}[kind]
    B = args["n_bins"]
    kw = {k: v for k, v in args.items() if k != "kind"}
    h = eng.bins_distance(kind, 0, eng.list(frm) if kind == 0 else 0, **kw)
    bins = orc.bins_distance(wb, box, kind, lst, frm if kind == 0 else None, **kw)
    L = float(f32(traj.box.min()))
    n, off = qvectors
    kv, off = n[off[0]:off[40]], off[:41] - off[0]
    frames = np.arange(traj.n_frames, dtype=np.int32)
    s_sum, cnt = eng.structure_factor_bins(0, h, B, kv, off, L, frames)
    s = orc.scheme(traj.scheme)
    ref = orc.structure_factor_bins(s, -1, wb, lst, bins, B, kv, off, float(wv.spacing(L)), L, orc.F64)
    np.testing.assert_array_equal(cnt, [(bins == b).sum() for b in range(B)])
    got = s_sum / np.maximum(cnt, 1)[:, None]
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-7)
    eng.bins_free(h)
