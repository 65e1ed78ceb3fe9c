"""GPU parity of the displacement family (MSD/NGP moments, F_s, G_s) against
the oracle, through the C ABI.  Tolerances: MSD and |dr|^4 sums <= 1e-6
relative to the FP64 oracle; F_s (normalised, F_s(q,0) = 1) <= 1e-6 absolute;
G_s counts equal to the reference's FP32 binning except counted bin-edge ties
(the engine forms dr from frame-0-referenced coordinates)."""
import numpy as np
import pytest

from amdat_gb300 import synth
from golden.make_golden import CASES, load
from oracle import oracle as orc
from oracle import wavevectors as wv

pytestmark = pytest.mark.gpu


def _ref_shells(qvec, m0, m1):
    n, off = qvec
    return n[off[m0]:off[m1 + 1]], off[m0:m1 + 2] - off[m0]


def lattice_shell(period, kmin, kmax):
    """All integer lattice vectors with kmin <= |2 pi n / period| < kmax."""
    nmax = int(np.ceil(kmax * period / (2 * np.pi))) + 1
    r = np.arange(-nmax, nmax + 1)
    g = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)
    k = 2 * np.pi * np.linalg.norm(g, axis=1) / period
    return g[(k >= kmin) & (k < kmax)].astype(np.int32)


@pytest.mark.parametrize("case", sorted(CASES))
def test_moments_match_oracle(case, eng):
    traj, _, _ = load(case)
    eng.upload(traj.unwrapped, traj.box, traj.box_lo)
    for fb in (0, 1):
        eng.set_scheme(traj.scheme)
        out = eng.disp(0, fullblock=fb)
        s = orc.scheme(traj.scheme)
        d2, d4, cnt = orc.disp_moments(s, traj.unwrapped, None, fb)
        np.testing.assert_array_equal(out["atom_pairs"], cnt)
        m = cnt > 0
        np.testing.assert_allclose(out["sum_d2"][m], d2[m], rtol=1e-6, atol=1e-12)
        np.testing.assert_allclose(out["sum_d4"][m], d4[m], rtol=1e-6, atol=1e-14)


def test_msd_ngp_normalised_vs_oracle(eng):
    traj, _, _ = load("exp_small")
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    out = eng.disp(0)
    s = orc.scheme(traj.scheme)
    lst = np.arange(traj.n_atoms, dtype=np.int32)
    msd = orc.msd(s, traj.unwrapped, lst, orc.F64)
    ngp = orc.ngp(s, traj.unwrapped, lst, orc.F64)
    w = out["atom_pairs"].astype(float)
    gm = out["sum_d2"] / w
    np.testing.assert_allclose(gm[1:], msd[1:], rtol=1e-6)
    gn = out["sum_d4"] * 3.0 / w / (5.0 * gm * gm) - 1.0
    np.testing.assert_allclose(gn[1:], ngp[1:], rtol=1e-6, atol=1e-9)


@pytest.mark.parametrize("limit", [0, 3])
def test_limit_and_lists(eng, limit):
    traj, _, _ = load("lin_binary")
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme, limit=limit)
    s = orc.scheme(traj.scheme, limit)
    a = np.nonzero(traj.types == 0)[0].astype(np.int32)
    b = np.nonzero(traj.types == 1)[0].astype(np.int32)
    odd = np.arange(1, traj.n_atoms, 2, dtype=np.int32)   # gathered (non-contiguous) list
    for lst in (a, b, odd):
        h = eng.list(lst)
        out = eng.disp(h)
        d2, d4, cnt = orc.disp_moments(s, traj.unwrapped, lst, 0)
        np.testing.assert_array_equal(out["atom_pairs"], cnt)
        np.testing.assert_allclose(out["sum_d2"], d2, rtol=1e-6, atol=1e-12)


def test_empty_and_single_atom_lists(eng):
    traj, _, _ = load("exp_frt")
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    h0 = eng.list(np.zeros(0, np.int32))
    out = eng.disp(h0)
    assert (out["atom_pairs"] == 0).all() and (out["sum_d2"] == 0).all()
    h1 = eng.list([5])
    out = eng.disp(h1)
    s = orc.scheme(traj.scheme)
    d2, d4, cnt = orc.disp_moments(s, traj.unwrapped, np.array([5], np.int32), 0)
    np.testing.assert_allclose(out["sum_d2"], d2, rtol=1e-6, atol=1e-14)
    # NGP of a single atom at gap 0 is 0/0, as in the reference
    with np.errstate(invalid="ignore", divide="ignore"):
        ngp0 = out["sum_d4"][0] * 3 / out["atom_pairs"][0] / (5 * (out["sum_d2"][0] / out["atom_pairs"][0]) ** 2) - 1
    assert np.isnan(ngp0)


@pytest.mark.parametrize("case,m0,m1,fb", [("exp_small", 10, 12, 0), ("exp_small", 14, 15, 1),
                                          ("lin_binary", 6, 9, 0), ("exp_frt", 3, 5, 1)])
def test_fs_reference_shells(case, m0, m1, fb, eng, qvectors):
    traj, _, _ = load(case)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    L = float(np.float32(traj.box.min()))
    kv, off = _ref_shells(qvectors, m0, m1)
    out = eng.disp(0, fullblock=fb, shells=(kv, off), period=L)
    s = orc.scheme(traj.scheme)
    lst = np.arange(traj.n_atoms, dtype=np.int32)
    ref = orc.isfs(s, traj.unwrapped, lst, kv, off, float(wv.spacing(L)), L, fb, orc.F64)
    got = out["fs_sum"] / out["atom_pairs"][:, None]
    assert np.abs(got - ref).max() <= 1e-6


def test_fs_single_vector_terms_within_cosine_bound(eng):
    """Vector-list F_s evaluates each cos(k.dr) with the SFU cosine of the
    fixed-point phase reduced to [-pi, pi).  On a dyadic grid (coordinates in
    multiples of 2^-10, box 8) every displacement and phase is exact, so
    one-vector shells of single atoms (phases of many turns, both signs) show
    the cosine's own error: within its 2^-21.4 bound of the FP64 oracle, plus
    the FP32 accumulation."""
    traj, _, _ = load("exp_small")
    u = (np.round(traj.unwrapped.astype(np.float64) * 1024.0) / 1024.0).astype(np.float32)
    box = np.full(3, 8.0, np.float32)
    eng.upload(u, box)
    eng.set_scheme(traj.scheme)
    kv = np.array([[1, 0, 0], [37, -11, 5], [0, 0, -48], [-23, 29, 31]], np.int32)
    off = np.arange(len(kv) + 1, dtype=np.int32)
    s = orc.scheme(traj.scheme)
    for atom in (0, 7, 100):
        h = eng.list([atom])
        out = eng.disp(h, shells=(kv, off), period=8.0)
        # the engine's k is 2 pi n / L exactly (phases in fixed-point turns): the
        # oracle gets the FP64 spacing, not the reference's FP32-rounded one
        ref = orc.isfs(s, u, np.array([atom], np.int32), kv, off, 2.0 * np.pi / 8.0, 8.0, 0, orc.F64)
        m = out["atom_pairs"] > 0
        got = out["fs_sum"][m] / out["atom_pairs"][m][:, None]
        assert np.abs(got - ref[m]).max() <= 3.6e-7 + 1e-7


def test_fs_lattice_shell_octant_mode(eng):
    """Whole lattice shell |k| in [7.0, 7.2] (sign-symmetric: octant tables)."""
    box = 16.8
    scheme = synth.TimeScheme.exponential(3, 6, 1.3, 0, 0, 0.005)
    traj = synth.random_walk(300, box, scheme, 0.5, seed=5)
    shell = lattice_shell(box, 7.0, 7.2)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(scheme)
    off = np.array([0, len(shell)], np.int32)
    out = eng.disp(0, shells=(shell, off), period=box)
    s = orc.scheme(scheme)
    lst = np.arange(traj.n_atoms, dtype=np.int32)
    ref = orc.isfs(s, traj.unwrapped, lst, shell, off, float(wv.spacing(box)), box, 0, orc.F64)
    got = out["fs_sum"] / out["atom_pairs"][:, None]
    assert np.abs(got - ref).max() <= 1e-6
    # many shells in one request (> 8 per pass)
    shells = [lattice_shell(box, 1.0 + 0.5 * i, 1.5 + 0.5 * i) for i in range(11)]
    kv = np.concatenate(shells)
    off = np.concatenate([[0], np.cumsum([len(x) for x in shells])]).astype(np.int32)
    out = eng.disp(0, shells=(kv, off), period=box)
    ref = orc.isfs(s, traj.unwrapped, lst, kv, off, float(wv.spacing(box)), box, 0, orc.F64)
    got = out["fs_sum"] / out["atom_pairs"][:, None]
    assert np.abs(got - ref).max() <= 1e-6


@pytest.mark.parametrize("case,rmax,nb", [("exp_small", 0.5, 50), ("lin_binary", 1.0, 40),
                                          ("exp_frt", 0.8, 20)])
def test_gs_counts(case, rmax, nb, eng):
    traj, _, _ = load(case)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    out = eng.disp(0, n_bins=nb, bin_max=rmax)
    s = orc.scheme(traj.scheme)
    lst = np.arange(traj.n_atoms, dtype=np.int32)
    counts, w, _ = orc.vhs(s, traj.unwrapped, lst, rmax, nb)
    diff = np.abs(out["gs_counts"] - counts).sum()
    # every atom-pair lands in exactly one bin or beyond the last one in both
    assert diff <= 2 * max(1, counts.sum() // 100000), diff
    np.testing.assert_array_equal(out["atom_pairs"], w)


def test_plain_fp64_path(eng, qvectors):
    traj, _, _ = load("exp_small")
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    L = float(np.float32(traj.box.min()))
    kv, off = _ref_shells(qvectors, 10, 12)
    a = eng.disp(0, shells=(kv, off), period=L, n_bins=50, bin_max=0.5)
    b = eng.disp(0, shells=(kv, off), period=L, n_bins=50, bin_max=0.5, precision=1)
    np.testing.assert_allclose(a["sum_d2"], b["sum_d2"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(a["fs_sum"] / a["atom_pairs"][:, None],
                               b["fs_sum"] / b["atom_pairs"][:, None], atol=1e-6)
    assert np.abs(a["gs_counts"] - b["gs_counts"]).sum() <= 4


def test_many_lists_one_launch(eng):
    traj, _, _ = load("lin_binary")
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    rng = np.random.default_rng(3)
    perm = rng.permutation(traj.n_atoms)
    sizes = [1, 7, 50, 120, 250]
    handles = [eng.list(np.sort(perm[:n]).astype(np.int32)) for n in sizes]
    shell = lattice_shell(7.0, 3.0, 3.4)
    off = np.array([0, len(shell)], np.int32)
    batch = eng.disp_lists(handles, shells=(shell, off), period=7.0, n_bins=30, bin_max=1.0)
    for i, h in enumerate(handles):
        one = eng.disp(h, shells=(shell, off), period=7.0, n_bins=30, bin_max=1.0)
        # nested lists share work through membership classes: the sums differ
        # from the single-list ones only in summation order
        np.testing.assert_allclose(batch["sum_d2"][i], one["sum_d2"], rtol=1e-9)
        np.testing.assert_allclose(batch["fs_sum"][i], one["fs_sum"], rtol=1e-9, atol=1e-9)
        np.testing.assert_array_equal(batch["gs_counts"][i], one["gs_counts"])


@pytest.mark.parametrize("layout", ["nested", "bins_and_union", "random_overlap", "disjoint"])
def test_plan_sharing_matches_per_list(eng, engine_mod, layout):
    """Membership-class sharing gives the per-list results (summation order
    aside) and is adopted only where it removes work."""
    traj, _, _ = load("lin_binary")
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    n = traj.n_atoms
    rng = np.random.default_rng(11)
    perm = rng.permutation(n)
    if layout == "nested":
        sets = [np.sort(perm[:k]) for k in (5, 30, 31, 120, n)]
    elif layout == "bins_and_union":
        bins = np.array_split(perm, 4)
        sets = [np.sort(b) for b in bins] + [np.arange(n)]
    elif layout == "random_overlap":
        sets = [np.sort(rng.choice(n, size=n // 2, replace=False)) for _ in range(9)]
    else:
        sets = [np.sort(b) for b in np.array_split(perm, 3)]
    handles = [eng.list(a.astype(np.int32)) for a in sets]
    shell = lattice_shell(7.0, 2.0, 2.6)
    off = np.array([0, len(shell)], np.int32)
    kw = dict(shells=(shell, off), period=7.0, n_bins=25, bin_max=1.0)
    shared = eng.plan(handles, flags=2, **kw)
    alone = eng.plan(handles, flags=2 | engine_mod.PLAN_NO_SHARING, **kw)
    shared.run()
    alone.run()
    a, b = shared.read(), alone.read()
    sh, sb = shared.sharing(), alone.sharing()
    total = sum(len(x) for x in sets)
    assert sb == dict(n_units=len(sets), unit_atoms=total, list_atoms=total)
    if layout in ("nested", "bins_and_union"):
        assert sh["unit_atoms"] == n and sh["n_units"] < 2 * len(sets)
    else:
        assert sh == sb
    np.testing.assert_allclose(a["sum_d2"], b["sum_d2"], rtol=1e-9)
    np.testing.assert_allclose(a["sum_d4"], b["sum_d4"], rtol=1e-9)
    np.testing.assert_allclose(a["fs_sum"], b["fs_sum"], rtol=1e-9, atol=1e-9)
    np.testing.assert_array_equal(a["gs_counts"], b["gs_counts"])
    np.testing.assert_array_equal(a["atom_pairs"], b["atom_pairs"])
    shared.close()
    alone.close()


@pytest.mark.parametrize("sharing", [True, False])
def test_bulk_staged_kernel_matches_direct_and_oracle(eng, engine_mod, monkeypatch, sharing):
    """The bulk-copy-staged MSD + NGP kernel (AMDAT_DISP_KERNEL=bulk at plan
    creation) gives the direct kernel's sums up to summation order and the
    oracle's to 1e-6, on
    contiguous lists with ragged ends, ranges under eight atoms (direct loads)
    and small lists whose items span several pairs."""
    E = engine_mod
    traj, _, _ = load("lin_binary")
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    n = traj.n_atoms
    ranges = [(0, n), (3, n - 2), (5, 6), (0, 8), (9, 17), (17, 250), (1, 130)]
    handles = [eng.list(np.arange(a, b, dtype=np.int32)) for a, b in ranges]
    flags = 0 if sharing else E.PLAN_NO_SHARING
    monkeypatch.delenv("AMDAT_DISP_KERNEL", raising=False)
    direct = eng.plan(handles, flags=flags)
    monkeypatch.setenv("AMDAT_DISP_KERNEL", "bulk")
    bulk = eng.plan(handles, flags=flags)
    monkeypatch.delenv("AMDAT_DISP_KERNEL")
    direct.run()
    bulk.run()
    a, b = direct.read(), bulk.read()
    direct.close()
    bulk.close()
    np.testing.assert_array_equal(a["atom_pairs"], b["atom_pairs"])
    # both kernels keep compensated FP32 sums per thread in their own order
    # (each within a few 1e-9 of the exact sum): 1e-7 between them, 1e-6 to the oracle
    np.testing.assert_allclose(b["sum_d2"], a["sum_d2"], rtol=1e-7, atol=1e-12)
    np.testing.assert_allclose(b["sum_d4"], a["sum_d4"], rtol=1e-7, atol=1e-14)
    s = orc.scheme(traj.scheme)
    for i, (lo, hi) in enumerate(ranges[:3]):
        d2, d4, cnt = orc.disp_moments(s, traj.unwrapped[:, lo:hi])
        np.testing.assert_array_equal(b["atom_pairs"][i], cnt)
        np.testing.assert_allclose(b["sum_d2"][i], d2, rtol=1e-6, atol=1e-12)
        np.testing.assert_allclose(b["sum_d4"][i], d4, rtol=1e-6, atol=1e-14)


@pytest.mark.parametrize("fb", [0, 1])
def test_multi_pair_items_match_oracle(eng, engine_mod, fb):
    """Moments-only plans give lists below half a chunk several pairs of one
    gap per work item, and contiguous ranges are read four atoms per load;
    sizes around every threshold (1 member, the block size, half a chunk,
    whole chunks, ranges off the 4-atom grid), contiguous and gathered, match
    the oracle."""
    scheme = synth.TimeScheme.exponential(5, 9, 1.3, 0, 0, 0.005)
    traj = synth.random_walk(9000, 20.0, scheme, 0.4, 23)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    s = orc.scheme(traj.scheme)
    rng = np.random.default_rng(29)
    sizes = [1, 2, 3, 37, 255, 256, 257, 1000, 2047, 2048, 2049, 4096, 4100, 9000]
    sets = [np.arange(n, dtype=np.int32) for n in sizes]
    # contiguous ranges off the 4-atom grid (16-byte loads with ragged ends)
    sets += [np.arange(a, b, dtype=np.int32) for a, b in ((3, 5004), (77, 9000), (1, 6), (5, 4103))]
    sets += [np.sort(rng.choice(traj.n_atoms, size=n, replace=False)).astype(np.int32)
             for n in (1, 5, 300, 2000, 3000)]
    handles = [eng.list(x) for x in sets]
    plans = [eng.plan(handles, fullblock=fb, flags=engine_mod.PLAN_NO_SHARING),
             eng.plan(handles, fullblock=fb)]
    for pl in plans:
        pl.run()
        out = pl.read()
        for i, lst in enumerate(sets):
            d2, d4, cnt = orc.disp_moments(s, traj.unwrapped, lst, fb)
            np.testing.assert_array_equal(out["atom_pairs"][i], cnt)
            np.testing.assert_allclose(out["sum_d2"][i], d2, rtol=1e-6, atol=1e-12)
            np.testing.assert_allclose(out["sum_d4"][i], d4, rtol=1e-6, atol=1e-14)
    # the descriptors hold the scheme's frames: a plan made for another scheme
    # is refused, not run on stale pairs
    eng.set_scheme(synth.TimeScheme.exponential(4, 9, 1.3, 0, 0, 0.005))
    with pytest.raises(RuntimeError, match="time scheme changed"):
        plans[0].run()
    for pl in plans:
        pl.close()


def test_one_shot_plan_cache(eng, engine_mod):
    """Repeated one-shot runs reuse the request's prepared plan: the same
    request gives identical numbers, and a new scheme, a new trajectory or
    other shells are never served from the cache."""
    traj, _, _ = load("lin_binary")
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    shell = lattice_shell(7.0, 2.0, 2.6)
    off = np.array([0, len(shell)], np.int32)
    kw = dict(shells=(shell, off), period=7.0, n_bins=25, bin_max=1.0)
    a = eng.disp(0, **kw)
    for _ in range(3):
        b = eng.disp(0, **kw)
        for k in a:
            np.testing.assert_array_equal(a[k], b[k])
    far = lattice_shell(7.0, 5.0, 5.4)
    other = eng.disp(0, shells=(far, np.array([0, len(far)], np.int32)), period=7.0)
    m = a["atom_pairs"] > 0
    assert np.abs(other["fs_sum"][m] - a["fs_sum"][m]).max() > 1e-3 * a["atom_pairs"].max()
    s2 = synth.TimeScheme.linear(traj.n_frames - 3)
    eng.set_scheme(s2)
    c = eng.disp(0)
    d2, _, cnt = orc.disp_moments(orc.scheme(s2), traj.unwrapped, None, 0)
    np.testing.assert_array_equal(c["atom_pairs"], cnt)
    np.testing.assert_allclose(c["sum_d2"], d2, rtol=1e-6, atol=1e-12)
    moved = traj.unwrapped * np.float32(1.5)
    eng.upload(moved, traj.box)
    eng.set_scheme(traj.scheme)
    e = eng.disp(0)
    d2, _, _ = orc.disp_moments(orc.scheme(traj.scheme), moved, None, 0)
    np.testing.assert_allclose(e["sum_d2"], d2, rtol=1e-6, atol=1e-12)
    # a prepared plan survives a re-upload of the same shape, not of another
    plan = eng.plan([0])
    eng.upload(traj.unwrapped, traj.box)
    plan.run()
    np.testing.assert_allclose(plan.read()["sum_d2"][0], a["sum_d2"], rtol=1e-7)
    eng.upload(traj.unwrapped[:, :-5], traj.box)
    with pytest.raises(RuntimeError, match="another shape"):
        plan.run()
    plan.close()


def test_errors_are_status_codes(eng, engine_mod):
    with pytest.raises(engine_mod.AmdatError) as e:
        eng.disp(0)
    assert e.value.status == 2  # no trajectory yet
    traj, _, _ = load("exp_frt")
    eng.upload(traj.unwrapped, traj.box)
    with pytest.raises(engine_mod.AmdatError):
        eng.disp(0)  # no scheme
    eng.set_scheme(traj.scheme)
    with pytest.raises(engine_mod.AmdatError) as e:
        eng.disp(99)
    assert e.value.status == 1
    with pytest.raises(engine_mod.AmdatError):
        eng.list([3, 2])  # not ascending
    # a scheme needing more frames than uploaded
    eng.set_scheme(synth.TimeScheme.linear(500, 1.0))
    with pytest.raises(engine_mod.AmdatError) as e:
        eng.disp(0)
    assert e.value.status == 2


def test_plans_graph_and_autotune(eng, tmp_path, monkeypatch):
    """A prepared many-list plan gives the single-list results; its CUDA-graph
    replay and its autotuned tile give the same numbers run after run."""
    traj, _, _ = load("lin_binary")
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    rng = np.random.default_rng(5)
    perm = rng.permutation(traj.n_atoms)
    handles = [eng.list(np.sort(perm[:n]).astype(np.int32)) for n in (3, 40, 250)]
    shell = lattice_shell(7.0, 2.0, 2.6)
    off = np.array([0, len(shell)], np.int32)
    kw = dict(shells=(shell, off), period=7.0, n_bins=25, bin_max=1.0)
    ref = [eng.disp(h, **kw) for h in handles]
    plain = eng.plan(handles, **kw)
    plain.run()
    a = plain.read()
    graph = eng.plan(handles, flags=2, **kw)
    for _ in range(3):
        graph.run()
    b = graph.read()
    cache = tmp_path / "tune.jsonl"
    monkeypatch.setenv("AMDAT_TUNE_CACHE", str(cache))
    tuned = eng.plan(handles, flags=3, **kw)
    tuned.run()
    c = tuned.read()
    info = tuned.info()
    assert info["chunk"] in (256, 512, 1024, 2048) and info["blocks_per_sm"] in (2, 4, 8, 16)
    assert cache.exists() and '"chunk"' in cache.read_text()
    for out in (a, b, c):
        for i, r in enumerate(ref):
            np.testing.assert_allclose(out["sum_d2"][i], r["sum_d2"], rtol=1e-7)
            np.testing.assert_allclose(out["fs_sum"][i], r["fs_sum"], rtol=1e-6, atol=1e-9)
            np.testing.assert_array_equal(out["gs_counts"][i], r["gs_counts"])
            np.testing.assert_array_equal(out["atom_pairs"][i], r["atom_pairs"])
    for p in (plain, graph, tuned):
        p.close()


@pytest.mark.parametrize("case", ["siblings", "siblings_lin", "exp_frt"])
def test_disp_axes_match_oracle(case, eng):
    """Per-axis sums (msd_2d, mean_displacement) over all gaps and the |dr|^2
    distribution at single gaps against the FP64 oracle."""
    traj, _, _ = load(case)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    s = orc.scheme(traj.scheme)
    lst = np.arange(traj.n_atoms, dtype=np.int32)
    out = eng.disp_axes(0)
    w = out["atom_pairs"].astype(np.float64)
    ax = out["axis_sums"]
    with np.errstate(invalid="ignore", divide="ignore"):
        for plane, (a, b) in enumerate([(0, 1), (0, 2), (1, 2)]):
            ref = orc.msd2d(s, traj.unwrapped, lst, plane, orc.F64)
            got = (ax[:, 3 + a] + ax[:, 3 + b]) / w
            np.testing.assert_allclose(got[1:], ref[1:], rtol=1e-6, atol=1e-12)
        md = orc.mean_disp(s, traj.unwrapped, lst, orc.F64)
        # sums of signed displacements: error relative to the rms displacement
        scale = np.sqrt((ax[:, 3] + ax[:, 4] + ax[:, 5]) / w)
        got = ax[:, :3] / w[:, None]
        assert (np.abs(got - md)[1:] <= 1e-6 * scale[1:, None] + 1e-12).all()
    G = orc.n_timegaps(s)
    for gap in (1, G // 2, G - 1):
        bins, vmax = 20, 2.0
        one = eng.disp_axes(0, gap=gap, n_bins=bins + 1, bin_size=vmax / bins)
        assert (one["atom_pairs"][np.arange(G) != gap] == 0).all()
        assert one["atom_pairs"][gap] == out["atom_pairs"][gap]
        np.testing.assert_allclose(one["axis_sums"][gap], ax[gap], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(one["sum_d4"][gap], out["sum_d4"][gap], rtol=1e-12)
        counts = one["d2_counts"][gap]
        assert counts.sum() == one["atom_pairs"][gap]
        mean, var, dist = orc.u2dist(s, traj.unwrapped, lst, gap, bins, vmax, orc.F64)
        # the oracle's normalisation: dist = counts / w / atomcount; compare shapes
        frac = counts / counts.sum()
        ref = dist / dist.sum()
        assert np.abs(frac - ref).sum() <= 4.0 / counts.sum() + 1e-12
