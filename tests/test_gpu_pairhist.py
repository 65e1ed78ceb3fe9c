"""GPU pair histograms (RDF per frame, distinct van Hove per time pair)
against the oracle's FP32 restatement of the reference's binning: integer
counts must be identical."""
import numpy as np
import pytest

from amdat_gb300 import synth
from golden.make_golden import load
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case,nb,maxd", [("exp_small", 100, 4.0), ("lin_binary", 60, 3.5),
                                          ("lin_binary", 30, 2.5)])
def test_rdf_counts_exact(case, nb, maxd, eng):
    traj, _, _ = load(case)
    eng.upload(traj.unwrapped, traj.box)
    s = orc.scheme(traj.scheme)
    lst = np.arange(traj.n_atoms, dtype=np.int32)
    frames = np.arange(traj.n_frames, dtype=np.int32)
    counts = eng.rdf(0, 0, frames, maxd, nb)
    ref, _ = orc.rdf(s, -1, traj.wrapped(), traj.box, lst, nb, maxd)
    np.testing.assert_array_equal(counts, ref)


def test_rdf_sublists_and_cross(eng):
    traj, _, _ = load("lin_binary")
    eng.upload(traj.unwrapped, traj.box)
    s = orc.scheme(traj.scheme)
    a = np.nonzero(traj.types == 0)[0].astype(np.int32)
    ha = eng.list(a)
    frames = np.arange(traj.n_frames, dtype=np.int32)
    counts = eng.rdf(ha, ha, frames, 3.0, 40)
    ref, _ = orc.rdf(s, -1, traj.wrapped(), traj.box, a, 40, 3.0)
    np.testing.assert_array_equal(counts, ref)
    # cross list (ordered pairs i in list1, j in list2): compare with a brute force
    b = np.arange(0, traj.n_atoms, 3, dtype=np.int32)
    hb = eng.list(b)
    got = eng.rdf(ha, hb, np.array([4], np.int32), 3.0, 40)[0]
    w = traj.wrapped()[4].astype(np.float32)
    L = traj.box.astype(np.float32)
    exp = np.zeros(40, np.int64)
    bs = np.float32(np.float32(3.0) / np.float32(40))
    for i in a:
        d = (w[b] - w[i]).astype(np.float32)
        m = np.minimum(np.abs(d), (L - np.abs(d)).astype(np.float32)).astype(np.float32)
        s2 = ((m[:, 0] * m[:, 0] + m[:, 1] * m[:, 1]).astype(np.float32) + m[:, 2] * m[:, 2]).astype(np.float32)
        r = np.sqrt(s2).astype(np.float32)
        bi = (r / bs).astype(np.float32).astype(np.int64)
        ok = (bi < 40) & (b != i)
        np.add.at(exp, bi[ok], 1)
    np.testing.assert_array_equal(got, exp)


def test_vhd_counts_exact(eng):
    scheme = synth.TimeScheme.linear(6, 1.0)
    traj = synth.random_walk(180, 5.0, scheme, 0.2, seed=4, time_scaled=False)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(scheme)
    counts = eng.vhd(0, 0, 2.5, 25)
    s = orc.scheme(scheme)
    lst = np.arange(traj.n_atoms, dtype=np.int32)
    ref, w = orc.vhd(s, traj.wrapped(), traj.box, lst, 2.5, 25)
    np.testing.assert_array_equal(counts, ref)


def test_rdf_large_symmetric_matches_ordered(eng):
    """Symmetric (j > i, counted twice) vs an ordered cross-list run over the
    same atoms: identical counts on a larger system."""
    scheme = synth.TimeScheme.linear(2, 1.0)
    traj = synth.random_walk(5000, 15.0, scheme, 0.1, seed=8, time_scaled=False)
    eng.upload(traj.unwrapped, traj.box)
    allh = eng.list(np.arange(5000, dtype=np.int32))  # same members, different handle
    fr = np.array([0, 1], np.int32)
    sym = eng.rdf(0, 0, fr, 7.5, 300)
    ordered = eng.rdf(0, allh, fr, 7.5, 300)
    np.testing.assert_array_equal(sym, ordered)
    assert sym[0].sum() > 0


@pytest.mark.parametrize("nb,maxd", [(40, 4.0), (80, 4.0), (64, 3.2)])
def test_rdf_lattice_distances_on_bin_edges(eng, nb, maxd):
    """Atoms on a cubic lattice whose spacing is a whole number of bins: many pair
    distances (a, 2a, 3a, ...) fall exactly on bin edges, where the bin must come
    from the correctly rounded chain; counts equal the oracle's."""
    a = 0.5
    g = np.arange(12, dtype=np.float64) * a
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(8)
    pos = pos[rng.permutation(len(pos))[:900]]
    jitter = np.zeros_like(pos)
    jitter[::7] = rng.normal(0, 1e-6, (len(pos[::7]), 3))  # a few just off the edges
    frame = (pos + jitter).astype(np.float32)
    L = np.float32(12 * a)
    traj = synth.Trajectory(unwrapped=np.stack([frame, frame]), box=np.full(3, L, np.float32),
                            box_lo=np.zeros(3, np.float32), types=np.zeros(len(pos), np.int32),
                            scheme=synth.TimeScheme.linear(2, 1.0))
    eng.upload(traj.unwrapped, traj.box, traj.box_lo, wrapped=traj.unwrapped)
    s = orc.scheme(traj.scheme)
    lst = np.arange(len(pos), dtype=np.int32)
    counts = eng.rdf(0, 0, np.array([0, 1], np.int32), maxd, nb)
    ref, _ = orc.rdf(s, -1, traj.unwrapped, traj.box, lst, nb, maxd)
    np.testing.assert_array_equal(counts, ref)


def test_vhd_cells_match_all_pairs_and_oracle(eng, monkeypatch):
    """Short-range distinct van Hove on a box of six cells per axis: the cell-list
    pass (27 neighbour cells of each atom) gives the all-pairs pass's counts and
    the oracle's, bit for bit."""
    scheme = synth.TimeScheme.linear(5, 1.0)
    traj = synth.random_walk(3000, 20.0, scheme, 0.6, seed=21, time_scaled=False)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(scheme)
    monkeypatch.delenv("AMDAT_PAIR_CELLS", raising=False)
    cells = eng.vhd(0, 0, 3.0, 60)
    monkeypatch.setenv("AMDAT_PAIR_CELLS", "off")
    direct = eng.vhd(0, 0, 3.0, 60)
    monkeypatch.delenv("AMDAT_PAIR_CELLS")
    np.testing.assert_array_equal(cells, direct)
    assert cells.sum() > 0
    s = orc.scheme(scheme)
    lst = np.arange(traj.n_atoms, dtype=np.int32)
    ref, _ = orc.vhd(s, traj.wrapped(), traj.box, lst, 3.0, 60)
    np.testing.assert_array_equal(cells, ref)


@pytest.mark.parametrize("maxd,nb", [(3.0, 60), (2.0, 40)])
def test_pair_cells_lattice_on_cell_and_bin_edges(eng, monkeypatch, maxd, nb):
    """A cubic lattice (1331 atoms, spacing 1) whose sites sit on cell edges and
    whose distances fall on bin edges: the cell-list ordered pass (two handles
    of the same atoms) gives the all-pairs ordered pass's and the symmetric
    pass's counts, and the oracle's."""
    g = np.arange(11, dtype=np.float64)
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(3)
    jitter = np.zeros_like(pos)
    jitter[::5] = rng.normal(0, 1e-6, (len(pos[::5]), 3))
    frame = (pos + jitter).astype(np.float32)
    traj = synth.Trajectory(unwrapped=np.stack([frame, frame]), box=np.full(3, np.float32(11.0), np.float32),
                            box_lo=np.zeros(3, np.float32), types=np.zeros(len(pos), np.int32),
                            scheme=synth.TimeScheme.linear(2, 1.0))
    eng.upload(traj.unwrapped, traj.box, traj.box_lo, wrapped=traj.unwrapped)
    fr = np.array([0, 1], np.int32)
    allh = eng.list(np.arange(len(pos), dtype=np.int32))  # same members, another handle
    monkeypatch.delenv("AMDAT_PAIR_CELLS", raising=False)
    cells = eng.rdf(0, allh, fr, maxd, nb)
    monkeypatch.setenv("AMDAT_PAIR_CELLS", "off")
    direct = eng.rdf(0, allh, fr, maxd, nb)
    monkeypatch.delenv("AMDAT_PAIR_CELLS")
    sym = eng.rdf(0, 0, fr, maxd, nb)
    np.testing.assert_array_equal(cells, direct)
    np.testing.assert_array_equal(cells, sym)
    s = orc.scheme(traj.scheme)
    ref, _ = orc.rdf(s, -1, traj.unwrapped, traj.box, np.arange(len(pos), dtype=np.int32), nb, maxd)
    np.testing.assert_array_equal(cells, ref)
