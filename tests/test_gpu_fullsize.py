"""Parity at the sizes the benchmark times, against the FP64 oracle.

- Coherent ISF + S(k) shape: N = 32000 (80:20), L = 33.6, every half-space
  lattice vector with |k| <= 20 (2,562,052 vectors, nmax 106, 1000 atom chunks
  per tensor-core tile, i.e. 500 accumulator drains per element), on the first
  three frames of the benchmark's 400-frame walk (the walk's prefix is the same).
  The tensor-core densities are compared element by element on a seeded sample
  of 100 vectors from every 0.1-wide shell, and S(k) and F(k,t) over whole
  shells spread across the range.  The oracle for these sizes is
  orc.rhok_lattice (FP64 products of exact per-axis phasor tables), itself
  pinned in this file against the direct FP64 sum orc.rhok_parallel.
- MSD + NGP + F_s shape: N = 4000, exponential 10 x 27, all 2,246 lattice
  vectors with |k| in [7.0, 7.2] (octant mode), every one of the 316 time pairs.
- Batched shape: the largest of the 64 nested lists (200,000-atom walk,
  exponential 12 x 30) read from the shared-class plan the benchmark times.

Tolerances: rho elements rms <= 1e-6 sqrt(N), largest <= 3e-6 sqrt(N); S(k)
and F(k,t) <= 1e-5 relative to S(k); MSD and |dr|^4 sums <= 1e-6 relative;
F_s <= 1e-6 absolute (normalised, F_s(q, 0) = 1)."""
import os

import numpy as np
import pytest

import bench
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def headline():
    traj, scheme, lat = bench.isf_workload(frames=3)
    return traj, scheme, lat


def _shell_sample(off, per_shell, seed):
    rng = np.random.default_rng(seed)
    idx = []
    for m in range(len(off) - 1):
        n = off[m + 1] - off[m]
        if n:
            idx.append(off[m] + np.sort(rng.choice(n, size=min(n, per_shell), replace=False)))
    return np.concatenate(idx)


def test_headline_lattice_density_isf_and_sk(eng, headline):
    traj, scheme, lat = headline
    N, T = traj.n_atoms, traj.n_frames
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(scheme)
    frames = np.arange(T, dtype=np.int32)
    h, nk, ns = eng.wave_density_lattice(0, lat["kmax"], lat["dk"], lat["period"], frames)
    assert (nk, ns) == (2562052, 200)
    kv, off = eng.wave_density_vectors(h, nk, ns)
    rho = eng.wave_density_read(h, T, nk)
    # the engine forms phases with the FP32 box length (33.6f): so does the oracle
    L = float(np.float32(lat["period"]))
    wrapped = traj.wrapped()

    # the lattice oracle against the direct FP64 sum on a few vectors
    few = _shell_sample(off, 1, seed=3)[::4]
    direct = orc.rhok_parallel(wrapped, frames[:1], kv[few], L, THREADS)
    fact = orc.rhok_lattice(wrapped, frames[:1], kv[few], L, THREADS)
    assert np.abs(direct - fact).max() <= 1e-9 * np.sqrt(N)

    # element-wise on 100 vectors of every shell (all three frames)
    sel = _shell_sample(off, 100, seed=11)
    assert len(sel) > 19000
    ref = orc.rhok_lattice(wrapped, frames, kv[sel], L, THREADS)
    d = (rho[:, sel].astype(np.float64) - ref) / np.sqrt(N)
    rms, worst = float(np.sqrt((d ** 2).mean())), float(np.abs(d).max())
    print(f"rho sample: {len(sel)} vectors x {T} frames, rms {rms:.3e} sqrt(N), worst {worst:.3e} sqrt(N)")
    assert rms <= 1e-6 and worst <= 3e-6, (rms, worst)

    # whole shells across the range: S(k) and F(k,t) of the linear scheme
    shells = sorted(set(range(0, ns, 20)) | {ns - 1})
    shells = [m for m in shells if off[m + 1] > off[m]]
    vidx = np.concatenate([np.arange(off[m], off[m + 1]) for m in shells])
    sub_off = np.concatenate([[0], np.cumsum([off[m + 1] - off[m] for m in shells])]).astype(np.int32)
    ref_rho = orc.rhok_lattice(wrapped, frames, kv[vidx], L, THREADS)
    ref_sk = np.array([(ref_rho[:, sub_off[i]:sub_off[i + 1]] ** 2).sum(-1).mean() for i in range(len(shells))]) / N
    sk = eng.structure_factor(h, h, off) / (N * T)
    rel = np.abs(sk[shells] - ref_sk) / ref_sk
    print(f"S(k) over {len(shells)} whole shells ({len(vidx)} vectors): worst relative {rel.max():.3e}")
    assert rel.max() <= 1e-5
    corr, pc = eng.isf(h, h, off)
    got = corr[:, shells] / (pc[:, None] * N)
    s = orc.scheme(scheme)
    ref_f = orc.isf(s, ref_rho, ref_rho, sub_off, N, 0, orc.F64)
    err = (np.abs(got - ref_f) / np.maximum(np.abs(ref_f[0]), 1e-3)).max()
    print(f"F(k,t) over the same shells, {len(pc)} gaps: worst {err:.3e} of S(k)")
    assert err <= 1e-5
    eng.wave_density_free(h)


def test_msd_workload_full_size(eng):
    traj, scheme = bench.msd_workload()
    shell = bench.lattice_shell(16.8, 7.0, 7.2)
    assert len(shell) == 2246
    off = np.array([0, len(shell)], np.int32)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(scheme)
    out = eng.disp(0, shells=(shell, off), period=16.8)
    s = orc.scheme(scheme)
    d2, d4, cnt = orc.disp_moments(s, traj.unwrapped)
    np.testing.assert_array_equal(out["atom_pairs"], cnt)
    assert int(cnt.sum()) == 316 * traj.n_atoms
    np.testing.assert_allclose(out["sum_d2"], d2, rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(out["sum_d4"], d4, rtol=1e-6, atol=1e-14)
    _, fs = orc.disp_fs_parallel(s, traj.unwrapped, shell, float(np.float32(16.8)), THREADS)
    c = np.maximum(cnt, 1)
    err = np.abs(out["fs_sum"][:, 0] / c - fs / (c * len(shell))).max()
    print(f"F_s, 2246 vectors x 316 pairs x 4000 atoms: worst {err:.3e}")
    assert err <= 1e-6


def test_batched_largest_list_from_shared_plan(eng):
    E = pytest.importorskip("amdat_gb300.engine")
    traj, scheme, sizes, perm = bench.batched_workload()
    shells = bench.reference_shells([10, 20, 40, 60, 80])
    L = 61.9
    u = np.ascontiguousarray(traj.unwrapped[:, perm])
    eng.upload(u, traj.box)
    eng.set_scheme(scheme)
    nested = [eng.list(np.arange(n, dtype=np.int32)) for n in sizes]
    plan = eng.plan(nested, shells=shells, period=L, flags=E.PLAN_AUTOTUNE | E.PLAN_GRAPH)
    plan.run()
    out = plan.read()
    plan.close()
    big = int(sizes[-1])
    s = orc.scheme(scheme)
    d2, d4, cnt = orc.disp_moments(s, u[:, :big])
    np.testing.assert_array_equal(out["atom_pairs"][-1], cnt)
    np.testing.assert_allclose(out["sum_d2"][-1], d2, rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(out["sum_d4"][-1], d4, rtol=1e-6, atol=1e-14)
    # F_s of the first shell (m = 10) over every time pair of the largest list
    kv, off = shells
    _, fs = orc.disp_fs_parallel(s, u[:, :big], kv[off[0]:off[1]], float(np.float32(L)), THREADS)
    c = np.maximum(cnt, 1)
    err = np.abs(out["fs_sum"][-1][:, 0] / c - fs / (c * (off[1] - off[0]))).max()
    print(f"largest list ({big} atoms, {int(cnt.sum()) // big} pairs): F_s shell 10 worst {err:.3e}")
    assert err <= 1e-6
