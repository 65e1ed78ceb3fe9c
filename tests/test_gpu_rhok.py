"""GPU parity of the Fourier densities rho(k,t), the coherent ISF correlator
and S(k) against the FP64 oracle.  Tolerances: |rho_gpu - rho_oracle| <=
2e-6 * sqrt(N) per element (N unit phasors); coherent F(k,t) and S(k) <= 1e-5
relative to their values scaled by S(k) (F(k,0) = S(k))."""
import os

import numpy as np
import pytest

from amdat_gb300 import synth
from golden.make_golden import load
from oracle import oracle as orc
from oracle import wavevectors as wv

pytestmark = pytest.mark.gpu


def _shells(qvec, m0, m1):
    n, off = qvec
    return n[off[m0]:off[m1 + 1]], off[m0:m1 + 2] - off[m0]


@pytest.mark.parametrize("case", ["exp_small", "lin_binary"])
def test_rhok_reference_shells(case, eng, qvectors):
    traj, _, _ = load(case)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    L = float(np.float32(traj.box.min()))
    kv, off = _shells(qvectors, 0, 98)
    frames = np.arange(traj.n_frames, dtype=np.int32)
    h = eng.wave_density(0, kv, L, frames)
    rho = eng.wave_density_read(h, len(frames), len(kv)).astype(np.float64)
    lst = np.arange(traj.n_atoms, dtype=np.int32)
    ref = orc.rhok(traj.wrapped(), lst, frames, kv, float(wv.spacing(L)), L, orc.F64)
    err = np.abs(rho - ref).max() / np.sqrt(traj.n_atoms)
    assert err <= 2e-6, err
    eng.wave_density_free(h)


@pytest.mark.parametrize("fb", [0, 1])
def test_isf_and_sk_reference_shells(fb, eng, qvectors):
    traj, _, _ = load("exp_small")
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(traj.scheme)
    L = float(np.float32(traj.box.min()))
    kv, off = _shells(qvectors, 0, 20)
    frames = np.arange(traj.n_frames, dtype=np.int32)
    h = eng.wave_density(0, kv, L, frames)
    corr, pc = eng.isf(h, h, off, fullblock=fb)
    N = traj.n_atoms
    got = corr / (pc[:, None] * N)
    lst = np.arange(N, dtype=np.int32)
    s = orc.scheme(traj.scheme)
    rho = orc.rhok(traj.wrapped(), lst, frames, kv, float(wv.spacing(L)), L, orc.F64)
    ref = orc.isf(s, rho, rho, off, N, fb, orc.F64)
    scale = np.maximum(np.abs(ref[0]), 1e-3)
    assert (np.abs(got - ref) / scale).max() <= 1e-5
    sk = eng.structure_factor(h, h, off) / (N * traj.n_frames)
    ref_sk = orc.structure_factor(s, -1, traj.wrapped(), lst, kv, off, float(wv.spacing(L)), L,
                                  orc.F64)
    np.testing.assert_allclose(sk, ref_sk, rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("frames,n", [(72, 300), (137, 200)])
def test_isf_linear_scheme_lag_kernel(eng, monkeypatch, qvectors, frames, n):
    """Linear schemes take the sliding-window correlator: its per-gap sums equal
    the pair-table kernel's to the bit (same Kahan order), and the FP64 oracle."""
    scheme = synth.TimeScheme.linear(frames, 1.0)
    traj = synth.random_walk(n, 7.0, scheme, 0.2, seed=31, time_scaled=False)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(scheme)
    L = float(np.float32(traj.box.min()))
    kv, off = _shells(qvectors, 0, 12)
    fr = np.arange(traj.n_frames, dtype=np.int32)
    h = eng.wave_density(0, kv, L, fr)
    corr, pc = eng.isf(h, h, off)
    monkeypatch.setenv("AMDAT_ISF_KERNEL", "pairs")
    corr_p, pc_p = eng.isf(h, h, off)
    monkeypatch.delenv("AMDAT_ISF_KERNEL")
    np.testing.assert_array_equal(pc, pc_p)
    np.testing.assert_array_equal(corr, corr_p)
    got = corr / (pc[:, None] * n)
    s = orc.scheme(scheme)
    rho = orc.rhok(traj.wrapped(), np.arange(n, dtype=np.int32), fr, kv, float(wv.spacing(L)), L, orc.F64)
    ref = orc.isf(s, rho, rho, off, n, 0, orc.F64)
    scale = np.maximum(np.abs(ref[0]), 1e-3)
    assert (np.abs(got - ref) / scale).max() <= 1e-5
    eng.wave_density_free(h)


def test_rhok_lattice_mode(eng):
    """All half-space lattice vectors |k| <= kmax, shell-sorted: every element
    against the FP64 oracle on the returned vector list."""
    box = 9.0
    scheme = synth.TimeScheme.linear(4, 1.0)
    traj = synth.random_walk(700, box, scheme, 0.1, seed=9, time_scaled=False)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(scheme)
    frames = np.arange(4, dtype=np.int32)
    h, nk, ns = eng.wave_density_lattice(0, 9.0, 0.1, box, frames)
    kv, off = eng.wave_density_vectors(h, nk, ns)
    # half-space, |k| <= kmax, no duplicates, sorted into 0.1-wide shells
    k = 2 * np.pi * np.linalg.norm(kv, axis=1) / box
    assert (k <= 9.0 + 1e-9).all() and len(np.unique(kv, axis=0)) == nk
    assert ((kv[:, 2] > 0) | ((kv[:, 2] == 0) & ((kv[:, 1] > 0) | ((kv[:, 1] == 0) & (kv[:, 0] > 0))))).all()
    R = 9.0 * box / (2 * np.pi)
    full = sum(1 for x in range(-20, 21) for y in range(-20, 21) for z in range(-20, 21)
               if 0 < x * x + y * y + z * z <= R * R)
    assert nk == full // 2
    sh = np.repeat(np.arange(ns), np.diff(off))
    assert (np.floor(k / 0.1).astype(int).clip(max=ns - 1) == sh).all()
    rho = eng.wave_density_read(h, 4, nk).astype(np.float64)
    lst = np.arange(traj.n_atoms, dtype=np.int32)
    ref = orc.rhok(traj.wrapped(), lst, frames, kv, float(wv.spacing(box)), box, orc.F64)
    err = np.abs(rho - ref).max() / np.sqrt(traj.n_atoms)
    assert err <= 2e-6, err
    # shell structure factors from these densities: <= 1e-5 relative
    def shell_sk(r):
        p = (r ** 2).sum(-1).mean(0)  # |rho|^2 averaged over frames
        return np.array([p[off[i]:off[i + 1]].mean() for i in range(ns) if off[i + 1] > off[i]])
    sk_gpu, sk_ref = shell_sk(rho), shell_sk(ref)
    assert (np.abs(sk_gpu - sk_ref) / sk_ref).max() <= 1e-5
    # the same vectors through list mode agree
    h2 = eng.wave_density(0, kv, box, frames)
    rho2 = eng.wave_density_read(h2, 4, nk).astype(np.float64)
    assert np.abs(rho2 - ref).max() / np.sqrt(traj.n_atoms) <= 2e-6


@pytest.mark.parametrize("box,kmax,n_atoms,n_frames", [
    (20.0, 19.0, 300, 2),    # nmax 60: one 64-wide nz window, tiles trimmed to 16..64 columns
    (25.0, 35.5, 40, 1),     # nmax 141: two 128-wide nz windows
    (8.0, 3.0, 33, 3),       # nmax 3: 16-column tiles, a one-atom last chunk
])
def test_rhok_lattice_tilings(eng, box, kmax, n_atoms, n_frames):
    """Lattice densities whose tilings exercise every tensor-core tile shape,
    against the FP64 oracle.  These cases hold up to 1e6 elements, so the bound
    is on the rms error (<= 1e-6 sqrt(N)) and on the largest one (<= 3e-6 sqrt(N)):
    the rounding of the tensor core's FP32 accumulation over 64 atoms gives
    independent errors whose extreme over many elements passes 2e-6 sqrt(N)."""
    scheme = synth.TimeScheme.linear(n_frames + 1, 1.0)
    traj = synth.random_walk(n_atoms, box, scheme, 0.1, seed=17, time_scaled=False)
    eng.upload(traj.unwrapped, traj.box)
    frames = np.arange(n_frames, dtype=np.int32)
    h, nk, ns = eng.wave_density_lattice(0, kmax, 0.1, box, frames)
    kv, off = eng.wave_density_vectors(h, nk, ns)
    rho = eng.wave_density_read(h, n_frames, nk).astype(np.float64)
    eng.wave_density_free(h)
    ref = orc.rhok_parallel(traj.wrapped(), frames, kv, box, os.cpu_count() or 1)
    d = (rho - ref) / np.sqrt(n_atoms)
    rms, worst = float(np.sqrt((d ** 2).mean())), float(np.abs(d).max())
    assert rms <= 1e-6 and worst <= 3e-6, (rms, worst)


def test_rhok_plain_fp64(eng, qvectors):
    traj, _, _ = load("exp_frt")
    eng.upload(traj.unwrapped, traj.box)
    L = float(np.float32(traj.box.min()))
    kv, off = _shells(qvectors, 0, 30)
    frames = np.array([0, 5, 30], np.int32)
    a = eng.wave_density_read(eng.wave_density(0, kv, L, frames), 3, len(kv))
    b = eng.wave_density_read(eng.wave_density(0, kv, L, frames, precision=1), 3, len(kv))
    assert np.abs(a - b).max() <= 2e-6 * np.sqrt(traj.n_atoms)


def test_rhok_sublist(eng, qvectors):
    traj, _, _ = load("lin_binary")
    eng.upload(traj.unwrapped, traj.box)
    L = float(np.float32(traj.box.min()))
    kv, off = _shells(qvectors, 0, 10)
    b = np.nonzero(traj.types == 1)[0].astype(np.int32)
    h = eng.wave_density(eng.list(b), kv, L, np.array([3], np.int32))
    rho = eng.wave_density_read(h, 1, len(kv)).astype(np.float64)
    ref = orc.rhok(traj.wrapped(), b, np.array([3], np.int32), kv, float(wv.spacing(L)), L, orc.F64)
    assert np.abs(rho - ref).max() <= 2e-6 * np.sqrt(len(b))
