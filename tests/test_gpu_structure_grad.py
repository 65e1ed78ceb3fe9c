"""GPU parity of the differentiable-structure kernels: the Gaussian-smoothed
pair histogram against the FP64 oracle, its adjoint and the structure-factor
adjoint (column and direct kernels) against the oracle's FP64 gradients, both
adjoints against central finite differences (h = 1e-4) of the engine's own
forward sums, and the libtorch autograd functions end to end.

Tolerances (stated relative to the largest gradient component, or the largest
bin, of the case): forward histogram 1e-4; adjoints vs FP64 gradient 5e-4;
finite differences of the FP32/FP64 forward 5e-3 for g(r) and 2e-2 for S(k)
(the forward's own rounding, divided by the 2e-4 step, sets those floors)."""
import os

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu

SIGMA, R_MAX, N_BINS = 0.02, 4.0, 400
THREADS = os.cpu_count() or 1


def _pos(F, n, L, seed):
    rng = np.random.default_rng(seed)
    return (rng.random((F, n, 3)) * L).astype(np.float32)


def _upload(eng, pos, L):
    eng.upload(pos, [L, L, L], box_lo=[0.0, 0.0, 0.0], wrapped=pos)


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


# (box, atoms): all partners (box under three cutoffs wide), and cell lists
GS_CASES = [(12.0, 1500), (16.0, 3000)]


@pytest.mark.parametrize("L,n", GS_CASES)
def test_gsmooth_forward_matches_oracle(eng, L, n):
    F = 2
    pos = _pos(F, n, L, 11)
    _upload(eng, pos, L)
    h = eng.gsmooth(0, [0, 1], SIGMA, R_MAX, N_BINS)
    ref = orc.gsmooth(pos, [L, L, L], np.arange(n), [0, 1], SIGMA, R_MAX, N_BINS)
    assert _rel(h, ref) <= 1e-4
    # a sub-list (gathered indices) and one frame
    sub = np.arange(3, n, 3, dtype=np.int32)
    hl = eng.list(sub)
    h2 = eng.gsmooth(hl, [1], SIGMA, R_MAX, N_BINS)
    ref2 = orc.gsmooth(pos, [L, L, L], sub, [1], SIGMA, R_MAX, N_BINS)
    assert _rel(h2, ref2) <= 1e-4


@pytest.mark.parametrize("L,n", GS_CASES)
def test_gsmooth_adjoint_matches_oracle(eng, L, n):
    F = 2
    pos = _pos(F, n, L, 12)
    _upload(eng, pos, L)
    w = np.random.default_rng(13).standard_normal(N_BINS)
    g = eng.gsmooth_adjoint(0, [0, 1], SIGMA, R_MAX, N_BINS, w, n)
    ref = orc.gsmooth_grad(pos, [L, L, L], np.arange(n), [0, 1], SIGMA, R_MAX, N_BINS, w)
    assert _rel(g, ref) <= 5e-4


@pytest.mark.parametrize("L,n", [(12.0, 600), (14.0, 1200)])
def test_gsmooth_adjoint_matches_fd(eng, L, n):
    pos = _pos(1, n, L, 14)
    _upload(eng, pos, L)
    w = np.random.default_rng(15).standard_normal(N_BINS)
    g = eng.gsmooth_adjoint(0, [0], SIGMA, R_MAX, N_BINS, w, n)
    scale = np.abs(g).max()
    for (i, c) in [(0, 0), (101, 1), (377, 2), (n - 1, 0)]:
        vals = []
        for sgn in (1, -1):
            p = pos.copy()
            p[0, i, c] = np.float32(pos[0, i, c] + sgn * 1e-4)
            _upload(eng, p, L)
            vals.append((float(w @ eng.gsmooth(0, [0], SIGMA, R_MAX, N_BINS)), float(p[0, i, c])))
        fd = (vals[0][0] - vals[1][0]) / (vals[0][1] - vals[1][1])
        assert abs(fd - g[0, i, c]) <= 5e-3 * scale, (i, c, fd, g[0, i, c])


def _sraw(eng, d, off):
    return eng.structure_factor(d, d, off)


@pytest.mark.parametrize("kmax", [12.0, 6.5])
def test_sk_adjoint_columns_matches_oracle(eng, kmax):
    L, F, n = 12.0, 2, 1200
    pos = _pos(F, n, L, 21)
    _upload(eng, pos, L)
    d, nk, ns = eng.wave_density_lattice(0, kmax, 0.1, L, [0, 1])
    kv, off = eng.wave_density_vectors(d, nk, ns)
    w = np.random.default_rng(22).standard_normal(ns)
    g = eng.structure_factor_adjoint(d, off, w, F, n)
    ref = orc.sk_grad(pos, np.arange(n), [0, 1], kv, off, L, w, THREADS)
    assert _rel(g, ref) <= 5e-4
    eng.wave_density_free(d)


def test_sk_adjoint_direct_matches_oracle(eng, qvectors):
    # thin reference q-vector shells: short lattice columns, the direct kernel
    L, F, n = 12.0, 2, 1000
    pos = _pos(F, n, L, 23)
    _upload(eng, pos, L)
    kv_all, off_all = qvectors
    sel = [10, 20, 40]
    kv = np.concatenate([kv_all[off_all[m]:off_all[m + 1]] for m in sel])
    off = np.concatenate([[0], np.cumsum([off_all[m + 1] - off_all[m] for m in sel])]).astype(np.int32)
    d = eng.wave_density(0, kv, L, [0, 1])
    w = np.random.default_rng(24).standard_normal(len(sel))
    g = eng.structure_factor_adjoint(d, off, w, F, n)
    ref = orc.sk_grad(pos, np.arange(n), [0, 1], kv, off, L, w, THREADS)
    assert _rel(g, ref) <= 5e-4
    eng.wave_density_free(d)


def test_sk_adjoint_matches_fd(engine_mod, eng):
    L, n = 12.0, 800
    pos = _pos(1, n, L, 25)
    _upload(eng, pos, L)
    d, nk, ns = eng.wave_density_lattice(0, 8.0, 0.1, L, [0])
    kv, off = eng.wave_density_vectors(d, nk, ns)
    w = np.random.default_rng(26).standard_normal(ns)
    g = eng.structure_factor_adjoint(d, off, w, 1, n)
    eng.wave_density_free(d)
    scale = np.abs(g).max()
    for (i, c) in [(0, 0), (250, 1), (511, 2), (799, 2)]:
        vals = []
        for sgn in (1, -1):
            p = pos.copy()
            p[0, i, c] = np.float32(pos[0, i, c] + sgn * 1e-4)
            _upload(eng, p, L)
            dp = eng.wave_density(0, kv, L, [0], precision=engine_mod.PLAIN_FP64)
            vals.append((float(w @ _sraw(eng, dp, off)), float(p[0, i, c])))
            eng.wave_density_free(dp)
        fd = (vals[0][0] - vals[1][0]) / (vals[0][1] - vals[1][1])
        assert abs(fd - g[0, i, c]) <= 2e-2 * scale, (i, c, fd, g[0, i, c])


def test_torch_autograd_structure_loss():
    torch = pytest.importorskip("torch")
    from amdat_gb300 import autograd as AG
    from amdat_gb300 import build
    build.build_torch_ext()
    L, F, n = 12.0, 2, 1000
    box = [L, L, L]
    pos_np = _pos(F, n, L, 31)
    tgt_np = _pos(F, n, L, 32)
    dev = torch.device("cuda:0")
    pos = torch.tensor(pos_np, device=dev, requires_grad=True)
    tgt = torch.tensor(tgt_np, device=dev)
    kmax, dk = 6.0, 0.1
    with torch.no_grad():
        g_t = AG.g_of_r(AG.gsmooth(tgt, box, SIGMA, R_MAX, N_BINS), n, F, box, R_MAX)
        s_t = AG.s_of_k(AG.structure_factor_raw(tgt, box, kmax, dk), n, F)
    loss, g, s = AG.structure_loss(pos, box, g_t, s_t, SIGMA, R_MAX, N_BINS, kmax, dk)
    loss.backward()
    grad = pos.grad.cpu().numpy()
    # the same gradient from the FP64 oracle, with dLoss/dh and dLoss/dS_raw by hand
    r = (np.arange(N_BINS) + 0.5) * (R_MAX / N_BINS)
    ideal = F * 0.5 * n * (n - 1) / L ** 3 * 4 * np.pi * r * r
    w_h = 2 * (g.detach().cpu().numpy() - g_t.cpu().numpy()) / ideal
    w_s = 2 * (s.detach().cpu().numpy() - s_t.cpu().numpy()) / (F * n)
    kv, off = AG.lattice(pos.detach(), box, kmax, dk)
    lst = np.arange(n)
    ref = orc.gsmooth_grad(pos_np, box, lst, list(range(F)), SIGMA, R_MAX, N_BINS, w_h)
    ref += orc.sk_grad(pos_np, lst, list(range(F)), kv.numpy(), off.numpy(), L, w_s, THREADS)
    assert _rel(grad, ref) <= 5e-4
    # forward values against the oracle as well
    h_ref = orc.gsmooth(pos_np, box, lst, list(range(F)), SIGMA, R_MAX, N_BINS)
    assert _rel(g.detach().cpu().numpy() * ideal, h_ref) <= 1e-4


@pytest.mark.parametrize("L,kmax,n", [(12.0, 12.0, 1200), (25.0, 35.5, 300)])
def test_sk_adjoint_tensor_cores_match_column_kernel(eng, monkeypatch, L, kmax, n):
    """The tensor-core adjoint (default for lattice densities) against the FP32
    column kernel on the same density, including a lattice with two nz windows."""
    F = 2
    pos = _pos(F, n, L, 27)
    _upload(eng, pos, L)
    d, nk, ns = eng.wave_density_lattice(0, kmax, 0.1, L, [0, 1])
    kv, off = eng.wave_density_vectors(d, nk, ns)
    w = np.random.default_rng(28).standard_normal(ns)
    g_tc = eng.structure_factor_adjoint(d, off, w, F, n)
    monkeypatch.setenv("AMDAT_SK_ADJOINT", "columns")
    g_col = eng.structure_factor_adjoint(d, off, w, F, n)
    monkeypatch.delenv("AMDAT_SK_ADJOINT")
    eng.wave_density_free(d)
    assert _rel(g_tc, g_col) <= 5e-4
