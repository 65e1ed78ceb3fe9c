"""CPU checks of the differentiable-structure oracle (FP64): its gradients agree
with central finite differences of its own forward sums, the smoothed
histogram integrates to the pair count, and the libtorch autograd extension
loads and exposes its functions.  The GPU adjoints are checked against these
oracle gradients in test_gpu_structure_grad.py."""
import numpy as np
import pytest

from oracle import oracle as orc


def _config(n, L, seed):
    rng = np.random.default_rng(seed)
    return (rng.random((1, n, 3)) * L).astype(np.float32)


def _loss_h(pos, box, lst, sigma, r_max, n_bins, w):
    return float(w @ orc.gsmooth(pos, box, lst, [0], sigma, r_max, n_bins))


def _fd(fun, pos, f, i, c, h):
    """central difference with the float32 step actually taken"""
    p1, p2 = pos.copy(), pos.copy()
    p1[f, i, c] = np.float32(pos[f, i, c] + h)
    p2[f, i, c] = np.float32(pos[f, i, c] - h)
    step = float(p1[f, i, c]) - float(p2[f, i, c])
    return (fun(p1) - fun(p2)) / step


def test_gsmooth_integrates_to_pair_count():
    L, sigma, r_max, n_bins = 6.0, 0.05, 2.0, 200
    pos = _config(80, L, 1)
    box = np.array([L, L, L], np.float32)
    lst = np.arange(80, dtype=np.int32)
    h = orc.gsmooth(pos, box, lst, [0], sigma, r_max, n_bins)
    d = pos[0][:, None, :] - pos[0][None, :, :]
    d -= L * np.rint(d / L)
    r = np.sqrt((d ** 2).sum(-1))[np.triu_indices(80, 1)]
    # pairs well inside (0, r_max) carry their whole Gaussian weight
    inner = ((r > 8 * sigma) & (r < r_max - 8 * sigma)).sum()
    edge = ((r <= 8 * sigma) | ((r >= r_max - 8 * sigma) & (r < r_max + 6 * sigma))).sum()
    total = h.sum() * (r_max / n_bins)
    assert inner - 1e-6 <= total + 1e-9 and total <= inner + edge + 1e-6


@pytest.mark.parametrize("seed", [3, 4])
def test_gsmooth_grad_matches_fd(seed):
    L, sigma, r_max, n_bins, n = 5.0, 0.05, 2.0, 100, 60
    pos = _config(n, L, seed)
    box = np.array([L, L, L], np.float32)
    lst = np.arange(n, dtype=np.int32)
    w = np.random.default_rng(seed + 10).standard_normal(n_bins)
    g = orc.gsmooth_grad(pos, box, lst, [0], sigma, r_max, n_bins, w)
    fun = lambda p: _loss_h(p, box, lst, sigma, r_max, n_bins, w)  # noqa: E731
    scale = np.abs(g).max()
    for (i, c) in [(0, 0), (7, 1), (33, 2), (59, 0)]:
        fd = _fd(fun, pos, 0, i, c, 1e-4)
        # FD truncation ~ (h/sigma)^2 plus the float32 step: 1e-4 of the gradient scale
        assert abs(fd - g[0, i, c]) <= 1e-4 * scale, (i, c, fd, g[0, i, c])


def _half_space(R):
    v = []
    for x in range(-R, R + 1):
        for y in range(-R, R + 1):
            for z in range(0, R + 1):
                if x * x + y * y + z * z > R * R:
                    continue
                if z > 0 or (z == 0 and (y > 0 or (y == 0 and x > 0))):
                    v.append((x, y, z))
    v = np.array(v, np.int32)
    m = np.sqrt((v.astype(np.float64) ** 2).sum(1))
    order = np.argsort(m, kind="stable")
    v, m = v[order], m[order]
    shell = np.floor(m).astype(int)
    off = np.searchsorted(shell, np.arange(shell.max() + 2)).astype(np.int32)
    return v, off


def test_sk_grad_matches_fd():
    L, n = 7.0, 50
    pos = _config(n, L, 5)
    lst = np.arange(n, dtype=np.int32)
    kv, off = _half_space(4)
    ns = len(off) - 1
    w = np.random.default_rng(6).standard_normal(ns)
    H = np.diff(off)

    def loss(p):
        rho = orc.rhok(p, lst, [0], kv, 2 * np.pi / L, L, orc.F64)[0]
        s2 = (rho ** 2).sum(1)
        sraw = np.array([s2[off[s]:off[s + 1]].sum() / H[s] if H[s] else 0.0 for s in range(ns)])
        return float(w @ sraw)

    g = orc.sk_grad(pos, lst, [0], kv, off, L, w)
    scale = np.abs(g).max()
    for (i, c) in [(0, 0), (11, 1), (25, 2), (49, 1)]:
        fd = _fd(loss, pos, 0, i, c, 1e-4)
        assert abs(fd - g[0, i, c]) <= 1e-5 * scale, (i, c, fd, g[0, i, c])


def test_torch_extension_loads():
    pytest.importorskip("torch")
    from amdat_gb300 import build
    build.build_torch_ext()
    from amdat_gb300 import autograd
    m = autograd.ext()
    for name in ("gsmooth", "structure_factor", "lattice"):
        assert hasattr(m, name)
