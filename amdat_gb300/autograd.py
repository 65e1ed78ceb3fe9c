"""Differentiable structure on the GPU: torch autograd functions whose forward
and backward passes are the engine's CUDA kernels (amdat_gsmooth_run /
amdat_gsmooth_adjoint, amdat_wave_density_lattice + amdat_structure_factor_run /
amdat_structure_factor_adjoint), wrapped as libtorch ``torch::autograd::Function``
classes in the amdat_torch extension (amdat_gb300/torch_ext/amdat_torch.cpp).

The reference has no differentiable path; its nearest parts are the hard-binned
g(r) (Radial_Distribution_Function, src/radial_distribution_function.cpp:233-285)
and S(k) (Structure_Factor, src/structure_factor.cpp:201-320).  The
normalisations below follow those: g(r) against the ideal-gas pair count of a
spherical shell, S(k) = <|rho_k|^2> / N per shell.
"""
from __future__ import annotations

import importlib.util
import math
import os

import torch

from . import build as _build

_ext = None


def ext():
    """The compiled amdat_torch extension (raises ImportError when not built)."""
    global _ext
    if _ext is None:
        path = _build.torch_ext_path()
        if not os.path.exists(path):
            raise ImportError(f"{path} not built: run amdat_gb300.build.build_torch_ext()")
        spec = importlib.util.spec_from_file_location("amdat_torch", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        _ext = mod
    return _ext


def gsmooth(pos: torch.Tensor, box, sigma: float = 0.02, r_max: float = 4.0,
            n_bins: int = 400) -> torch.Tensor:
    """Gaussian-smoothed unordered pair histogram h[n_bins] (float64) summed over
    the frames of pos [frames][atoms][3] (float32, CUDA); differentiable in pos."""
    return ext().gsmooth(pos, [float(b) for b in box], float(sigma), float(r_max), int(n_bins))


def structure_factor_raw(pos: torch.Tensor, box, kmax: float = 12.0, dk: float = 0.1) -> torch.Tensor:
    """sum over frames and shell vectors of |rho_k|^2 / H_s for every half-space
    lattice vector with |k| <= kmax, shells of width dk (float64); differentiable."""
    return ext().structure_factor(pos, [float(b) for b in box], float(kmax), float(dk))


def lattice(pos: torch.Tensor, box, kmax: float = 12.0, dk: float = 0.1):
    """(vectors [n_k][3] int32, shell offsets [n_shells+1] int32) of structure_factor_raw."""
    kv, off = ext().lattice(pos, [float(b) for b in box], float(kmax), float(dk))
    return kv, off


def g_of_r(h: torch.Tensor, n_atoms: int, n_frames: int, box, r_max: float = 4.0) -> torch.Tensor:
    """Smoothed g(r_b) = h_b / (frames * N/2 * (N-1)/V * 4 pi r_b^2): the ideal-gas
    density of unordered pairs per unit distance at the bin centre."""
    n_bins = h.shape[0]
    dr = r_max / n_bins
    r = (torch.arange(n_bins, dtype=torch.float64, device=h.device) + 0.5) * dr
    vol = float(box[0]) * float(box[1]) * float(box[2])
    ideal = n_frames * 0.5 * n_atoms * (n_atoms - 1) / vol * 4.0 * math.pi * r * r
    return h / ideal


def s_of_k(s_raw: torch.Tensor, n_atoms: int, n_frames: int) -> torch.Tensor:
    """S(k) per shell = <|rho_k|^2> / N."""
    return s_raw / (n_frames * n_atoms)


def structure_loss(pos: torch.Tensor, box, g_target: torch.Tensor, s_target: torch.Tensor,
                   sigma: float = 0.02, r_max: float = 4.0, n_bins: int = 400, kmax: float = 12.0,
                   dk: float = 0.1):
    """sum_r (g(r) - g_target(r))^2 + sum_k (S(k) - S_target(k))^2 and its parts."""
    F, N = pos.shape[0], pos.shape[1]
    g = g_of_r(gsmooth(pos, box, sigma, r_max, n_bins), N, F, box, r_max)
    s = s_of_k(structure_factor_raw(pos, box, kmax, dk), N, F)
    loss = ((g - g_target) ** 2).sum() + ((s - s_target) ** 2).sum()
    return loss, g, s
