"""Seeded synthetic trajectories in the shapes AMDAT analyses consume.

A trajectory is an unwrapped Gaussian random walk in a cubic periodic box:
initial positions uniform in [0, L)^3, and between consecutive frames every
coordinate moves by sigma * sqrt(dt) * N(0, 1), where dt is the time between
the two frames of the time scheme.  The walk is generated in FP64 and rounded
once to FP32, the precision AMDAT stores coordinates in
(src/coordinate.h:16), so the dump written by :func:`write_custom_dump`
(``%.9g``, FP32-exact) is read back by AMDAT's ``custom`` reader
(src/system.cpp:1026-1360) into exactly the same FP32 values this module
returns.

Frame times follow AMDAT's ``create_timelist`` (src/system.cpp:3542-3566).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class TimeScheme:
    """AMDAT time scheme line (src/system.cpp:83-140).

    kind: "exponential", "linear" or "snapshot".
    """
    kind: str = "exponential"
    n_exponentials: int = 1
    n_exponential_steps: int = 1
    exp_base: float = 1.0
    frt: int = 0
    first_exponent: int = 0
    time_unit: float = 1.0

    @staticmethod
    def exponential(blocks, steps, base, frt=0, first_exponent=0, unit=1.0):
        return TimeScheme("exponential", blocks, steps, base, frt, first_exponent, unit)

    @staticmethod
    def linear(n_frames, unit=1.0):
        return TimeScheme("linear", n_frames - 1, 1, 1.0, 0, 0, unit)

    @property
    def n_timesteps(self) -> int:
        if self.kind == "exponential":
            return self.n_exponential_steps * self.n_exponentials + 1
        if self.kind == "linear":
            return self.n_exponentials + 1
        return 1

    def script_line(self) -> str:
        if self.kind == "exponential":
            return (f"exponential {self.n_exponentials} {self.n_exponential_steps} "
                    f"{self.exp_base!r} {self.frt} {self.first_exponent} {self.time_unit!r}")
        if self.kind == "linear":
            return f"linear {self.n_timesteps} {self.time_unit!r}"
        return "snapshot"

    def timelist(self) -> np.ndarray:
        """Frame times, computed like System::create_timelist (FP32 store)."""
        t = np.zeros(self.n_timesteps, dtype=np.float32)
        ii = 0
        block_start = np.float32(0.0)
        unit = np.float32(self.time_unit)
        base = float(np.float32(self.exp_base)) if self.kind != "exponential" else self.exp_base
        for _ in range(self.n_exponentials if self.kind != "snapshot" else 0):
            for e in range(1, self.n_exponential_steps + 1):
                ii += 1
                p = math.pow(base, e - 1 + self.first_exponent)
                if p <= e:
                    t[ii] = np.float32(block_start + np.float32(e) * unit)
                else:
                    t[ii] = np.float32(block_start + np.float32(math.floor(p)) * unit)
            block_start = t[ii]
        return t


@dataclass
class Trajectory:
    """FP32 unwrapped positions [frames][atoms][3], box lengths and types."""
    unwrapped: np.ndarray
    box: np.ndarray                      # [3] box lengths (constant volume)
    box_lo: np.ndarray                   # [3] lower box bounds
    types: np.ndarray                    # [atoms] int32 type index (0-based)
    scheme: TimeScheme = field(default_factory=TimeScheme)
    type_names: tuple = ("1",)
    species: tuple = (("particle", None),)
    # wrapped positions as a trajectory file gave them (xyz input); None means
    # derived from the unwrapped ones
    wrapped_given: np.ndarray | None = None
    # the trajectory file type it is written as: "custom", "custom_byid" or "xyz"
    file_format: str = "custom"

    @property
    def n_frames(self):
        return self.unwrapped.shape[0]

    @property
    def n_atoms(self):
        return self.unwrapped.shape[1]

    def wrapped(self) -> np.ndarray:
        """Wrapped coordinates derived from unwrapped ones exactly as AMDAT's
        custom reader does (src/system.cpp, ``calc_wrapped``):
        c = u - L * floor((u - lo) / L), every operation in FP32."""
        if self.wrapped_given is not None:
            return self.wrapped_given
        u = self.unwrapped.astype(np.float32)
        lo = self.box_lo.astype(np.float32)
        L = self.box.astype(np.float32)
        f = np.floor(((u - lo).astype(np.float32) / L).astype(np.float32)).astype(np.float32)
        return (u - (L * f).astype(np.float32)).astype(np.float32)


def random_walk(n_atoms: int, box: float, scheme: TimeScheme, sigma: float, seed: int,
                type_fractions=(1.0,), type_names=None, time_scaled=True, type_mobility=None) -> Trajectory:
    """Unwrapped FP64 random walk, rounded to FP32.

    sigma is the per-frame step for unit time; with time_scaled the step of a
    frame interval dt is sigma*sqrt(dt) (the convention of the exponential
    schemes), otherwise sigma per frame.  type_mobility scales the step of each
    atom type (a mixture of mobilities gives a non-Gaussian self van Hove).
    """
    rng = np.random.default_rng(seed)
    T = scheme.n_timesteps
    times = scheme.timelist().astype(np.float64)
    counts = np.floor(np.asarray(type_fractions) * n_atoms).astype(int)
    counts[-1] = n_atoms - counts[:-1].sum()
    types = np.repeat(np.arange(len(counts), dtype=np.int32), counts)
    scale = np.ones((n_atoms, 1)) if type_mobility is None else np.asarray(type_mobility, np.float64)[types][:, None]
    pos = np.empty((T, n_atoms, 3), dtype=np.float64)
    pos[0] = rng.random((n_atoms, 3)) * box
    for t in range(1, T):
        dt = times[t] - times[t - 1]
        step = sigma * math.sqrt(max(dt, 0.0)) if time_scaled else sigma
        pos[t] = pos[t - 1] + step * scale * rng.standard_normal((n_atoms, 3))
    names = tuple(type_names or [str(i + 1) for i in range(len(counts))])
    return Trajectory(unwrapped=pos.astype(np.float32),
                      box=np.full(3, box, dtype=np.float32),
                      box_lo=np.zeros(3, dtype=np.float32),
                      types=types, scheme=scheme, type_names=names)


def write_custom_dump(traj: Trajectory, path: str, shuffle_seed: int | None = None) -> None:
    """LAMMPS ``custom`` dump with columns ``id type xu yu zu`` (FP32-exact).

    With shuffle_seed the atom lines of every frame are written in a seeded
    random order (the layout ``custom_byid`` reads; ids stay 1..N)."""
    lo = traj.box_lo.astype(np.float64)
    hi = lo + traj.box.astype(np.float64)
    ids = np.arange(1, traj.n_atoms + 1)
    tnames = np.asarray(traj.type_names)[traj.types]
    rng = np.random.default_rng(shuffle_seed) if shuffle_seed is not None else None
    with open(path, "w") as f:
        for t in range(traj.n_frames):
            f.write(f"ITEM: TIMESTEP\n{t}\nITEM: NUMBER OF ATOMS\n{traj.n_atoms}\n")
            f.write("ITEM: BOX BOUNDS pp pp pp\n")
            for d in range(3):
                f.write(f"{np.float32(lo[d]):.9g} {np.float32(hi[d]):.9g}\n")
            f.write("ITEM: ATOMS id type xu yu zu\n")
            u = traj.unwrapped[t]
            lines = [f"{i} {n} {x:.9g} {y:.9g} {z:.9g}\n"
                     for i, n, (x, y, z) in zip(ids, tnames, u.tolist())]
            if rng is not None:
                lines = [lines[k] for k in rng.permutation(len(lines))]
            f.writelines(lines)


def write_trajectory(traj: Trajectory, path: str, shuffle_seed: int = 0) -> None:
    """Write traj in its file_format (xyz, custom, or custom with shuffled lines)."""
    if traj.file_format == "xyz":
        write_xyz(traj, path)
    elif traj.file_format == "custom_byid":
        write_custom_dump(traj, path, shuffle_seed=shuffle_seed)
    else:
        write_custom_dump(traj, path)


def write_xyz(traj: Trajectory, path: str) -> None:
    """xyz trajectory (src/system.cpp:610-700): atom count, a comment line, then
    ``type x y z`` per atom with the wrapped FP32 coordinates (``%.9g``)."""
    w = traj.wrapped()
    tnames = np.asarray(traj.type_names)[traj.types]
    with open(path, "w") as f:
        for t in range(traj.n_frames):
            f.write(f"{traj.n_atoms}\nAtoms. Timestep: {t}\n")
            f.writelines(f"{n} {x:.9g} {y:.9g} {z:.9g}\n" for n, (x, y, z) in zip(tnames, w[t].tolist()))


def unwrap_from_wrapped(wrapped: np.ndarray, box: np.ndarray) -> np.ndarray:
    """Trajectory::unwrap (src/trajectory.cpp:236-271) in FP32: u(0) = w(0), then
    u(t) = u(t-1) + d - L * int(d / (0.55 L)) with d = w(t) - w(t-1)."""
    w = wrapped.astype(np.float32)
    L = box.astype(np.float32)
    den = (L * np.float32(0.55)).astype(np.float32)
    u = np.empty_like(w)
    u[0] = w[0]
    for t in range(1, w.shape[0]):
        d = (w[t] - w[t - 1]).astype(np.float32)
        q = np.trunc((d / den).astype(np.float32)).astype(np.float32)
        u[t] = (u[t - 1] + (d - (L * q).astype(np.float32)).astype(np.float32)).astype(np.float32)
    return u


def as_xyz_input(traj: Trajectory) -> Trajectory:
    """The trajectory an xyz file of traj reads back as: the wrapped positions
    as written and the unwrapped ones derived from them by the reader."""
    w = traj.wrapped()
    return Trajectory(unwrapped=unwrap_from_wrapped(w, traj.box), box=traj.box, box_lo=traj.box_lo,
                      types=traj.types, scheme=traj.scheme, type_names=traj.type_names,
                      species=traj.species, wrapped_given=w, file_format="xyz")


def system_header(traj: Trajectory, dump_path: str, fmt: str | None = None) -> str:
    """AMDAT ``system`` block for a dump written by write_custom_dump.

    One species per atom type, one atom per molecule, so species i is the
    contiguous run of atoms of type i (the custom reader requires atoms
    grouped by species in declaration order, src/system.cpp:1026).
    """
    fmt = fmt or traj.file_format
    ntypes = len(traj.type_names)
    counts = np.bincount(traj.types, minlength=ntypes)
    species = " ".join(f"sp{i + 1} {counts[i]}" for i in range(ntypes))
    lines = ["system", fmt, dump_path, traj.scheme.script_line(), species,
             " ".join(traj.type_names)]
    for i in range(ntypes):
        lines.append(" ".join("1" if j == i else "0" for j in range(ntypes)))
    if fmt == "xyz":
        # System::xyz_prep (src/system.cpp:389-407): box lengths, then bounds
        lo = traj.box_lo.astype(np.float32)
        hi = (traj.box_lo.astype(np.float64) + traj.box.astype(np.float64)).astype(np.float32)
        lines.append(" ".join(f"{np.float32(v):.9g}" for v in traj.box))
        lines.append(" ".join(f"{lo[d]:.9g} {hi[d]:.9g}" for d in range(3)))
    return "\n".join(lines) + "\n"
