"""Generates the golden parity fixtures under tests/golden/<case>/.

For each case: a seeded synthetic trajectory (amdat_gb300.synth) is written as
a LAMMPS custom dump, the reference AMDAT binary (built from its own sources by
oracle/ref.mk) runs an input script of the hot-path commands on it, and the
fixture keeps
  traj.npz    FP32 unwrapped positions, box, types, time scheme
  script.in   the command part of the input script (after the system block)
  *.dat       the reference's output files, verbatim.
The reference tree itself is not needed to use the fixtures.
Run: python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from amdat_gb300 import synth  # noqa: E402
from oracle import build_oracle  # noqa: E402

CASES = {
    # single species, blocked-exponential scheme, all seven hot commands
    "exp_small": dict(
        n=216, box=8.0, sigma=0.5, seed=11, fractions=(1.0,),
        scheme=synth.TimeScheme.exponential(4, 8, 1.3, 0, 0, 0.005),
        commands="""create_list all
all
msd ./msd.dat
list all
ngp ./ngp.dat
list all
isfs ./isfs.dat 10 12 xyz 0
list all
isfs ./isfs_fb.dat 14 15 xyz 0 1
list all
vhs ./vhs.dat 0.5 50
list all
structure_factor ./sk.dat symmetric xyz 0 -1
list all
isf ./isf.dat auto symmetric xyz 0 0 20
list all
isf ./isf_fb.dat auto symmetric xyz 1 3 6
list all
rdf ./rdf.dat symmetric 100 -1 0
list all
limit 3
msd ./msd_lim.dat
list all
isfs ./isfs_lim.dat 12 12 xyz 0 1
list all
"""),
    # binary 80:20 mixture, linear scheme (its dropped-last-start quirk), type lists
    "lin_binary": dict(
        n=250, box=7.0, sigma=0.08, seed=22, fractions=(0.8, 0.2), time_scaled=False,
        scheme=synth.TimeScheme.linear(20, 1.0),
        commands="""create_list all
all
create_list a
type_system 1
create_list b
type_system 2
msd ./msd_a.dat
list a
ngp ./ngp_b.dat
list b
isfs ./isfs_a.dat 6 9 xyz 0
list a
vhs ./vhs.dat 1.0 40
list all
structure_factor ./sk_b.dat symmetric xyz 0 -1
list b
isf ./isf.dat auto symmetric xyz 0 0 15
list all
rdf ./rdf.dat symmetric 60 -1 0
list all
rdf ./rdf_a.dat symmetric 30 -1 2.5
list a
"""),
    # frt = 1, first_exponent = 2, base 1.5 (other branches of create_timelist)
    "exp_frt": dict(
        n=64, box=5.0, sigma=0.3, seed=33, fractions=(1.0,),
        scheme=synth.TimeScheme.exponential(5, 6, 1.5, 1, 2, 0.01),
        commands="""create_list all
all
msd ./msd.dat
list all
ngp ./ngp.dat
list all
isfs ./isfs.dat 3 5 xyz 0 1
list all
vhs ./vhs.dat 0.8 20
list all
isf ./isf.dat auto symmetric xyz 1 0 8
list all
"""),
    # sibling displacement analyses on the same scheduler (exponential and linear)
    "siblings": dict(
        n=150, box=6.5, sigma=0.4, seed=44, fractions=(0.7, 0.3),
        scheme=synth.TimeScheme.exponential(4, 8, 1.3, 0, 0, 0.005),
        commands="""create_list all
all
create_list b
type_system 2
msd_2d ./msd2d_xy.dat xy
list all
msd_2d ./msd2d_yz.dat yz
list b
mean_displacement ./md.dat
list all
u2dist ./u2_in_block.dat 40 2.0 5
list all
u2dist ./u2_cross.dat 25 3.0 9
list b
u2dist ./u2_last.dat 30 4.0 11
list all
displacement_dist ./dd.dat 2 30 1.5 3
list all
limit 2
u2dist ./u2_lim.dat 20 2.0 10
list all
mean_displacement ./md_lim.dat
list all
"""),
    # S(k) from a stored g(r) (rdf with the \\s flag, then structure_factor_from_rdf)
    "sk_from_rdf": dict(
        n=400, box=8.0, sigma=0.2, seed=66, fractions=(1.0,), time_scaled=False,
        scheme=synth.TimeScheme.linear(6, 1.0),
        commands="""create_list all
all
rdf ./rdf.dat symmetric 80 -1 0 \\sg1
list all
structure_factor_from_rdf ./sk_rdf.dat 40 g1
rdf ./rdf2.dat symmetric 50 0 3.0 \\sg2
list all
structure_factor_from_rdf ./sk_rdf2.dat 25 g2
"""),
    # xyz input (wrapped coordinates only; the reader unwraps them), binary mixture
    "xyz_binary": dict(
        n=180, box=6.0, sigma=0.6, seed=77, fractions=(0.6, 0.4), fmt="xyz",
        scheme=synth.TimeScheme.exponential(3, 8, 1.4, 0, 0, 0.01),
        commands="""create_list all
all
create_list b
type_system 2
msd ./msd.dat
list all
ngp ./ngp_b.dat
list b
isfs ./isfs.dat 8 10 xyz 0
list all
vhs ./vhs.dat 0.5 30
list all
structure_factor ./sk.dat symmetric xyz 0 -1
list all
isf ./isf.dat auto symmetric xyz 0 0 10
list all
rdf ./rdf.dat symmetric 60 -1 0
list all
"""),
    # custom_byid: atom lines shuffled in every frame, placed by their id column
    "byid_binary": dict(
        n=160, box=6.0, sigma=0.3, seed=88, fractions=(0.5, 0.5), fmt="custom_byid",
        scheme=synth.TimeScheme.exponential(3, 6, 1.4, 0, 0, 0.01),
        commands="""create_list all
all
create_list a
type_system 1
msd ./msd_a.dat
list a
ngp ./ngp.dat
list all
vhs ./vhs.dat 0.5 30
list all
rdf ./rdf.dat symmetric 40 -1 0
list all
isfs ./isfs.dat 8 9 xyz 0
list a
"""),
    # spatial bins (create_bin_list): per-bin MSD and F_s, membership at the start
    # frame (bin_list <bins> <list>) or at both frames (persistence flag 1)
    "bins": dict(
        n=300, box=6.0, sigma=0.25, seed=99, fractions=(0.7, 0.3),
        scheme=synth.TimeScheme.exponential(3, 6, 1.4, 0, 0, 0.01),
        commands="""create_list all
all
create_list b
type_system 2
create_bin_list slabs
all 1 1 3
msd ./msd_slabs.dat
bin_list slabs all
isfs ./isfs_slabs.dat 8 9 xyz 0
bin_list slabs all
msd ./msd_persist.dat
bin_list slabs all 1
isfs ./isfs_persist.dat 8 8 xyz 0 1
bin_list slabs b 1
create_bin_list cells
region 2 1 2 1.0 5.0 0 0 0 4.0
msd ./msd_cells.dat
bin_list cells b
isfs ./isfs_cells.dat 7 7 xyz 0 1
bin_list cells all
"""),
    # distance bin lists (trajectory, point, plane with each direction) as targets of
    # msd, isfs and structure_factor, and rectangular bins as structure_factor targets
    "bins_distance": dict(
        n=240, box=6.0, sigma=0.25, seed=131, fractions=(0.9, 0.1),
        scheme=synth.TimeScheme.exponential(3, 6, 1.4, 0, 0, 0.01),
        commands="""create_list all
all
create_list b
type_system 2
create_bin_list near_b
distance trajectory all b 0.5 4
msd ./msd_near.dat
bin_list near_b all
isfs ./isfs_near.dat 8 9 xyz 0
bin_list near_b all 1
structure_factor ./sk_near.dat symmetric xyz 0 -1
bin_list near_b all
create_bin_list shells
distance point all 3.0 2.5 1.0 0.75 3
msd ./msd_shells.dat
bin_list shells all
structure_factor ./sk_shells.dat symmetric xyz 0 -1
bin_list shells all
create_bin_list zlayers
distance plane average all z 2.0 0.8 3
msd ./msd_zavg.dat
bin_list zlayers all
create_bin_list xabove
distance plane above all x 1.5 1.0 4
msd ./msd_xabove.dat
bin_list xabove all 1
create_bin_list ybelow
distance plane below all y 4.0 1.25 3
isfs ./isfs_ybelow.dat 7 7 xyz 0
bin_list ybelow all
create_bin_list grid
all 1 2 1
structure_factor ./sk_grid.dat symmetric xyz 0 -1
bin_list grid all
"""),
    # msd_2d and mean_displacement per bin (static and persistent) and of a
    # fast-particle list
    "bins_axes": dict(
        n=260, box=6.0, sigma=0.25, seed=121, fractions=(0.6, 0.4), mobility=(1.0, 3.0),
        scheme=synth.TimeScheme.exponential(3, 6, 1.4, 0, 0, 0.01),
        commands="""create_list all
all
create_list b
type_system 2
create_bin_list slabs
all 1 2 2
msd_2d ./msd2d_slabs.dat xy
bin_list slabs all
mean_displacement ./md_slabs.dat
bin_list slabs b 1
msd_2d ./msd2d_p.dat yz
bin_list slabs all 1
find_fast_fixedthreshold quick ./quick.dat 5 0.02
list all
mean_displacement ./md_quick.dat
list quick
msd_2d ./msd2d_quick.dat xz
list quick
"""),
    # a two-mobility mixture: self van Hove vs its Gaussian (compare_gaussian), the
    # fast particles per block (find_fast, find_fast_fixedthreshold) and analyses
    # of those time-dependent lists
    "fast": dict(
        n=400, box=7.0, sigma=0.12, seed=111, fractions=(0.75, 0.25), mobility=(1.0, 4.0),
        scheme=synth.TimeScheme.exponential(4, 8, 1.3, 0, 0, 0.01),
        commands="""create_list all
all
create_list b
type_system 2
vhs ./vhs.dat 0.6 60
list all
compare_gaussian ./gc.dat
list all
find_fast fast ./fast_count.dat
list all
msd ./msd_fast.dat
list fast
ngp ./ngp_fast.dat
list fast
isfs ./isfs_fast.dat 8 9 xyz 0
list fast
find_fast_fixedthreshold quick ./fast_fixed.dat 6 0.05
list b
msd ./msd_quick.dat
list quick
compare_gaussian ./gc_t5.dat 5
list b
"""),
    "siblings_lin": dict(
        n=120, box=6.0, sigma=0.1, seed=55, fractions=(1.0,), time_scaled=False,
        scheme=synth.TimeScheme.linear(16, 1.0),
        commands="""create_list all
all
msd_2d ./msd2d_xz.dat xz
list all
mean_displacement ./md.dat
list all
u2dist ./u2.dat 25 0.5 4
list all
displacement_dist ./dd.dat 4 20 1.0 14
list all
"""),
}


def make(case: str) -> None:
    cfg = CASES[case]
    ref = build_oracle.build_reference()
    if ref is None:
        raise SystemExit("reference source tree not found; set AMDAT_REFERENCE")
    traj = synth.random_walk(cfg["n"], cfg["box"], cfg["scheme"], cfg["sigma"], cfg["seed"],
                             type_fractions=cfg["fractions"],
                             time_scaled=cfg.get("time_scaled", True),
                             type_mobility=cfg.get("mobility"))
    fmt = cfg.get("fmt", "custom")
    if fmt == "xyz":
        traj = synth.as_xyz_input(traj)
    traj.file_format = fmt
    out_dir = os.path.join(HERE, case)
    os.makedirs(out_dir, exist_ok=True)
    s = cfg["scheme"]
    extra = {"wrapped": traj.wrapped_given} if fmt == "xyz" else {}
    np.savez_compressed(os.path.join(out_dir, "traj.npz"), unwrapped=traj.unwrapped,
                        box=traj.box, box_lo=traj.box_lo, types=traj.types, fmt=np.asarray(fmt), **extra,
                        scheme=np.asarray([s.n_exponentials, s.n_exponential_steps, s.frt,
                                           s.first_exponent]),
                        scheme_f=np.asarray([s.exp_base, s.time_unit]),
                        scheme_kind=np.asarray(s.kind))
    with open(os.path.join(out_dir, "script.in"), "w") as f:
        f.write(cfg["commands"])
    with tempfile.TemporaryDirectory() as tmp:
        dump = os.path.join(tmp, "traj.dump")
        synth.write_trajectory(traj, dump)
        with open(os.path.join(tmp, "in.amdat"), "w") as f:
            f.write(synth.system_header(traj, dump) + cfg["commands"])
        r = subprocess.run([ref, "-i", "in.amdat"], cwd=tmp, capture_output=True, text=True)
        if r.returncode != 0:
            raise SystemExit(f"reference failed on {case}:\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        for fn in sorted(os.listdir(tmp)):
            if fn.endswith((".dat", ".bindata")):
                shutil.copy(os.path.join(tmp, fn), os.path.join(out_dir, fn))
    print(case, "->", out_dir)


def load(case: str):
    """Fixture loader: (Trajectory, script text, {name: text})."""
    d = os.path.join(HERE, case)
    z = np.load(os.path.join(d, "traj.npz"))
    kind = str(z["scheme_kind"])
    a, b, frt, fe = (int(v) for v in z["scheme"])
    base, unit = (float(v) for v in z["scheme_f"])
    if kind == "linear":
        s = synth.TimeScheme.linear(a + 1, unit)
    else:
        s = synth.TimeScheme.exponential(a, b, base, frt, fe, unit)
    ntypes = int(z["types"].max()) + 1
    traj = synth.Trajectory(unwrapped=z["unwrapped"], box=z["box"], box_lo=z["box_lo"],
                            types=z["types"], scheme=s,
                            type_names=tuple(str(i + 1) for i in range(ntypes)),
                            wrapped_given=z["wrapped"] if "wrapped" in z.files else None,
                            file_format=str(z["fmt"]) if "fmt" in z.files else "custom")
    with open(os.path.join(d, "script.in")) as f:
        script = f.read()
    outs = {fn: open(os.path.join(d, fn)).read() for fn in sorted(os.listdir(d))
            if fn.endswith((".dat", ".bindata"))}
    return traj, script, outs


if __name__ == "__main__":
    for c in (sys.argv[1:] or list(CASES)):
        make(c)
