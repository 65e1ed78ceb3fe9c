"""Input faults of the command-line driver, checked without a GPU: the driver
reports them as an error message and exit status 1 (the reference prints and
calls exit()).  Faults are planted in the inputs, never on a device."""
import os

import numpy as np
import pytest

from amdat_gb300 import synth
from cli_util import CLI, run_cli


@pytest.fixture(scope="module")
def built():
    from amdat_gb300 import build
    build.build()
    assert os.path.exists(CLI)


@pytest.fixture()
def traj():
    return synth.random_walk(20, 4.0, synth.TimeScheme.exponential(2, 3, 1.3, 0, 0, 0.01), 0.3, seed=3)


def test_wrong_atom_count(built, traj, tmp_path):
    synth.write_custom_dump(traj, str(tmp_path / "traj.dump"))
    bad = synth.Trajectory(unwrapped=traj.unwrapped[:, :19], box=traj.box, box_lo=traj.box_lo,
                           types=traj.types[:19], scheme=traj.scheme)
    # header declares 19 atoms, the dump holds 20 per frame
    with open(tmp_path / "in.amdat", "w") as f:
        f.write(synth.system_header(bad, str(tmp_path / "traj.dump")))
    import subprocess
    r = subprocess.run([CLI, "-i", "in.amdat"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "inconsistent with user input: 20 != 19" in r.stderr


def test_missing_trajectory(built, traj, tmp_path):
    with open(tmp_path / "in.amdat", "w") as f:
        f.write(synth.system_header(traj, str(tmp_path / "none.dump")))
    import subprocess
    r = subprocess.run([CLI, "-i", "in.amdat"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "Custom Trajectory file not found" in r.stderr


def test_truncated_trajectory(built, traj, tmp_path):
    synth.write_custom_dump(traj, str(tmp_path / "traj.dump"))
    txt = open(tmp_path / "traj.dump").read()
    open(tmp_path / "traj.dump", "w").write(txt[: len(txt) // 2])
    with open(tmp_path / "in.amdat", "w") as f:
        f.write(synth.system_header(traj, str(tmp_path / "traj.dump")))
    import subprocess
    r = subprocess.run([CLI, "-i", "in.amdat"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "ends before frame" in r.stderr


def test_bad_time_scheme_and_command(built, tmp_path):
    import subprocess
    (tmp_path / "in.amdat").write_text("system\ncustom\nx.dump\nlogarithmic 3 2\nA 1\n1\n1\n")
    r = subprocess.run([CLI, "-i", "in.amdat"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "Time scheme logarithmic not recognized" in r.stderr
    (tmp_path / "in.amdat").write_text("# comment\nbond_autocorrelation_function ./x.dat\n")
    r = subprocess.run([CLI, "-i", "in.amdat"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "not part of this engine" in r.stderr


def test_valid_script_without_gpu(built, traj, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = run_cli(traj, "create_list all\nall\nmsd ./msd.dat\nlist all\n", str(tmp_path))
    assert r.returncode == 1 and "no CUDA device" in r.stderr


def _xyz_script(traj, path, fmt="xyz", drop_box=False):
    hdr = synth.system_header(traj, path, fmt)
    if drop_box:
        hdr = "\n".join(hdr.splitlines()[:-2]) + "\n"
    return hdr


def test_xyz_input_faults(built, traj, tmp_path):
    import subprocess
    xyz = str(tmp_path / "traj.xyz")
    synth.write_xyz(traj, xyz)
    bad = synth.Trajectory(unwrapped=traj.unwrapped[:, :19], box=traj.box, box_lo=traj.box_lo,
                           types=traj.types[:19], scheme=traj.scheme)
    (tmp_path / "in.amdat").write_text(_xyz_script(bad, xyz))
    r = subprocess.run([CLI, "-i", "in.amdat"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "inconsistent with user input: 20 != 19" in r.stderr
    # the box lines are part of the xyz system block
    (tmp_path / "in.amdat").write_text(_xyz_script(traj, xyz, drop_box=True))
    r = subprocess.run([CLI, "-i", "in.amdat"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "input script ended early" in r.stderr
    (tmp_path / "in.amdat").write_text(_xyz_script(traj, xyz, drop_box=True) + "10 10\n0 10 0 10 0 10\n")
    r = subprocess.run([CLI, "-i", "in.amdat"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "bad box lines" in r.stderr
    # a type label beyond the declared atom types
    txt = open(xyz).read().splitlines()
    txt[5] = "7" + txt[5][1:]
    open(xyz, "w").write("\n".join(txt) + "\n")
    (tmp_path / "in.amdat").write_text(_xyz_script(traj, xyz))
    r = subprocess.run([CLI, "-i", "in.amdat"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "out of range" in r.stderr
    (tmp_path / "in.amdat").write_text(_xyz_script(traj, str(tmp_path / "none.xyz")))
    r = subprocess.run([CLI, "-i", "in.amdat"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "XYZ Trajectory file not found" in r.stderr


def test_xyz_valid_script_parses_without_gpu(built, traj, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    xyz = synth.as_xyz_input(traj)
    r = run_cli(xyz, "create_list all\nall\nmsd ./msd.dat\nlist all\n", str(tmp_path))
    assert r.returncode == 1 and "no CUDA device" in r.stderr


def test_xyz_unwrap_rule():
    # Trajectory::unwrap: a crossing of the periodic boundary is undone, a
    # displacement below 0.55 L is kept as it is
    box = np.array([10.0, 10.0, 10.0], np.float32)
    w = np.array([[[9.5, 0.2, 5.0]], [[0.3, 9.9, 5.0]], [[5.6, 4.0, 5.0]]], np.float32)
    u = synth.unwrap_from_wrapped(w, box)
    assert np.allclose(u[1, 0], [10.3, -0.1, 5.0], atol=1e-5)
    # a step of 5.3 (< 0.55 L) is kept; a step of -5.9 is folded by one box length
    assert np.allclose(u[2, 0], [15.6, 4.0, 5.0], atol=1e-5)


def test_custom_byid_faults(built, traj, tmp_path):
    import subprocess
    dump = str(tmp_path / "traj.dump")
    synth.write_custom_dump(traj, dump, shuffle_seed=5)
    lines = open(dump).read().splitlines()
    # frame 0's first atom line takes the id of its second: one id repeats
    a, b = lines[9].split(), lines[10].split()
    lines[9] = " ".join([b[0]] + a[1:])
    open(dump, "w").write("\n".join(lines) + "\n")
    (tmp_path / "in.amdat").write_text(synth.system_header(traj, dump, "custom_byid"))
    r = subprocess.run([CLI, "-i", "in.amdat"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "Atom ids should begin with 1" in r.stderr
    # the same file without an id column
    lines = [ln.replace("ITEM: ATOMS id type", "ITEM: ATOMS ix type") for ln in lines]
    open(dump, "w").write("\n".join(lines) + "\n")
    r = subprocess.run([CLI, "-i", "in.amdat"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "atom id data not provided" in r.stderr
