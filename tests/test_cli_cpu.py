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
