"""The reference-side binding, compiled and run: tests/binding/gpu_msd_binding.cpp
subclasses AMDAT's own Analysis interface as a GPU-backed mean-square
displacement, compiles against AMDAT's unmodified headers, links AMDAT's own
objects (Control, System, Trajectory_List, the readers) and libamdat_gb300.so,
runs AMDAT's Control on the exponential golden case's system block, and must
write the msd.dat the reference binary wrote: the same times, values within
2e-3 relative of the reference's FP32 sums (the engine sums in compensated FP32
with FP64 reductions)."""
import glob
import os
import subprocess

import pytest

from golden.make_golden import load
from amdat_gb300 import synth

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def binding(tmp_path_factory, engine_mod):
    from oracle import build_oracle
    ref = build_oracle.reference_source()
    if ref is None:
        pytest.skip("reference sources not present (baseline/_ref/src or AMDAT_REFERENCE)")
    binary = build_oracle.build_reference()
    out = os.path.dirname(binary)
    objs = [o for o in sorted(glob.glob(os.path.join(out, "obj", "*.o")))
            if os.path.basename(o) != "amdat.o"]
    exe = str(tmp_path_factory.mktemp("binding") / "gpu_msd_binding")
    lib = os.path.join(REPO, "amdat_gb300", "_lib")
    cmd = (["g++", "-std=c++17", "-O2", "-fopenmp", "-w",
            "-I", os.path.join(ref, "src"), "-I", os.path.join(out, "gen"),
            "-I", os.path.join(out, "gen", "generated"),
            "-I", os.path.join(ref, "third_party", "voro++-0.4.6", "src"),
            "-I", os.path.join(ref, "third_party", "xdrfile-1.1b", "include"),
            "-I", os.path.join(REPO, "include"),
            os.path.join(HERE, "binding", "gpu_msd_binding.cpp")] + objs
           + ["-o", exe, "-L", lib, "-lamdat_gb300", f"-Wl,-rpath,{lib}", "-lm"])
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.parametrize("case,list_name,golden", [("exp_small", "all", "msd.dat"),
                                                   ("exp_frt", "all", "msd.dat"),
                                                   ("lin_binary", "a", "msd_a.dat")])
def test_binding_writes_reference_msd(binding, tmp_path, case, list_name, golden):
    traj, script, outs = load(case)
    dump = str(tmp_path / "traj.dump")
    synth.write_trajectory(traj, dump)
    lists = script.split("msd ")[0]  # the script's list commands, before its analyses
    with open(tmp_path / "in.amdat", "w") as f:
        f.write(synth.system_header(traj, dump) + lists)
    r = subprocess.run([binding, "in.amdat", list_name, "msd.dat"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:] + r.stdout[-2000:]
    got = open(tmp_path / "msd.dat").read().splitlines()
    ref = outs[golden].splitlines()
    assert got[0] == ref[0] and len(got) == len(ref)
    for a, b in zip(got[1:], ref[1:]):
        ta, va = a.split("\t")
        tb, vb = b.split("\t")
        # times: the reference objects built on this machine form them (aarch64 gcc
        # contracts the time line's multiply-add, x86-64 does not), the file came
        # from an x86-64 build
        assert abs(float(ta) - float(tb)) <= 1e-5 * max(abs(float(tb)), 1e-12), (a, b)
        assert abs(float(va) - float(vb)) <= 2e-3 * max(abs(float(vb)), 1e-12), (a, b)
