"""Helpers to run AMDAT input scripts through the engine's command-line driver."""
import os
import subprocess

import numpy as np

from amdat_gb300 import synth

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(REPO, "amdat_gb300", "_lib", "amdat_gb300")


def write_qvectors(qvec, directory):
    """Write the q-vector fixture as the reference's text files qvector.NNN."""
    n, off = qvec
    d = os.path.join(directory, "qvectors3d")
    os.makedirs(d, exist_ok=True)
    for m in range(len(off) - 1):
        with open(os.path.join(d, f"qvector.{m + 2:03d}"), "w") as f:
            for v in n[off[m]:off[m + 1]]:
                f.write(f"   {float(v[0]):.7e}   {float(v[1]):.7e}   {float(v[2]):.7e}\r\n")
    return os.path.join(d, "qvector")


def run_cli(traj, commands, directory, qvec=None, extra_env=None):
    # written in the trajectory's own file format (custom, custom_byid or xyz)
    dump = os.path.join(directory, "traj.dump")
    if not os.path.exists(dump):
        synth.write_trajectory(traj, dump)
    with open(os.path.join(directory, "in.amdat"), "w") as f:
        f.write(synth.system_header(traj, dump) + commands)
    env = dict(os.environ)
    if qvec is not None:
        env["AMDAT_QVECTORS"] = write_qvectors(qvec, directory)
    env.update(extra_env or {})
    return subprocess.run([CLI, "-i", "in.amdat"], cwd=directory, capture_output=True, text=True,
                          env=env, timeout=600)
