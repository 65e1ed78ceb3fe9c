"""Writes tests/golden/qvectors3d.npz from the reference's q-vector tables.

AMDAT's Wave_Vectors(System*, plane, L) reads shell m (m = 0..98) from the
text file qvectors3d/qvector.(m+2) (src/wave_vectors.cpp:430-480); each line
is one integer lattice vector n, the wave vector being n * 2*pi/L.  Those
files ship zipped in src/qvectors/qvectors.zip.  This script stores the same
integers as a compact fixture (int8 [K,3] plus shell offsets) so the parity
tests can use the reference's exact wave vectors on machines without the
reference tree.  Run: python tests/golden/make_qvectors.py /path/to/AMDAT
"""
import os
import sys
import zipfile

import numpy as np

if len(sys.argv) != 2:
    raise SystemExit("usage: make_qvectors.py <AMDAT source tree>")
ref = sys.argv[1]
z = zipfile.ZipFile(os.path.join(ref, "src", "qvectors", "qvectors.zip"))
vecs, off = [], [0]
for m in range(99):
    vals = z.read(f"qvectors3d/qvector.{m + 2:03d}").decode().split()
    n = np.asarray([float(v) for v in vals], dtype=np.float64).reshape(-1, 3)
    assert np.all(n == np.round(n)) and np.abs(n).max() < 128
    vecs.append(n.astype(np.int8))
    off.append(off[-1] + len(n))
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "qvectors3d.npz")
np.savez_compressed(out, n=np.concatenate(vecs), offsets=np.asarray(off, np.int32))
print(out, off[-1], "vectors")
