"""Formatting and parsing of AMDAT output files for the parity tests.

AMDAT writes numbers with a default C++ ostream (6 significant digits, %g
style), floats promoted to double, and NaN as glibc prints it on x86-64
("-nan" for the default quiet NaN of 0*inf).
"""
import math

import numpy as np


def fmt(x) -> str:
    x = float(x)
    if math.isnan(x):
        return "-nan" if math.copysign(1.0, x) < 0 else "nan"
    if math.isinf(x):
        return "-inf" if x < 0 else "inf"
    return "%g" % x


def tokens(text: str):
    return text.split()


def body_rows(text: str, skip: int = 1):
    lines = text.splitlines()[skip:]
    return [ln.split() for ln in lines if ln.strip()]


def two_col(text: str):
    """msd/ngp files: header, then time<TAB>value rows."""
    rows = body_rows(text, 1)
    return np.array([float(r[0]) for r in rows]), [r[1] for r in rows]


def correlation_2d(text: str):
    """isfs/isf files: header, a row of nominal q, then time + values rows."""
    rows = body_rows(text, 1)
    qs = rows[0]
    times = [r[0] for r in rows[1:]]
    vals = [r[1:] for r in rows[1:]]
    return qs, times, vals


def stcf(text: str):
    """vhs file: header, 'n bins', 'n times', blank, bin centres, rows."""
    lines = [ln for ln in text.splitlines()[1:] if ln.strip()]
    nb = int(lines[0].split()[0])
    nt = int(lines[1].split()[0])
    centres = lines[2].split()
    rows = [ln.split() for ln in lines[3:3 + nt]]
    return nb, nt, centres, [r[0] for r in rows], [r[1:] for r in rows]


def rdf(text: str):
    lines = [ln for ln in text.splitlines()[1:] if ln.strip()]
    return lines[0].split(), lines[1].split()


def sk(text: str):
    lines = [ln for ln in text.splitlines()[2:] if ln.strip()]
    return [ln.split() for ln in lines]


def ulp_close(a: str, b: str, digits_slack: int = 0) -> bool:
    """Equal as printed, or (with slack) within one unit of the 6th digit."""
    if a == b:
        return True
    if digits_slack == 0:
        return False
    try:
        fa, fb = float(a), float(b)
    except ValueError:
        return False
    if math.isnan(fa) or math.isnan(fb):
        return math.isnan(fa) and math.isnan(fb)
    scale = max(abs(fa), abs(fb))
    if scale == 0:
        return True
    return abs(fa - fb) <= digits_slack * 10 ** (math.floor(math.log10(scale)) - 5) * 1.0001
