"""Pins the oracle: its reference-arithmetic mode must reproduce, digit for
digit, the output files the reference AMDAT binary wrote for the golden
trajectories (tests/golden/*, made by tests/golden/make_golden.py).  The FP64
mode must agree with them to the reference's own FP32 accuracy."""
import math

import numpy as np
import pytest

from amdat_files import tokens
from oracle import oracle as orc
from oracle_script import OracleRun
from golden.make_golden import CASES, load


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_ref32_matches_reference_files(case, qvectors):
    traj, script, golden = load(case)
    files = OracleRun(traj, qvectors, orc.REF32).run(script)
    assert sorted(files) == sorted(golden)
    for name, text in golden.items():
        got, want = tokens(files[name]), tokens(text)
        assert len(got) == len(want), name
        bad = [(i, g, w) for i, (g, w) in enumerate(zip(got, want)) if g != w]
        assert not bad, f"{case}/{name}: {len(bad)} tokens differ, first {bad[:5]}"


def _num(tok):
    try:
        return float(tok)
    except ValueError:
        return None


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_f64_close_to_reference_files(case, qvectors):
    """FP64 mode vs the reference's FP32 results: agreement to ~1e-3 relative
    (the reference accumulates in FP32 and forms k.r in FP32)."""
    traj, script, golden = load(case)
    files = OracleRun(traj, qvectors, orc.F64).run(script)
    for name, text in golden.items():
        got, want = tokens(files[name]), tokens(text)
        assert len(got) == len(want)
        for g, w in zip(got, want):
            fg, fw = _num(g), _num(w)
            if fg is None or fw is None:
                assert g == w
                continue
            if math.isnan(fw):
                assert math.isnan(fg)
                continue
            assert abs(fg - fw) <= 2e-3 * max(abs(fw), 1e-2), (name, g, w)


def test_pair_counts():
    """Pair enumeration counts for the benchmark schemes (system.cpp:4090-4179)."""
    from amdat_gb300.synth import TimeScheme
    s = orc.scheme(TimeScheme.exponential(10, 27, 1.3, 0, 0, 0.005))
    g, t0, t1 = orc.pairs(s, 0)
    assert len(g) == 316 and orc.n_timegaps(s) == 37
    s = orc.scheme(TimeScheme.linear(400, 1.0))
    g, t0, t1 = orc.pairs(s, 0)
    # gap 0: 399 pairs; gaps 1..398 drop the last start frame; last gap (0, 399)
    assert len(g) == 399 + 398 * 399 // 2 + 1
    assert (t1 < 400).all() and (t1 - t0 >= 0).all()
    s = orc.scheme(TimeScheme.exponential(12, 30, 1.25, 0, 0, 1.0))
    assert len(orc.pairs(s, 0)[0]) == 12 * 30 + 66 + 1
