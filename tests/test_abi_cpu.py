"""CPU checks of the C ABI: the library loads and exports every function the
header declares; the host-only scheduler entry points agree with the oracle;
GPU entry points report a status code (never exit) when no device exists."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from amdat_gb300 import synth
from oracle import oracle as orc

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                   "amdat_gb300.h")


@pytest.fixture(scope="module")
def E():
    from amdat_gb300 import build
    build.build()
    from amdat_gb300 import engine
    return engine


def declared():
    txt = open(HDR).read()
    return sorted(set(re.findall(r"^(?:amdat_status|const char\*)\s+(amdat_\w+)\s*\(", txt, re.M)))


def test_every_declared_symbol_exported(E):
    names = declared()
    assert len(names) >= 25
    lib = E.lib()
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(E.EXPORTED)


SCHEMES = [
    synth.TimeScheme.exponential(10, 27, 1.3, 0, 0, 0.005),
    synth.TimeScheme.exponential(4, 8, 1.3, 0, 0, 0.005),
    synth.TimeScheme.exponential(5, 6, 1.5, 1, 2, 0.01),
    synth.TimeScheme.exponential(12, 30, 1.25, 0, 0, 1.0),
    synth.TimeScheme.linear(400, 1.0),
    synth.TimeScheme.linear(20, 0.5),
]


@pytest.mark.parametrize("ts", SCHEMES, ids=lambda t: t.script_line())
@pytest.mark.parametrize("fullblock", [0, 1])
@pytest.mark.parametrize("limit", [0, 3])
def test_scheduler_matches_oracle(E, ts, fullblock, limit):
    s = E.make_scheme(ts, limit)
    o = orc.scheme(ts, limit)
    T, G, P = E.scheme_counts(s, fullblock)
    assert (T, G) == (orc.n_timesteps(o), orc.n_timegaps(o))
    for loop in (0, 1):
        g, a, b = E.scheme_pairs(s, fullblock, loop)
        og, oa, ob = orc.pairs(o, fullblock, loop_order=bool(loop))
        np.testing.assert_array_equal(g, og)
        np.testing.assert_array_equal(a, oa)
        np.testing.assert_array_equal(b, ob)
    tl, gt = E.scheme_times(s)
    np.testing.assert_array_equal(tl, orc.timelist(o))
    np.testing.assert_array_equal(gt, orc.displacement_times(o))
    np.testing.assert_array_equal(E.scheme_weighting(s, fullblock), orc.timegap_weighting(o, fullblock))


def test_bad_scheme_is_an_error(E):
    s = E.Scheme()
    st = E.lib().amdat_scheme_init(C.byref(s), 7, 1, 1, C.c_float(1.0), 0, 0, C.c_float(1.0))
    assert st == 1 and b"unknown" in E.lib().amdat_last_error()


def test_no_device_reports_status(E):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ctx = C.c_void_p()
    st = E.lib().amdat_create(0, C.byref(ctx))
    assert st == 4  # AMDAT_ERR_NO_DEVICE
    assert E.lib().amdat_last_error()


@pytest.mark.parametrize("frames", [1000, 1300])
def test_noalloc_rejects_too_many_time_pairs_before_any_gpu_work(E, frames):
    """Linear schemes of 1000 and 1300 frames (499,501 and 844,351 time pairs)
    pass the fixed-table size check but need more work items than the fixed
    scratch holds even at one atom chunk per pair.  The entry point must return
    AMDAT_ERR_ARGUMENT from its host-side check, not loop or divide by zero.
    The pointers are never dereferenced: the check runs before any CUDA call."""
    st = _noalloc_call(E, frames)
    assert st == 1, E.lib().amdat_last_error()
    msg = E.lib().amdat_last_error()
    assert b"time pairs" in msg and b"16 MiB" in msg


def _noalloc_call(E, frames):
    s = E.make_scheme(synth.TimeScheme.linear(frames, 1.0))
    fake = C.c_void_p(256)  # never dereferenced: rejected on the host
    return E.lib().amdat_disp_moments_noalloc(C.byref(s), 0, fake, frames, 1, None, fake, fake)
