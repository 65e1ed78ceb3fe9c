"""amdat_disp_moments_noalloc: the displacement-moment entry point for callers
that cannot allocate device memory (the caller owns the input and output
buffers; the temporaries live in the library's fixed __device__ scratch).
Its sums must match amdat_disp_run's (list of all atoms) to 1e-6 relative,
call after call.  This file is collected last so a failure here does not stop
the other GPU tests."""
import ctypes as C
import warnings

import numpy as np
import pytest

from amdat_gb300 import synth

pytestmark = pytest.mark.gpu


def test_noalloc_matches_disp_run(engine_mod):
    import torch
    E = engine_mod
    scheme = synth.TimeScheme.exponential(6, 10, 1.3, 0, 0, 0.01)
    traj = synth.random_walk(3000, 14.0, scheme, 0.4, seed=12)
    eng = E.Engine(0)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(scheme)
    ref = eng.disp(0)
    eng.close()
    torch.cuda.set_device(0)
    x = torch.from_numpy(np.ascontiguousarray(traj.unwrapped)).cuda()  # caller-owned input
    G = len(ref["sum_d2"])
    s = E.make_scheme(scheme)
    for call in range(2):
        d2 = torch.full((G,), -1.0, dtype=torch.float64, device="cuda")  # caller-owned outputs
        d4 = torch.full((G,), -1.0, dtype=torch.float64, device="cuda")
        st = E.lib().amdat_disp_moments_noalloc(C.byref(s), 0, C.c_void_p(x.data_ptr()),
                                                traj.n_frames, traj.n_atoms, None,
                                                C.c_void_p(d2.data_ptr()), C.c_void_p(d4.data_ptr()))
        torch.cuda.synchronize()
        assert st == 0, E.lib().amdat_last_error()
        np.testing.assert_allclose(d2.cpu().numpy(), ref["sum_d2"], rtol=1e-6, atol=1e-12)
        np.testing.assert_allclose(d4.cpu().numpy(), ref["sum_d4"], rtol=1e-6, atol=1e-14)


def test_noalloc_rejects_oversized_work(engine_mod):
    import torch
    E = engine_mod
    s = E.make_scheme(synth.TimeScheme.linear(5000, 1.0))   # ~12.5M time pairs
    # buffers of the sizes the call declares, so nothing reads past them even if
    # the host-side check were to let the call through
    x = torch.zeros((5000, 1, 3), dtype=torch.float32, device="cuda")
    out = torch.zeros(5000, dtype=torch.float64, device="cuda")
    st = E.lib().amdat_disp_moments_noalloc(C.byref(s), 0, C.c_void_p(x.data_ptr()), 5000, 1,
                                            None, C.c_void_p(out.data_ptr()),
                                            C.c_void_p(out.data_ptr()))
    assert st == 1 and b"16 MiB" in E.lib().amdat_last_error()


def test_noalloc_rejects_pairs_beyond_items(engine_mod):
    """1000 linear frames give 499,501 time pairs: the pair tables fit the
    scratch but one work item per pair does not, so the call is refused."""
    import torch
    E = engine_mod
    s = E.make_scheme(synth.TimeScheme.linear(1000, 1.0))
    x = torch.zeros((1000, 2, 3), dtype=torch.float32, device="cuda")
    out = torch.zeros(1000, dtype=torch.float64, device="cuda")
    st = E.lib().amdat_disp_moments_noalloc(C.byref(s), 0, C.c_void_p(x.data_ptr()), 1000, 2,
                                            None, C.c_void_p(out.data_ptr()),
                                            C.c_void_p(out.data_ptr()))
    torch.cuda.synchronize()
    assert st == 1 and b"time pairs" in E.lib().amdat_last_error()


def test_noalloc_many_pairs_one_chunk(engine_mod):
    """900 linear frames (404,551 time pairs) of 5 atoms: one atom chunk per pair
    fills most of the scratch; sums must still match amdat_disp_run."""
    import torch
    E = engine_mod
    scheme = synth.TimeScheme.linear(900, 1.0)
    traj = synth.random_walk(5, 6.0, scheme, 0.2, seed=5)
    eng = E.Engine(0)
    eng.upload(traj.unwrapped, traj.box)
    eng.set_scheme(scheme)
    ref = eng.disp(0)
    eng.close()
    x = torch.from_numpy(np.ascontiguousarray(traj.unwrapped)).cuda()
    G = len(ref["sum_d2"])
    d2 = torch.full((G,), -1.0, dtype=torch.float64, device="cuda")
    d4 = torch.full((G,), -1.0, dtype=torch.float64, device="cuda")
    s = E.make_scheme(scheme)
    st = E.lib().amdat_disp_moments_noalloc(C.byref(s), 0, C.c_void_p(x.data_ptr()),
                                            traj.n_frames, traj.n_atoms, None,
                                            C.c_void_p(d2.data_ptr()), C.c_void_p(d4.data_ptr()))
    torch.cuda.synchronize()
    assert st == 0, E.lib().amdat_last_error()
    np.testing.assert_allclose(d2.cpu().numpy(), ref["sum_d2"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(d4.cpu().numpy(), ref["sum_d4"], rtol=1e-6, atol=1e-14)


def test_noalloc_refuses_stream_capture(engine_mod):
    """A call on a stream under capture is refused before any GPU work (its
    table copies read host memory freed on return); the same call made after
    the capture runs normally."""
    import torch
    E = engine_mod
    scheme = synth.TimeScheme.exponential(3, 5, 1.3, 0, 0, 0.01)
    traj = synth.random_walk(64, 6.0, scheme, 0.2, seed=7)
    x = torch.from_numpy(np.ascontiguousarray(traj.unwrapped)).cuda()
    s = E.make_scheme(scheme)
    G = E.scheme_counts(s)[1]
    d2 = torch.zeros(G, dtype=torch.float64, device="cuda")
    d4 = torch.zeros_like(d2)
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()

    def call(strm):
        return E.lib().amdat_disp_moments_noalloc(C.byref(s), 0, C.c_void_p(x.data_ptr()),
                                                  traj.n_frames, traj.n_atoms,
                                                  C.c_void_p(strm.cuda_stream),
                                                  C.c_void_p(d2.data_ptr()), C.c_void_p(d4.data_ptr()))
    torch.cuda.synchronize()
    with warnings.catch_warnings():  # the captured graph is empty
        warnings.simplefilter("ignore")
        with torch.cuda.graph(graph, stream=stream):
            st = call(stream)
    assert st == 2 and b"capture" in E.lib().amdat_last_error()
    st = call(stream)
    stream.synchronize()
    assert st == 0, E.lib().amdat_last_error()
    assert float(d2.sum().item()) > 0.0
