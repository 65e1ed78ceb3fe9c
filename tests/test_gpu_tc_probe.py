"""Probe of the tcgen05 operand layout used by the tensor-core rho_k kernel:
one 128x64x64 fp16 MMA tile against a CPU product.  The engine's descriptor
convention (leading offset 128 B along K, stride offset K/8 * 128 B between
8-row groups) must reproduce A @ B^T."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    out = tmp_path_factory.mktemp("probe") / "tc_probe.so"
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                    "-shared", "-Xcompiler", "-fPIC", os.path.join(HERE, "tc_probe.cu"), "-o",
                    str(out)], check=True)
    return C.CDLL(str(out))


def test_umma_layout(probe):
    import torch
    g = torch.Generator().manual_seed(0)
    A = (torch.rand(128, 64, generator=g) * 2 - 1).half().cuda()
    B = (torch.rand(64, 64, generator=g) * 2 - 1).half().cuda()
    ref = (A.double().cpu() @ B.double().cpu().T).numpy()
    D = torch.zeros(128, 64, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = probe.tc_probe_run(C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()),
                            C.c_void_p(D.data_ptr()), 128, 8 * 128, C.c_void_p(err.data_ptr()))
    assert st == 0 and int(err.item()) == 0
    got = D.cpu().numpy()
    assert np.abs(got - ref).max() < 1e-4 * max(1.0, np.abs(ref).max()), np.abs(got - ref).max()


def test_umma_a_from_tensor_memory(probe):
    """The A operand read from tensor memory (the layout the lattice kernel's
    builders write): D = A @ B^T for a 128x32 A and a 32x32 B."""
    import torch
    g = torch.Generator().manual_seed(1)
    A = (torch.rand(128, 32, generator=g) * 2 - 1).half().cuda()
    B = (torch.rand(32, 32, generator=g) * 2 - 1).half().cuda()
    ref = (A.double().cpu() @ B.double().cpu().T).numpy()
    D = torch.zeros(128, 32, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = probe.tc_probe_tmem_a_run(C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()),
                                   C.c_void_p(D.data_ptr()), C.c_void_p(err.data_ptr()))
    assert st == 0 and int(err.item()) == 0
    got = D.cpu().numpy()
    assert np.abs(got - ref).max() < 1e-4 * max(1.0, np.abs(ref).max()), np.abs(got - ref).max()


def test_bounded_wait_times_out_and_context_stays_usable(probe):
    """A wait on an mbarrier that nothing completes gives up after its bounded
    number of polls and reports it; the context then still runs kernels."""
    import torch
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    rc = probe.wait_timeout_run(C.c_void_p(status.data_ptr()), C.c_uint(1000))
    assert rc == 0
    assert int(status.item()) == 1
    # the context is intact: the layout probe still runs and is correct
    test_umma_layout(probe)
