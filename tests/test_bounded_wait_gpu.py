"""The bounded wait of the sweep's bulk-copy ring (mbar_wait_bounded in
simplemoc-kernel_gb300/csrc/moc_device.cuh): a wait on a barrier that nothing completes
gives up after its clock limit and reports it, and the context stays usable; a completed
barrier is seen at once. The probe is a test-only kernel compiled here from
tests/native/bounded_wait_probe.cu; it faults nothing and every wait has a limit."""
import ctypes as C
import os
import subprocess

import pytest

import mocatt
import mocatt_build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def probe():
    src = os.path.join(HERE, "native", "bounded_wait_probe.cu")
    out_dir = os.path.join(mocatt.BUILD, "tests")
    os.makedirs(out_dir, exist_ok=True)
    so = os.path.join(out_dir, "libboundedwait.so")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run([mocatt_build.nvcc()] + mocatt_build.NVCC_FLAGS +
                       ["-shared", "-cudart", "static", src, "-o", so], check=True)
    lib = C.CDLL(so)
    lib.bounded_wait_probe.restype = C.c_int
    lib.bounded_wait_probe.argtypes = [C.c_int, C.c_longlong, C.POINTER(C.c_int)]
    return lib


def test_wait_gives_up_and_context_stays_usable(cuda, probe):
    import torch

    out = (C.c_int * 2)()
    limit = 20_000_000  # ~10 ms of SM clocks
    assert probe.bounded_wait_probe(0, limit, out) == 0
    assert out[0] == 0, "a wait on a barrier nothing completes must give up"
    assert out[1] * 1024 >= limit
    # the context still works: a completed barrier is seen, and torch runs a kernel
    assert probe.bounded_wait_probe(1, limit, out) == 0
    assert out[0] == 1 and out[1] * 1024 < limit
    x = torch.ones(1024, device=cuda)
    assert float(x.sum()) == 1024.0
