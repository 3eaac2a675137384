"""The C host program mocatt_run (host/moc_driver.c): the reference's command line and
output lines (src/cpu/io.c:99-161, src/cpu/main.c:55-58) over moc_attenuate_fwd_host."""
import os
import re
import subprocess

import numpy as np
import pytest

import mocatt

EXE = os.path.join(mocatt.BUILD, "mocatt_run")


def run(*args, timeout=600):
    return subprocess.run([EXE, *args], capture_output=True, text=True, timeout=timeout)


def test_driver_without_a_device_exits_cleanly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    out = run("-s", "1000", "-e", "8")
    assert out.returncode == 2
    assert "no CUDA device" in out.stderr


def test_driver_rejects_bad_sizes():
    assert run("-s", "-5", "-e", "8").returncode != 0


@pytest.mark.gpu
@pytest.mark.parametrize("table", [False, True])
def test_driver_matches_the_library(handle, table):
    """mocatt_run sweeps its seeded problem 1 + n times in place (one untimed call, n
    timed) and prints the sum of psi; the same problem through the Python binding, swept
    as often, gives the same sum."""
    S, G, R, T, n = 300_000, 64, 500, 600, 2
    args = ["-s", str(S), "-e", str(G), "-r", str(R), "-k", str(T), "-n", str(n), "-t", "16"]
    if table:
        args.append("-x")
    out = run(*args)
    assert out.returncode == 0, out.stderr
    check = float(re.search(r"psi checksum:\s+(\S+)", out.stdout).group(1))
    tpi = float(re.search(r"Time per Intersection:\s+(\S+) ns", out.stdout).group(1))
    assert tpi > 0.0
    hp = mocatt.generate(mocatt.Workload("driver", 1, R, 5, G, T, S))
    opts = mocatt.default_opts(exp_mode=mocatt.MOC_EXP_TABLE if table else mocatt.MOC_EXP_FULL)
    for _ in range(1 + n):
        handle.fwd_host(hp, opts)
    ref = float(hp.psi.astype(np.float64).sum())
    assert abs(check - ref) <= 1e-6 * abs(ref), (check, ref)


@pytest.mark.gpu
def test_driver_sweeps_a_track_file(handle):
    """mocatt_run -f sweeps the golden track file's segments with seeded tables: the same
    problem through the Python binding gives the same psi sum."""
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                          "tracks_3x2.moctrk")
    G, n = 8, 1
    out = run("-f", golden, "-e", str(G), "-n", str(n))
    assert out.returncode == 0, out.stderr
    check = float(re.search(r"psi checksum:\s+(\S+)", out.stdout).group(1))
    R, I, off, reg, itv, ds = mocatt.read_trackfile(golden)
    T, S = len(off) - 1, len(reg)
    hp = mocatt.generate(mocatt.Workload("driver", 1, R, I, G, T, S))
    hp.track_offsets[:] = off
    hp.seg_region[:] = reg
    hp.seg_interval[:] = itv
    hp.seg_ds[:] = ds
    for _ in range(1 + n):
        handle.fwd_host(hp, mocatt.default_opts())
    ref = float(hp.psi.astype(np.float64).sum())
    assert abs(check - ref) <= 1e-6 * abs(ref), (check, ref)

