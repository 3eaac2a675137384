"""The on-disk track format (include/moc_trackfile.h): the library's reader and writer
against the golden file written by the oracle's own writer (tests/golden/make_trackfile.py),
round trips, corrupt and inconsistent files, and both harnesses reading the same file
(oracle/cpu_bench --track-file here; mocatt_run -f in test_driver.py)."""
import json
import os
import platform
import subprocess

import numpy as np
import pytest

import mocatt
import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "tracks_3x2.moctrk")


def golden_arrays():
    return oracle.trackfile_parse(open(GOLDEN, "rb").read())


def test_library_reads_the_golden_file():
    R, I, off, reg, itv, ds = mocatt.read_trackfile(GOLDEN)
    oR, oI, ooff, oreg, oitv, ods = golden_arrays()
    assert (R, I) == (oR, oI) == (48, 5)
    np.testing.assert_array_equal(off, ooff)
    np.testing.assert_array_equal(reg, oreg)
    np.testing.assert_array_equal(itv, oitv)
    assert ds.tobytes() == ods.tobytes()


def test_library_writes_the_golden_bytes(tmp_path):
    R, I, off, reg, itv, ds = golden_arrays()
    p = str(tmp_path / "w.moctrk")
    mocatt.write_trackfile(p, R, I, off, reg, itv, ds)
    assert open(p, "rb").read() == open(GOLDEN, "rb").read()


def test_golden_file_matches_a_fresh_trace():
    import sys

    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_trackfile as mk

    if platform.machine() != "x86_64":
        pytest.skip("the fixture's plan was made with an x86_64 libm's cos/sin")
    g, q = mocatt.geometry(**mk.GEOMETRY), mocatt.quadrature(**mk.QUADRATURE)
    off, reg, itv, ds = oracle.trace(g, mocatt.tracks_plan(g, q))
    R, I, foff, freg, fitv, fds = golden_arrays()
    np.testing.assert_array_equal(foff, off)
    np.testing.assert_array_equal(freg, reg)
    assert fds.tobytes() == ds.tobytes()


@pytest.mark.parametrize("case", ["random", "empty_tracks", "no_segments", "odd_payload"])
def test_round_trip(tmp_path, case):
    rng = np.random.default_rng(4)
    R, I = 37, 7
    if case == "no_segments":
        lens = np.zeros(3, np.int64)
    elif case == "empty_tracks":
        lens = rng.integers(0, 3, 50)
    elif case == "odd_payload":
        lens = np.array([3])          # 8*2 + 8*3 bytes: not a whole number of words
    else:
        lens = rng.integers(1, 40, 200)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    S = int(off[-1])
    reg = rng.integers(0, R, S).astype(np.int32)
    itv = rng.integers(0, I, S).astype(np.uint8)
    ds = rng.random(S).astype(np.float32)
    p = str(tmp_path / "t.moctrk")
    mocatt.write_trackfile(p, R, I, off, reg, itv, ds)
    assert os.path.getsize(p) == 48 + 8 * len(off) + 8 * S
    got = mocatt.read_trackfile(p)
    assert got[:2] == (R, I)
    for a, b in zip(got[2:], (off, reg, itv, ds)):
        np.testing.assert_array_equal(a, b)
    assert oracle.trackfile_parse(open(p, "rb").read())[0] == R


def test_corrupt_and_inconsistent_files(tmp_path):
    good = open(GOLDEN, "rb").read()
    cases = {
        "flipped payload byte": good[:2000] + bytes([good[2000] ^ 1]) + good[2001:],
        "truncated": good[:-5],
        "trailing bytes": good + b"x",
        "bad magic": b"MOCTRK02" + good[8:],
        "bad version": good[:8] + (3).to_bytes(4, "little") + good[12:],
        "version 2 header on a version 1 payload": good[:8] + (2).to_bytes(4, "little") + good[12:],
        "header only": good[:48],
    }
    R, I, off, reg, itv, ds = golden_arrays()
    bad_cells = (reg.astype(np.uint64) * I + itv).copy()
    bad_cells[17] = R * I                             # out of range, checksum valid
    cases["cell out of range"] = oracle.trackfile_bytes(R, I, off, reg, itv, ds, bad_cells)
    bad_off = off.copy()
    bad_off[5], bad_off[6] = bad_off[6], bad_off[5]   # not monotone, checksum valid
    cases["offsets out of order"] = oracle.trackfile_bytes(R, I, bad_off, reg, itv, ds)
    for name, data in cases.items():
        p = str(tmp_path / "bad.moctrk")
        open(p, "wb").write(data)
        with pytest.raises(mocatt.MocError) as e:
            mocatt.read_trackfile(p)
        assert e.value.status == mocatt.MOC_ERR_IO, name
    with pytest.raises(mocatt.MocError) as e:
        mocatt.read_trackfile(str(tmp_path / "missing.moctrk"))
    assert e.value.status == mocatt.MOC_ERR_IO


def test_write_rejects_bad_arrays(tmp_path):
    R, I, off, reg, itv, ds = golden_arrays()
    p = str(tmp_path / "x.moctrk")
    for bad in ({"reg": np.where(np.arange(len(reg)) == 3, R, reg).astype(np.int32)},
                {"itv": np.where(np.arange(len(itv)) == 3, I, itv).astype(np.uint8)},
                {"off": np.concatenate([[1], off[1:]])}):
        args = dict(off=off, reg=reg, itv=itv, ds=ds)
        args.update(bad)
        with pytest.raises(mocatt.MocError) as e:
            mocatt.write_trackfile(p, R, I, args["off"], args["reg"], args["itv"], args["ds"])
        assert e.value.status == mocatt.MOC_ERR_INVALID_ARG
    with pytest.raises(mocatt.MocError) as e:
        mocatt.write_trackfile(str(tmp_path / "no" / "dir.moctrk"), R, I, off, reg, itv, ds)
    assert e.value.status == mocatt.MOC_ERR_IO


def test_cpu_harness_reads_the_file(tmp_path):
    exe = os.path.join(oracle.HERE, "_build", "cpu_bench")
    out = subprocess.run([exe, "--groups", "8", "--track-file", GOLDEN, "--steps", "1",
                          "--warmup", "0", "--threads", "2"], capture_output=True, text=True,
                         timeout=120)
    assert out.returncode == 0, out.stderr
    r = json.loads(out.stdout.strip().splitlines()[-1])
    assert r["sample_segments"] == 4063 and r["sample_tracks"] == 368
    bad = str(tmp_path / "bad.moctrk")
    open(bad, "wb").write(open(GOLDEN, "rb").read()[:-1])
    out = subprocess.run([exe, "--track-file", bad], capture_output=True, text=True,
                         timeout=60)
    assert out.returncode == 2


def test_gpu_program_writes_without_a_device(tmp_path):
    """mocatt_run -w writes the generated segments before it needs the GPU."""
    exe = os.path.join(mocatt.BUILD, "mocatt_run")
    p = str(tmp_path / "gen.moctrk")
    subprocess.run([exe, "-s", "3000", "-e", "8", "-r", "40", "-k", "7", "-w", p],
                   capture_output=True, text=True, timeout=120)
    R, I, off, reg, itv, ds = mocatt.read_trackfile(p)
    assert (R, I, len(off) - 1, len(reg)) == (40, 5, 7, 3000)
    # the same seeded problem from the generator
    hp = mocatt.generate(mocatt.Workload("driver", 1, 40, 5, 8, 7, 3000))
    np.testing.assert_array_equal(off, hp.track_offsets)
    np.testing.assert_array_equal(reg, hp.seg_region)
    assert ds.tobytes() == hp.seg_ds.tobytes()


def test_compact_version_matches_the_oracle_and_rounds_lengths_to_half(tmp_path):
    """Version 2 (6 bytes per segment): the library's bytes equal the oracle's own writer
    (numpy's float16 rounding), and reading widens the half lengths exactly."""
    R, I, off, reg, itv, ds = golden_arrays()
    p = str(tmp_path / "c.moctrk")
    mocatt.write_trackfile(p, R, I, off, reg, itv, ds, compact=True)
    data = open(p, "rb").read()
    assert data == oracle.trackfile_bytes(R, I, off, reg, itv, ds, compact=True)
    S = len(ds)
    assert len(data) == 48 + 8 * len(off) + 6 * S
    gR, gI, goff, greg, gitv, gds = mocatt.read_trackfile(p)
    assert (gR, gI) == (R, I)
    np.testing.assert_array_equal(goff, off)
    np.testing.assert_array_equal(greg, reg)
    np.testing.assert_array_equal(gitv, itv)
    half = ds.astype(np.float16).astype(np.float32)
    assert gds.tobytes() == half.tobytes()
    assert np.all(np.abs(gds - ds) <= 2.0 ** -11 * np.abs(ds) + 2.0 ** -25)
    info = mocatt.MocTrackfileInfo()
    assert mocatt.lib().moc_trackfile_info(os.fsencode(p), mocatt.C.byref(info)) == 0
    assert (info.version, info.bytes_per_segment) == (2, 6)
    # the oracle's parser and the CPU harness read it too
    assert oracle.trackfile_parse(data)[5].tobytes() == half.tobytes()
    exe = os.path.join(oracle.HERE, "_build", "cpu_bench")
    out = subprocess.run([exe, "--groups", "8", "--track-file", p, "--steps", "1",
                          "--warmup", "0", "--threads", "2"], capture_output=True, text=True,
                         timeout=120)
    assert out.returncode == 0, out.stderr
    assert json.loads(out.stdout.strip().splitlines()[-1])["sample_segments"] == S


def test_half_rounding_edge_cases(tmp_path):
    """Ties to even, subnormal halves, the largest finite half; lengths that would not be
    finite halves (or are negative or NaN) are refused."""
    vals = np.array([0.0, 1.0, 1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11, 2.0 ** -24, 2.0 ** -25,
                     3 * 2.0 ** -26, 6.0e-5, 1e-7, 65504.0, 65519.0, 0.7, 1.0 / 3.0],
                    np.float32)
    S = len(vals)
    off = np.array([0, S], np.int64)
    reg = np.zeros(S, np.int32)
    itv = np.zeros(S, np.uint8)
    p = str(tmp_path / "e.moctrk")
    mocatt.write_trackfile(p, 1, 2, off, reg, itv, vals, compact=True)
    assert open(p, "rb").read() == oracle.trackfile_bytes(1, 2, off, reg, itv, vals, compact=True)
    got = mocatt.read_trackfile(p)[5]
    assert got.tobytes() == vals.astype(np.float16).astype(np.float32).tobytes()
    for bad in (65520.0, -1.0, np.nan, np.inf):
        with pytest.raises(mocatt.MocError) as e:
            mocatt.write_trackfile(p, 1, 2, np.array([0, 1], np.int64), reg[:1], itv[:1],
                                   np.array([bad], np.float32), compact=True)
        assert e.value.status == mocatt.MOC_ERR_INVALID_ARG


def test_gpu_program_writes_compact_files_without_a_device(tmp_path):
    exe = os.path.join(mocatt.BUILD, "mocatt_run")
    p = str(tmp_path / "gen.moctrk")
    subprocess.run([exe, "-s", "3000", "-e", "8", "-r", "40", "-k", "7", "-W", p],
                   capture_output=True, text=True, timeout=120)
    R, I, off, reg, itv, ds = mocatt.read_trackfile(p)
    hp = mocatt.generate(mocatt.Workload("driver", 1, 40, 5, 8, 7, 3000))
    np.testing.assert_array_equal(reg, hp.seg_region)
    assert ds.tobytes() == hp.seg_ds.astype(np.float16).astype(np.float32).tobytes()
    assert os.path.getsize(p) == 48 + 8 * 8 + 6 * 3000
