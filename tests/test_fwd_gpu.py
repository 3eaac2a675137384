"""Parity of the GPU forward sweep (through the C ABI) with the CPU oracle."""
import numpy as np
import pytest

import mocatt
import oracle
import parity

pytestmark = pytest.mark.gpu


def run_gpu(handle, hp, opts=None, device="cuda:0"):
    dp = mocatt.DeviceProblem(hp, device)
    handle.fwd(dp, opts)
    st = handle.synchronize()
    assert st == 0, mocatt.lib().moc_status_string(st)
    return dp.to_host("psi"), dp.to_host("fine_flux")


def small(name="sweep_1M_g64", **kw):
    base = dict(regions=120, tracks=48, segments=12_000)
    base.update(kw)
    return mocatt.generate(mocatt.WORKLOADS[name].with_(**base))


def test_plain_sweep_1M_g64_full_size(handle):
    """The reference's CPU-sized run (1,000,000 segments, G=64) at full size."""
    hp = mocatt.generate(mocatt.WORKLOADS["sweep_1M_g64"])
    psi, ff = run_gpu(handle, hp)
    ref = oracle.fwd_fp64(hp)
    res = parity.check_plain(psi, ff, ref, hp.G)
    # and against the FP32 restatement of the reference itself
    p32, f32 = oracle.fwd_fp32(hp)
    parity.check_plain(p32, f32, ref, hp.G)
    print(res, parity.rel_err(psi[:, :hp.G], p32[:, :hp.G]))


@pytest.mark.parametrize("G", [1, 3, 16, 32, 33, 64, 65, 70, 128, 129, 130, 256])
def test_plain_group_counts(handle, G):
    hp = small(groups=G)
    psi, ff = run_gpu(handle, hp)
    parity.check_plain(psi, ff, oracle.fwd_fp64(hp), G)
    # padding entries are never written
    if hp.Gs > G:
        assert np.all(ff[:, G:] == 0)


@pytest.mark.parametrize("vec", [1, 2, 4])
@pytest.mark.parametrize("wpb", [1, 4, 8])
@pytest.mark.parametrize("prefetch", [1, 8])
def test_plain_launch_shapes(handle, vec, wpb, prefetch):
    hp = small(groups=64)
    opts = mocatt.default_opts(vec=vec, warps_per_block=wpb, prefetch=prefetch)
    psi, ff = run_gpu(handle, hp, opts)
    parity.check_plain(psi, ff, oracle.fwd_fp64(hp), hp.G)


@pytest.mark.parametrize("G", [3, 70, 128])
def test_prefetch_ring_matches_registers(handle, G):
    """The shared-memory prefetch ring computes exactly what the register path computes:
    psi bit for bit, including ragged tracks and out-of-range segments (skipped)."""
    hp = small(groups=G, tracks=300, segments=9000)
    hp.seg_region[17] = hp.R + 3
    p1, f1 = run_gpu_unchecked(handle, hp, mocatt.default_opts(prefetch=1))
    p8, f8 = run_gpu_unchecked(handle, hp, mocatt.default_opts(prefetch=8))
    assert np.array_equal(p1, p8)
    tab = dict(exp_mode=mocatt.MOC_EXP_TABLE, table_points=10_000)
    p1, _ = run_gpu_unchecked(handle, hp, mocatt.default_opts(prefetch=1, **tab))
    p8, _ = run_gpu_unchecked(handle, hp, mocatt.default_opts(prefetch=8, **tab))
    assert np.array_equal(p1, p8)


def run_gpu_unchecked(handle, hp, opts):
    """Run and expect exactly the bad-index report of a planted out-of-range segment."""
    dp = mocatt.DeviceProblem(hp)
    handle.fwd(dp, opts)
    assert handle.synchronize() == mocatt.MOC_ERR_BAD_INDEX
    return dp.to_host("psi"), dp.to_host("fine_flux")


@pytest.mark.parametrize("npts,maxv", [(353, 10.0), (10_000, 10.0), (50, 3.0)])
def test_table_mode_matches_reference_table(handle, npts, maxv):
    """Table mode: e is the reference's lookup, bit for bit; the rest within tolerance."""
    hp = small(groups=64)
    opts = mocatt.default_opts(exp_mode=mocatt.MOC_EXP_TABLE, table_points=npts,
                               table_max=maxv)
    psi, ff = run_gpu(handle, hp, opts)
    ref = oracle.fwd_fp64(hp, opts)
    parity.check_plain(psi, ff, ref, hp.G)


def test_psi_deterministic_and_tally_additive(handle):
    hp = small(groups=64)
    p1, f1 = run_gpu(handle, hp)
    p2, f2 = run_gpu(handle, hp)
    assert np.array_equal(p1, p2)           # psi has no reduction: bitwise
    # tallies arrive in another order each run: both inside the FP32 tolerance
    ref = oracle.fwd_fp64(hp)
    parity.check_plain(p1, f1, ref, hp.G)
    parity.check_plain(p2, f2, ref, hp.G)
    # tallies add into what fine_flux held
    hp2 = hp.copy()
    hp2.fine_flux[:] = f1
    p3, f3 = run_gpu(handle, hp2)
    parity.check_plain(p3, f3, oracle.fwd_fp64(hp2), hp.G)


def test_empty_and_ragged_tracks(handle):
    hp = small(groups=64, tracks=300, segments=400)  # many empty / 1-segment tracks
    lens = np.diff(hp.track_offsets)
    assert (lens == 0).any() and (lens == 1).any()
    psi, ff = run_gpu(handle, hp)
    parity.check_plain(psi, ff, oracle.fwd_fp64(hp), hp.G)
    empty = lens == 0
    np.testing.assert_array_equal(psi[empty], hp.psi[empty])


def test_zero_tracks_and_zero_segments(handle):
    hp = small(groups=16, tracks=5, segments=0)
    psi, ff = run_gpu(handle, hp)
    np.testing.assert_array_equal(psi, hp.psi)
    assert not ff.any()


def test_host_entry_point_matches_device(handle):
    hp = small(groups=64)
    psi_d, ff_d = run_gpu(handle, hp)
    q = hp.copy()
    handle.fwd_host(q)
    assert np.array_equal(q.psi, psi_d)
    ref = oracle.fwd_fp64(hp)
    parity.check_plain(q.psi, q.fine_flux, ref, hp.G)
    parity.check_plain(psi_d, ff_d, ref, hp.G)


@pytest.mark.parametrize("name,kw", [
    ("sweep_50M_g128", dict(segments=18_000_000, tracks=40_000, regions=2_000, groups=64)),
    ("adjoint_2M_g64", dict(tracks=50_000)),
])
def test_pipelined_host_entry_point(handle, name, kw):
    """From 16M segments on the host-buffer entry point copies and sweeps in parts (tracks
    cut into ranges of ~8M segments, copies overlapping the sweeps): psi equals the device
    entry point bit for bit (the long-track chunk length is the whole problem's), and both
    outputs are inside the FP64 tolerance. The lognormal case cuts long tracks."""
    hp = mocatt.generate(mocatt.WORKLOADS[name].with_(**kw))
    assert hp.S >= 2 * 8 * 2**20
    psi_d, ff_d = run_gpu(handle, hp)
    q = hp.copy()
    handle.fwd_host(q)
    assert np.array_equal(q.psi, psi_d)
    ref = oracle.fwd_fp64(hp)
    parity.check_plain(q.psi, q.fine_flux, ref, hp.G)
    parity.check_plain(psi_d, ff_d, ref, hp.G)
    # a bad segment in the last part is reported
    bad = hp.copy()
    bad.seg_region[hp.S - 3] = hp.R + 1
    with pytest.raises(mocatt.MocError):
        handle.fwd_host(bad)
    assert handle.synchronize() == 0


def pinned_copy(hp):
    """hp with every array in page-locked host memory (torch's pin_memory: mapped into the
    device's address space under unified addressing)."""
    import torch

    q = hp.copy()
    keep = []
    for name in mocatt.DeviceProblem.NAMES:
        t = torch.from_numpy(np.ascontiguousarray(getattr(hp, name))).pin_memory()
        keep.append(t)
        setattr(q, name, t.numpy())
    return q, keep


@pytest.mark.parametrize("name,kw", [
    ("sweep_1M_g64", dict(regions=120, tracks=48, segments=12_000)),
    ("sweep_50M_g128", dict(segments=18_000_000, tracks=40_000, regions=2_000, groups=64)),
    ("adjoint_2M_g64", dict(tracks=50_000)),
])
def test_host_entry_point_reads_pinned_arrays_in_place(handle, name, kw):
    """Pinned host arrays are swept in place (descriptors, offsets and psi read and psi
    written over the host link, the tables copied up, the tallies reduced on the device
    and added into fine_flux in place): psi equals the device entry point's bit for bit,
    both outputs are inside the FP64 tolerance, and a bad segment is still reported. A
    pageable fine_flux beside pinned inputs is copied up and back instead."""
    hp = mocatt.generate(mocatt.WORKLOADS[name].with_(**kw))
    psi_d, ff_d = run_gpu(handle, hp)
    q, keep = pinned_copy(hp)
    handle.fwd_host(q)
    assert np.array_equal(q.psi, psi_d)
    ref = oracle.fwd_fp64(hp)
    parity.check_plain(q.psi, q.fine_flux, ref, hp.G)
    c, keep_c = pinned_copy(hp)
    c.fine_flux = np.array(hp.fine_flux, copy=True)  # pageable
    handle.fwd_host(c)
    assert np.array_equal(c.psi, psi_d)
    parity.check_plain(c.psi, c.fine_flux, ref, hp.G)
    b, keep_b = pinned_copy(hp)
    b.seg_region[hp.S - 3] = hp.R + 1
    with pytest.raises(mocatt.MocError):
        handle.fwd_host(b)
    assert handle.synchronize() == 0


def test_bad_index_is_skipped_and_reported(handle):
    """A segment with an out-of-range region is skipped by the kernel's own bounds check
    and reported; checked mode rejects the problem before touching anything."""
    hp = small(groups=16)
    hp.seg_region[5] = hp.R + 7
    dp = mocatt.DeviceProblem(hp)
    opts = mocatt.default_opts(checked=1)
    st = mocatt.lib().moc_attenuate_fwd(handle.ptr, mocatt.C.byref(dp.c_struct()),
                                        mocatt.C.byref(opts), None)
    assert st == mocatt.MOC_ERR_BAD_INDEX
    np.testing.assert_array_equal(dp.to_host("psi"), hp.psi)
    assert not dp.to_host("fine_flux").any()
    assert handle.synchronize() == 0  # the refusal was the report
    handle.fwd(dp)
    assert handle.synchronize() == mocatt.MOC_ERR_BAD_INDEX
    assert handle.synchronize() == 0  # cleared


def test_invalid_arguments_return_status(handle):
    hp = small(groups=16)
    dp = mocatt.DeviceProblem(hp)
    L = mocatt.lib()
    o = mocatt.default_opts()

    def call(prob, opts=o):
        return L.moc_attenuate_fwd(handle.ptr, mocatt.C.byref(prob), mocatt.C.byref(opts), None)

    p = dp.c_struct(); p.group_stride = 18
    assert call(p) == mocatt.MOC_ERR_UNSUPPORTED
    p = dp.c_struct(); p.n_intervals = 1
    assert call(p) == mocatt.MOC_ERR_INVALID_ARG
    p = dp.c_struct(); p.sigT = dp.sigT.data_ptr() + 4
    assert call(p) == mocatt.MOC_ERR_MISALIGNED
    p = dp.c_struct(); p.psi = None
    assert call(p) == mocatt.MOC_ERR_INVALID_ARG
    p = dp.c_struct(); p.sigT = hp.sigT.ctypes.data   # host pointer to the device entry
    assert call(p) == mocatt.MOC_ERR_INVALID_ARG
    bad = mocatt.default_opts(exp_mode=7)
    assert call(dp.c_struct(), bad) == mocatt.MOC_ERR_INVALID_ARG
    assert L.moc_attenuate_fwd(None, mocatt.C.byref(dp.c_struct()), mocatt.C.byref(o),
                               None) == mocatt.MOC_ERR_INVALID_ARG


@pytest.mark.parametrize("exp_mode", ["full", "table10k"])
def test_sweep_50M_g128_full_size(handle, exp_mode):
    """The 50M segments x 128 groups workload at full size, every psi and fine_flux
    entry against the FP64 oracle (all host threads); a sample of tracks run alone
    reproduces the full run's psi bit for bit (psi depends only on its own track)."""
    import torch

    hp = mocatt.generate(mocatt.WORKLOADS["sweep_50M_g128"])
    opts = mocatt.default_opts()
    if exp_mode == "table10k":
        opts = mocatt.default_opts(exp_mode=mocatt.MOC_EXP_TABLE, table_points=10_000,
                                   table_max=10.0)
    dp = mocatt.DeviceProblem(hp)
    handle.fwd(dp, opts)
    assert handle.synchronize() == 0
    psi = dp.to_host("psi")
    ff = dp.to_host("fine_flux")
    del dp
    torch.cuda.empty_cache()
    ref = oracle.fwd_fp64(hp, opts)
    res = parity.check_plain(psi, ff, ref, hp.G)
    print(exp_mode, res, parity.rel_err(psi[:, :hp.G], ref["psi"][:, :hp.G]),
          parity.rel_err(ff[:, :hp.G], ref["ff"][:, :hp.G]))
    del ref
    sample = np.sort(np.random.default_rng(7).choice(hp.T, 64, replace=False))
    sub = hp.subset_tracks(sample)
    # the automatic chunk length of the full problem (S x 2 group chunks = 1e8 warp steps:
    # C = 2048) cuts none of its tracks; the small subset would get a short C, so it runs
    # uncut explicitly
    assert np.diff(hp.track_offsets).max() <= 4 * 2048
    sub_opts = mocatt.MocFwdOpts.from_buffer_copy(opts)
    sub_opts.track_chunk = -1
    p_sub, _ = run_gpu(handle, sub, sub_opts)
    assert np.array_equal(p_sub, psi[sample])


def test_arrays_of_another_device_are_refused():
    """A sweep on one device refuses arrays that live on another (it may have no peer
    access to them): MOC_ERR_INVALID_ARG from the handle and the no-allocation entry
    points. Needs two GPUs."""
    import ctypes as C

    import torch

    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    hp = small(regions=20, tracks=4, segments=100)
    dp1 = mocatt.DeviceProblem(hp, "cuda:1")
    h0 = mocatt.Handle(0)
    o = mocatt.default_opts()
    st = mocatt.lib().moc_attenuate_fwd(h0.ptr, C.byref(dp1.c_struct()), C.byref(o), None)
    assert st == mocatt.MOC_ERR_INVALID_ARG
    h0.close()
    torch.cuda.set_device(0)
    st = mocatt.lib().moc_attenuate_fwd_noalloc(C.byref(dp1.c_struct()), C.byref(o), None)
    assert st == mocatt.MOC_ERR_INVALID_ARG
