"""Long tracks cut into chunks (moc_fwd_opts_t.track_chunk): parity with the FP64 oracle,
and what must stay bit for bit.

A track of more than 4 * C segments sweeps as chunks of C segments joined through the
affine form of the psi recursion (psi_out = a psi_in + b per chunk). Its psi is rounded
differently from a one-pass sweep, so it is checked against the FP64 oracle with the
plain FP32 tolerance; tracks of at most 4 * C segments run exactly the one-pass
arithmetic, so their psi must equal the unsplit run bit for bit."""
import numpy as np
import pytest

import mocatt
import oracle
import parity

pytestmark = pytest.mark.gpu

NO_SPLIT = -1


def run(handle, hp, opts):
    dp = mocatt.DeviceProblem(hp)
    handle.fwd(dp, opts)
    st = handle.synchronize()
    assert st == 0, mocatt.lib().moc_status_string(st)
    return dp.to_host("psi"), dp.to_host("fine_flux")


def lognormal(**kw):
    """Lognormal track lengths (median 267, sigma 0.9005, 1..5000), G = 64 by default."""
    base = dict(tracks=1500)
    base.update(kw)
    return mocatt.generate(mocatt.WORKLOADS["adjoint_2M_g64"].with_(**base))


@pytest.fixture(scope="module")
def long_tracks():
    hp = lognormal()
    lens = np.diff(hp.track_offsets)
    assert lens.max() > 4 * 256  # C = 256 cuts some tracks
    return hp, oracle.fwd_fp64(hp)


@pytest.mark.parametrize("chunk", [0, 32, 100, 1000])
def test_split_matches_fp64(handle, long_tracks, chunk):
    hp, ref = long_tracks
    psi, ff = run(handle, hp, mocatt.default_opts(track_chunk=chunk))
    print(chunk, parity.check_plain(psi, ff, ref, hp.G))


def test_short_tracks_bitwise_equal_to_unsplit(handle, long_tracks):
    hp, ref = long_tracks
    p_split, f_split = run(handle, hp, mocatt.default_opts(track_chunk=256))
    p_one, f_one = run(handle, hp, mocatt.default_opts(track_chunk=NO_SPLIT))
    parity.check_plain(p_one, f_one, ref, hp.G)
    lens = np.diff(hp.track_offsets)
    whole = lens <= 4 * 256
    assert whole.any() and (~whole).any()
    assert np.array_equal(p_split[whole], p_one[whole])
    # cut tracks: the two roundings agree to the FP32 tolerance of the formula
    print("cut-track psi rel err", parity.rel_err(p_split[~whole, :hp.G],
                                                  p_one[~whole, :hp.G]))


def test_split_psi_depends_only_on_the_track(handle, long_tracks):
    """With a given chunk length, where a track is cut depends on its length alone: a
    sample of tracks run as their own problem reproduces the full run's psi bit for bit."""
    hp, _ = long_tracks
    opts = mocatt.default_opts(track_chunk=256)
    psi, _ = run(handle, hp, opts)
    lens = np.diff(hp.track_offsets)
    order = np.argsort(-lens)
    sample = np.sort(np.concatenate([order[:12], order[-12:],
                                     np.random.default_rng(3).choice(hp.T, 24, replace=False)]))
    sample = np.unique(sample)
    p_sub, _ = run(handle, hp.subset_tracks(sample), opts)
    assert np.array_equal(p_sub, psi[sample])


def test_auto_chunk_cuts_long_tracks_of_small_problems(handle, long_tracks):
    """The automatic chunk length follows the problem's size: about 600,000 segments x one
    group chunk gives C = 32 (tracks of more than 128 segments are cut) - the same psi as
    an explicit C = 32, bit for bit."""
    hp, ref = long_tracks
    p_auto, f_auto = run(handle, hp, mocatt.default_opts())
    p_32, _ = run(handle, hp, mocatt.default_opts(track_chunk=32))
    assert np.array_equal(p_auto, p_32)
    parity.check_plain(p_auto, f_auto, ref, hp.G)


def test_auto_chunk_floor_at_a_sixteenth_of_the_mean_track(handle):
    """1,000 equal tracks of 1,000 segments (1M x 64): the problem's size alone would give
    C = 32, but the chunk length is at least a sixteenth of the mean track length (rounded
    up to a power of two), 64 here - the same psi as an explicit C = 64, bit for bit."""
    hp = mocatt.generate(mocatt.WORKLOADS["sweep_1M_g64"])
    p_auto, _ = run(handle, hp, mocatt.default_opts())
    p_64, _ = run(handle, hp, mocatt.default_opts(track_chunk=64))
    assert np.array_equal(p_auto, p_64)


def test_split_deterministic(handle, long_tracks):
    hp, _ = long_tracks
    p1, _ = run(handle, hp, mocatt.default_opts(track_chunk=64))
    p2, _ = run(handle, hp, mocatt.default_opts(track_chunk=64))
    assert np.array_equal(p1, p2)


@pytest.mark.parametrize("G", [3, 70, 130])
def test_split_chunk_boundaries(handle, G):
    """Track lengths around the cut rule with C = 32: at most 128 segments stay whole,
    129 and more are cut into 32-segment chunks (the last one shorter)."""
    lens = [0, 1, 31, 32, 33, 127, 128, 129, 130, 159, 160, 161, 192, 193, 1000, 4097, 0, 5]
    hp = lognormal(groups=G, tracks=600).with_lengths(lens)
    opts = mocatt.default_opts(track_chunk=32)
    psi, ff = run(handle, hp, opts)
    ref = oracle.fwd_fp64(hp)
    parity.check_plain(psi, ff, ref, G)
    p_one, _ = run(handle, hp, mocatt.default_opts(track_chunk=NO_SPLIT))
    whole = np.asarray(lens) <= 128
    assert np.array_equal(psi[whole], p_one[whole])
    empty = np.asarray(lens) == 0
    np.testing.assert_array_equal(psi[empty], hp.psi[empty])


def test_split_one_long_track(handle):
    """All segments on one track: the extreme case of a lone long track."""
    hp = lognormal(tracks=600)
    one = hp.with_lengths([min(hp.S, 60_000)])
    psi, ff = run(handle, one, mocatt.default_opts())
    parity.check_plain(psi, ff, oracle.fwd_fp64(one), one.G)


def test_split_table_mode(handle, long_tracks):
    hp, _ = long_tracks
    opts = mocatt.default_opts(exp_mode=mocatt.MOC_EXP_TABLE, table_points=10_000,
                               table_max=10.0, track_chunk=64)
    psi, ff = run(handle, hp, opts)
    parity.check_plain(psi, ff, oracle.fwd_fp64(hp, opts), hp.G)


@pytest.mark.parametrize("prec", [mocatt.MOC_PREC_FP32_STABLE, mocatt.MOC_PREC_BF16])
def test_split_precision_forms(handle, long_tracks, prec):
    hp, _ = long_tracks
    opts = mocatt.default_opts(precision=prec, tally=mocatt.MOC_TALLY_COMPENSATED,
                               track_chunk=64)
    psi, ff = run(handle, hp, opts)
    qp, coef = oracle.quantized_inputs(hp, prec)
    parity.check_plain(psi, ff, oracle.fwd_fp64_coef(qp, coef), hp.G)


@pytest.mark.parametrize("vec", [1, 2, 4])
def test_split_ring_prefetch_and_vec(handle, long_tracks, vec):
    """The shared-memory prefetch ring computes the register path's psi bit for bit on
    cut tracks too."""
    hp, ref = long_tracks
    p1, f1 = run(handle, hp, mocatt.default_opts(vec=vec, prefetch=1))
    p8, f8 = run(handle, hp, mocatt.default_opts(vec=vec, prefetch=8))
    assert np.array_equal(p1, p8)
    parity.check_plain(p1, f1, ref, hp.G)
    parity.check_plain(p8, f8, ref, hp.G)


def test_split_host_entry_point(handle, long_tracks):
    hp, ref = long_tracks
    p_dev, _ = run(handle, hp, mocatt.default_opts())
    q = hp.copy()
    handle.fwd_host(q)
    assert np.array_equal(q.psi, p_dev)
    parity.check_plain(q.psi, q.fine_flux, ref, hp.G)


def test_split_bad_segment_reported(handle):
    hp = lognormal(tracks=600).with_lengths([3000, 20, 900])
    hp.seg_region[1500] = hp.R + 1  # inside a cut chunk of the first track
    dp = mocatt.DeviceProblem(hp)
    handle.fwd(dp, mocatt.default_opts(track_chunk=64))
    assert handle.synchronize() == mocatt.MOC_ERR_BAD_INDEX
    assert handle.synchronize() == 0


def test_track_chunk_rejected_values(handle):
    hp = lognormal(tracks=600).with_lengths([50, 60])
    dp = mocatt.DeviceProblem(hp)
    L = mocatt.lib()
    for bad in (-2, 1, 31, (1 << 24) + 1):
        o = mocatt.default_opts(track_chunk=bad)
        assert L.moc_attenuate_fwd(handle.ptr, mocatt.C.byref(dp.c_struct()), mocatt.C.byref(o),
                                   None) == mocatt.MOC_ERR_INVALID_ARG


def test_split_timings_report_the_passes(handle, long_tracks):
    hp, _ = long_tracks
    dp = mocatt.DeviceProblem(hp)
    handle.fwd(dp, mocatt.default_opts(profile=1))
    t = handle.timings()
    assert handle.synchronize() == 0
    assert t.launches == 2 + 5 and t.split_ms > 0 and t.sweep_ms > 0
    handle.fwd(dp, mocatt.default_opts(profile=1, track_chunk=NO_SPLIT))
    t = handle.timings()
    assert t.launches == 2 and t.split_ms == 0
