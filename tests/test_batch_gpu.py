"""The batching form: three problems with G = 16, 70 and 128 and lognormal track lengths
(median 200, clipped to 1..5,000, seed 3) swept by one persistent, graph-captured launch
(moc_attenuate_fwd_batch), and its autotuner (moc_autotune_batch)."""
import ctypes as C

import numpy as np
import pytest

import mocatt
import oracle
import parity

pytestmark = pytest.mark.gpu

NAMES = ("batch_20k_g16", "batch_20k_g70", "batch_20k_g128")


def problems(tracks=None):
    out = []
    for n in NAMES:
        w = mocatt.WORKLOADS[n]
        if tracks:
            w = w.with_(tracks=tracks)
        out.append(mocatt.generate(w))
    return out


def run_batch(handle, hps, opts=None):
    import torch

    dps = [mocatt.DeviceProblem(hp) for hp in hps]
    arr = (mocatt.MocProblem * len(dps))(*[dp.c_struct() for dp in dps])
    opts = opts or mocatt.default_opts()
    st = mocatt.lib().moc_attenuate_fwd_batch(handle.ptr, arr, len(dps), C.byref(opts),
                                              C.c_void_p(torch.cuda.current_stream().cuda_stream))
    handle.check(st)
    assert handle.synchronize() == 0
    return dps, arr


@pytest.mark.parametrize("chunk", [0, -1, 64])
def test_batch_matches_oracle_and_single_calls(handle, chunk):
    """Each problem of the batch against the FP64 oracle, and against a single call that
    cuts its tracks the same way (chunk -1: no cuts; 64: tracks of more than 256 segments
    cut into 64-segment chunks; 0: the automatic length, from the whole batch's size in
    the batch, so the single calls are compared only with the oracle)."""
    hps = problems(tracks=1500)
    opts = mocatt.default_opts(track_chunk=chunk)
    dps, _ = run_batch(handle, hps, opts)
    for hp, dp in zip(hps, dps):
        psi, ff = dp.to_host("psi"), dp.to_host("fine_flux")
        parity.check_plain(psi, ff, oracle.fwd_fp64(hp), hp.G)
        if hp.Gs > hp.G:
            assert not ff[:, hp.G:].any()
        if chunk == 0:
            continue
        single = mocatt.DeviceProblem(hp)
        handle.fwd(single, opts)
        assert handle.synchronize() == 0
        d = np.abs(psi[:, :hp.G].astype(np.float64) - single.to_host("psi")[:, :hp.G])
        assert np.all(d <= 1e-6 * np.abs(psi[:, :hp.G]) + 1e-30)


def test_batch_full_size_and_graph_replay(handle):
    """All three problems at full size (20,000 tracks each, ~6M segments); the second
    call with the same buffers replays the captured graph."""
    hps = problems()
    for hp in hps:
        assert 5.5e6 < hp.S < 6.5e6
    dps, arr = run_batch(handle, hps)
    first = [(dp.to_host("psi"), dp.to_host("fine_flux")) for dp in dps]
    for hp, (psi, ff) in zip(hps, first):
        parity.check_plain(psi, ff, oracle.fwd_fp64(hp), hp.G)
    # replay on the same buffers after restoring the inputs
    import torch

    for hp, dp in zip(hps, dps):
        dp.psi.copy_(torch.from_numpy(hp.psi))
        dp.fine_flux.zero_()
    opts = mocatt.default_opts()
    handle.check(mocatt.lib().moc_attenuate_fwd_batch(handle.ptr, arr, 3, C.byref(opts), None))
    assert handle.synchronize() == 0
    for dp, (psi, _) in zip(dps, first):
        np.testing.assert_array_equal(dp.to_host("psi"), psi)


def test_autotuner_reports_and_restores(handle):
    hps = problems(tracks=2000)
    dps = [mocatt.DeviceProblem(hp) for hp in hps]
    arr = (mocatt.MocProblem * 3)(*[dp.c_struct() for dp in dps])
    res = mocatt.MocTuneResult()
    opts = mocatt.default_opts()
    handle.check(mocatt.lib().moc_autotune_batch(handle.ptr, arr, 3, C.byref(opts), None,
                                                 C.byref(res)))
    assert res.n_candidates == 48  # groups per lane {1, 2, 4} x tracks per block 1..16
    assert res.vec in (1, 2, 4) and 1 <= res.warps_per_block <= 16
    assert res.tracks_per_block == res.warps_per_block
    assert res.best_ms == min(res.candidate_ms[:res.n_candidates])
    print({(res.candidate_vec[k], res.candidate_warps[k]): round(res.candidate_ms[k], 3)
           for k in range(res.n_candidates)}, "tracks/block", res.tracks_per_block)
    for hp, dp in zip(hps, dps):  # psi and fine_flux are left as they were
        np.testing.assert_array_equal(dp.to_host("psi"), hp.psi)
        assert not dp.to_host("fine_flux").any()
    # the tuned choice is used by the next batch call, and it is still correct
    handle.check(mocatt.lib().moc_attenuate_fwd_batch(handle.ptr, arr, 3, C.byref(opts), None))
    assert handle.synchronize() == 0
    for hp, dp in zip(hps, dps):
        parity.check_plain(dp.to_host("psi"), dp.to_host("fine_flux"), oracle.fwd_fp64(hp), hp.G)


def test_batch_rejects_bad_sets(handle):
    hps = problems(tracks=10)
    dps = [mocatt.DeviceProblem(hp) for hp in hps]
    arr = (mocatt.MocProblem * 3)(*[dp.c_struct() for dp in dps])
    L = mocatt.lib()
    o = mocatt.default_opts()
    assert L.moc_attenuate_fwd_batch(handle.ptr, arr, 0, C.byref(o), None) == \
        mocatt.MOC_ERR_INVALID_ARG
    assert L.moc_attenuate_fwd_batch(handle.ptr, arr, 9, C.byref(o), None) == \
        mocatt.MOC_ERR_INVALID_ARG
    bad = mocatt.default_opts(precision=mocatt.MOC_PREC_BF16)
    assert L.moc_attenuate_fwd_batch(handle.ptr, arr, 3, C.byref(bad), None) == \
        mocatt.MOC_ERR_UNSUPPORTED
    one = mocatt.default_opts(vec=1)  # G = 128 at one group per lane: 4 ranges, still fine
    handle.check(L.moc_attenuate_fwd_batch(handle.ptr, arr, 3, C.byref(one), None))
    assert handle.synchronize() == 0
