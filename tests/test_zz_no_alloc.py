"""moc_attenuate_fwd_noalloc, the entry point for callers that cannot allocate device
memory (their own pool allocator holds the GPU, or cudaMalloc's synchronisation is not
acceptable inside their sweep loop, or they have nowhere to keep a handle).

Called through the C ABI and compared with the handle-based moc_attenuate_fwd on the
same inputs, for two calls in a row: the second call reuses the fixed scratch array the
first one left behind, so it shows that everything that must start at zero is cleared.
This file sorts last so that a run stopping at the first failure has run every other
test before it.
"""
import ctypes as C

import numpy as np
import pytest

import mocatt
import oracle
import parity

pytestmark = pytest.mark.gpu


def _noalloc(dp, opts):
    import torch

    stream = torch.cuda.current_stream()
    st = mocatt.lib().moc_attenuate_fwd_noalloc(C.byref(dp.c_struct()), C.byref(opts),
                                                C.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    return st


@pytest.mark.parametrize("mode", ["full", "table"])
def test_noalloc_matches_handle_entry_point_twice(cuda, mode):
    # the reference's CPU-sized workload: 1,000,000 segments, G=64, 2,000 regions
    hp = mocatt.generate(mocatt.WORKLOADS["sweep_1M_g64"])
    opts = mocatt.default_opts()
    if mode == "table":
        opts = mocatt.default_opts(exp_mode=mocatt.MOC_EXP_TABLE, table_points=10_000,
                                   table_max=10.0)
    h = mocatt.Handle(0)
    ref_dp = mocatt.DeviceProblem(hp)
    # the no-allocation entry point sweeps every track in one pass: compare with the
    # handle entry point run the same way
    ref_opts = mocatt.MocFwdOpts.from_buffer_copy(opts)
    ref_opts.track_chunk = -1
    h.fwd(ref_dp, ref_opts)
    assert h.synchronize() == 0
    psi_ref, ff_ref = ref_dp.to_host("psi"), ref_dp.to_host("fine_flux")
    h.close()
    exact = oracle.fwd_fp64(hp, opts)
    bound = parity.bound_ff(exact, hp.G)
    for call in range(2):
        dp = mocatt.DeviceProblem(hp)
        assert _noalloc(dp, opts) == mocatt.MOC_OK, f"call {call}"
        psi, ff = dp.to_host("psi"), dp.to_host("fine_flux")
        # same kernels and coefficients: psi is bit-identical, tallies differ only in
        # the order of their atomic additions
        np.testing.assert_array_equal(psi, psi_ref)
        diff = np.abs(ff[:, :hp.G].astype(np.float64) - ff_ref[:, :hp.G])
        assert np.all(diff <= 2 * bound), f"call {call}: {diff.max()}"
        parity.check_plain(psi, ff, exact, hp.G)


def test_noalloc_rejects_oversize_and_bad_indices(cuda):
    big = mocatt.generate(mocatt.WORKLOADS["sweep_1M_g64"].with_(
        regions=3000, groups=128, tracks=4, segments=100))  # 3000*5*128 > 655,360
    assert _noalloc(mocatt.DeviceProblem(big), mocatt.default_opts()) == \
        mocatt.MOC_ERR_TOO_LARGE
    hp = mocatt.generate(mocatt.WORKLOADS["sweep_1M_g64"].with_(regions=50, tracks=8,
                                                                 segments=400))
    hp.seg_interval[3] = hp.I + 2
    dp = mocatt.DeviceProblem(hp)
    assert _noalloc(dp, mocatt.default_opts(checked=1)) == mocatt.MOC_ERR_BAD_INDEX
    np.testing.assert_array_equal(dp.to_host("psi"), hp.psi)
    assert not dp.to_host("fine_flux").any()
