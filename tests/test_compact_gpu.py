"""moc_attenuate_fwd_compact: the sweep on compact descriptors (32-bit cells and half
lengths, 6 bytes per segment, the compact track file's payload). Its results equal
moc_attenuate_fwd's on the same problem with every length widened from its half (psi bit
for bit, fine_flux up to the order of atomic additions), are inside the FP64 oracle's
tolerance on those lengths, and bad cells are skipped and reported, or refused in checked
mode."""
import numpy as np
import pytest
import torch

import mocatt
import oracle
import parity

pytestmark = pytest.mark.gpu


def compact_arrays(hp):
    cell = (hp.seg_region.astype(np.uint32) * np.uint32(hp.I) +
            hp.seg_interval.astype(np.uint32))
    half = hp.seg_ds.astype(np.float16)
    return cell, half


def widened(hp):
    q = hp.copy()
    q.seg_ds = hp.seg_ds.astype(np.float16).astype(np.float32)
    return q


@pytest.mark.parametrize("name,kw,opts", [
    ("sweep_1M_g64", dict(regions=120, tracks=48, segments=12_000), {}),
    ("sweep_1M_g64", dict(), {}),
    ("sweep_1M_g64", dict(regions=120, tracks=48, segments=12_000, groups=70),
     dict(exp_mode=mocatt.MOC_EXP_TABLE, table_points=10_000)),
    ("adjoint_2M_g64", dict(tracks=2000), {}),                  # long tracks are cut
    ("widetau_50M_g128", dict(regions=400, tracks=400, segments=200_000),
     dict(precision=mocatt.MOC_PREC_FP32_STABLE)),
])
def test_compact_matches_widened_lengths(handle, name, kw, opts):
    hp = mocatt.generate(mocatt.WORKLOADS[name].with_(**kw))
    wide = widened(hp)
    ref_dp = mocatt.DeviceProblem(wide)
    o = mocatt.default_opts(**opts)
    handle.fwd(ref_dp, o)
    assert handle.synchronize() == 0
    cell, half = compact_arrays(hp)
    dp = mocatt.DeviceProblem(hp)
    d_cell = torch.from_numpy(cell).cuda()
    d_half = torch.from_numpy(half).cuda()
    handle.fwd_compact(dp, d_cell, d_half, o)
    assert handle.synchronize() == 0
    psi, ff = dp.to_host("psi"), dp.to_host("fine_flux")
    np.testing.assert_array_equal(psi, ref_dp.to_host("psi"))
    if opts.get("precision", mocatt.MOC_PREC_FP32) == mocatt.MOC_PREC_FP32:
        parity.check_plain(psi, ff, oracle.fwd_fp64(wide, o), hp.G)


def test_compact_bad_cells_are_reported(handle):
    hp = mocatt.generate(mocatt.WORKLOADS["sweep_1M_g64"].with_(regions=50, tracks=8,
                                                                 segments=400))
    cell, half = compact_arrays(hp)
    cell[17] = hp.R * hp.I  # one past the last cell
    dp = mocatt.DeviceProblem(hp)
    d_cell, d_half = torch.from_numpy(cell).cuda(), torch.from_numpy(half).cuda()
    handle.fwd_compact(dp, d_cell, d_half)
    assert handle.synchronize() == mocatt.MOC_ERR_BAD_INDEX
    dp2 = mocatt.DeviceProblem(hp)
    with pytest.raises(mocatt.MocError) as e:
        handle.fwd_compact(dp2, d_cell, d_half, mocatt.default_opts(checked=1))
    assert e.value.status == mocatt.MOC_ERR_BAD_INDEX
    np.testing.assert_array_equal(dp2.to_host("psi"), hp.psi)
    assert not dp2.to_host("fine_flux").any()
    # the refusal was the report: nothing is left for the next synchronisation
    assert handle.synchronize() == 0
