"""The source update and power iteration on the GPU: moc_source_update bit for bit
against the oracle's FP32 restatement, moc_region_sigT, and moc_power_iteration against
the oracle's iteration (FP32 sweep oracle + source update) on a small traced lattice."""
import numpy as np
import pytest

import mocatt
import oracle
from test_transport import small_case, traced_lattice

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("G", [1, 8, 33, 128, 200])
def test_source_update_matches_oracle_bit_for_bit(handle, G):
    import torch

    xs, mat, vol, tally = small_case(M=5, G=G, R=40, I=5, seed=G)
    dxs = mocatt.DeviceXS(xs)
    src, fis = handle.source_update(dxs, torch.from_numpy(mat).cuda(), 5,
                                    torch.from_numpy(vol).cuda(),
                                    torch.from_numpy(tally).cuda(), 1.07)
    assert handle.synchronize() == 0
    want, f = oracle.source_update(xs, mat, 40, 5, vol, tally, 1.07)
    got = src.cpu().numpy()
    assert got[:, :G].tobytes() == want[:, :G].tobytes()
    assert not got[:, G:].any()
    # the fission total is an FP64 sum in another order
    assert abs(fis.item() - f) <= 1e-12 * f


def test_region_sigT_and_bad_material(handle):
    import torch

    xs = mocatt.synth_xs(3, 20)
    dxs = mocatt.DeviceXS(xs)
    mat = np.array([0, 2, 1, 1, 0, 2], np.int32)
    sig = handle.region_sigT(dxs, torch.from_numpy(mat).cuda())
    assert handle.synchronize() == 0
    np.testing.assert_array_equal(sig.cpu().numpy(), xs.sigT[mat])
    mat[3] = 7
    handle.region_sigT(dxs, torch.from_numpy(mat).cuda())
    assert handle.synchronize() == mocatt.MOC_ERR_BAD_INDEX
    assert handle.synchronize() == 0


def device_lattice():
    import torch

    g, q, plan, xs, hp, mat, vol, opts = traced_lattice()
    return (hp, mat, vol, opts, xs, mocatt.DeviceXS(xs), torch.from_numpy(mat).cuda(),
            torch.from_numpy(vol).cuda())


def test_power_iteration_matches_oracle(handle):
    """20 iterations from a flat flux with k = 1: the eigenvalue after each run of
    iterations and the final tallies against the oracle's iteration. The GPU sweep rounds
    differently (ex2.approx, one reciprocal) from the FP32 sweep oracle, so the two agree
    to FP32 accuracy, not bit for bit."""
    hp, mat, vol, opts, xs, dxs, dmat, dvol = device_lattice()
    ref = hp.copy()
    ks = oracle.power_iteration(ref, opts, xs, mat, vol, 1.0, 20)
    dp = mocatt.DeviceProblem(hp)
    k, it = handle.power_iteration(dp, opts, dxs, dmat, dvol, 1.0, 20)
    assert it == 20
    assert abs(k - ks[-1]) <= 2e-5 * ks[-1], (k, ks[-1])
    ff = dp.to_host("fine_flux")[:, :xs.G].astype(np.float64)
    want = ref.fine_flux[:, :xs.G].astype(np.float64)
    rel = np.abs(ff - want) / np.abs(want)
    assert rel.max() < 1e-3 and np.sqrt(np.mean(rel ** 2)) < 1e-4, (rel.max(), rel.mean())
    src = dp.to_host("source")[:, :xs.G].astype(np.float64)
    np.testing.assert_allclose(src, ref.source[:, :xs.G], rtol=1e-3, atol=1e-7)


def test_power_iteration_stops_at_tolerance(handle):
    hp, mat, vol, opts, xs, dxs, dmat, dvol = device_lattice()
    dp = mocatt.DeviceProblem(hp)
    k, it = handle.power_iteration(dp, opts, dxs, dmat, dvol, 1.0, 200, tolerance=1e-4)
    assert 3 < it < 200
    dp2 = mocatt.DeviceProblem(hp)
    k2, it2 = handle.power_iteration(dp2, opts, dxs, dmat, dvol, 1.0, it)
    # the same number of iterations gives the same eigenvalue (the tallies are FP32
    # atomic sums, so not bit for bit)
    assert it2 == it and abs(k2 - k) <= 1e-5 * k
