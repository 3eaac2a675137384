"""Track generation on the GPU (moc_trace_count / moc_trace_segments) against the
oracle's sort-all-crossings tracer, bit for bit: offsets, regions, intervals and
lengths. Then the traced descriptors drive the sweep, checked against the FP64 oracle on
the same descriptors."""
import numpy as np
import pytest

import mocatt
import oracle
import parity
from test_tracks import CONFIGS, config

pytestmark = pytest.mark.gpu


def upload(plan):
    import torch

    return torch.from_numpy(plan.view(np.uint8)).cuda()


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_gpu_tracks_match_oracle(handle, name):
    g, q = config(name)
    plan = mocatt.tracks_plan(g, q)
    off, reg, itv, ds = handle.trace(g, upload(plan), len(plan))
    assert handle.synchronize() == 0
    o_off, o_reg, o_itv, o_ds = oracle.trace(g, plan)
    np.testing.assert_array_equal(off.cpu().numpy(), o_off)
    np.testing.assert_array_equal(reg.cpu().numpy(), o_reg)
    np.testing.assert_array_equal(itv.cpu().numpy(), o_itv)
    assert ds.cpu().numpy().tobytes() == o_ds.tobytes()


def test_assembly_plan_counts_and_sampled_tracks(handle):
    """A 17 x 17 assembly 200 cm tall at bench density: the total against the oracle's
    count, and 3,000 random tracks bit for bit."""
    g = mocatt.geometry()
    q = mocatt.quadrature(n_azim=8, n_polar=4, spacing=0.1, axial_spacing=2.0)
    plan = mocatt.tracks_plan(g, q)
    off, reg, itv, ds = handle.trace(g, upload(plan), len(plan))
    assert handle.synchronize() == 0
    off = off.cpu().numpy()
    assert off[-1] == oracle.trace_count_omp(g, plan)
    rng = np.random.default_rng(11)
    pick = np.sort(rng.choice(len(plan), size=3000, replace=False))
    o_off, o_reg, o_itv, o_ds = oracle.trace(g, plan[pick])
    idx = np.concatenate([np.arange(off[t], off[t + 1]) for t in pick])
    np.testing.assert_array_equal(np.diff(off)[pick], np.diff(o_off))
    np.testing.assert_array_equal(reg.cpu().numpy()[idx], o_reg)
    np.testing.assert_array_equal(itv.cpu().numpy()[idx], o_itv)
    assert ds.cpu().numpy()[idx].tobytes() == o_ds.tobytes()


def test_bad_track_record_is_reported(handle):
    """An inconsistent record (tb < ta, NaN direction) counts 0 segments and the call
    returns MOC_ERR_BAD_TRACK; the handle stays usable."""
    import torch

    g, q = config("3x2_both")
    plan = mocatt.tracks_plan(g, q)
    bad = plan.copy()
    bad["tb"][5] = bad["ta"][5] - 1.0
    bad["rux"][9] = np.nan
    with pytest.raises(mocatt.MocError) as e:
        handle.trace(g, upload(bad), len(bad))
    assert e.value.status == mocatt.MOC_ERR_BAD_TRACK
    assert handle.synchronize() == 0
    off, reg, itv, ds = handle.trace(g, upload(plan), len(plan))
    assert handle.synchronize() == 0
    assert off[-1].item() == oracle.trace(g, plan)[0][-1]
    # segments written against offsets from another plan: the mismatch is reported
    wrong = torch.zeros_like(off)
    import ctypes as C

    d_plan = upload(plan)
    st = mocatt.lib().moc_trace_segments(handle.ptr, C.byref(g), d_plan.data_ptr(),
                                         len(plan), wrong.data_ptr(), reg.data_ptr(),
                                         itv.data_ptr(), ds.data_ptr(),
                                         C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    assert handle.synchronize() == mocatt.MOC_ERR_BAD_TRACK
    assert handle.synchronize() == 0


@pytest.mark.parametrize("G", [16, 70])
def test_traced_problem_sweeps_like_the_oracle(handle, G):
    """Trace -> sweep: traced descriptors with seeded tables, the sweep against the FP64
    oracle run on the same descriptors."""
    g = mocatt.geometry(nx=4, ny=3, n_rings=2, n_axial=3, n_intervals=5, height=30.0)
    q = mocatt.quadrature(n_azim=4, n_polar=4, spacing=0.2, axial_spacing=2.0,
                          both_directions=1)
    plan = mocatt.tracks_plan(g, q)
    off, reg, itv, ds = handle.trace(g, upload(plan), len(plan))
    assert handle.synchronize() == 0
    R, I, T = mocatt.geometry_regions(g), g.n_intervals, len(plan)
    Gs = (G + 3) & ~3
    seed = 5
    sig = mocatt._aligned_empty((R, Gs), np.float32)
    sig[:] = mocatt.synth_uniform(seed, 1, R * Gs, 0.1, 2.0).reshape(R, Gs)
    src = mocatt._aligned_empty((R * I, Gs), np.float32)
    src[:] = mocatt.synth_uniform(seed, 2, R * I * Gs, 0.0, 1.0).reshape(R * I, Gs)
    psi = mocatt._aligned_empty((T, Gs), np.float32)
    psi[:] = mocatt.synth_uniform(seed, 3, T * Gs, 0.0, 1.0).reshape(T, Gs)
    ff = mocatt._aligned_empty((R * I, Gs), np.float32)
    ff[:] = 0
    off_h = off.cpu().numpy()
    hp = mocatt.HostProblem(R, I, G, Gs, T, int(off_h[-1]), off_h, reg.cpu().numpy(),
                            itv.cpu().numpy(), ds.cpu().numpy(), sig, src, ff, psi)
    opts = mocatt.default_opts(weight=mocatt.tracks_weight(q))
    dp = mocatt.DeviceProblem(hp)
    handle.fwd(dp, opts)
    assert handle.synchronize() == 0
    ref = oracle.fwd_fp64(hp, opts)
    parity.check_plain(dp.to_host("psi"), dp.to_host("fine_flux"), ref, G)
