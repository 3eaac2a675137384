"""The source update and power iteration (include/moc_transport.h) without a GPU: the
oracle's FP32 source update (the GPU's fused multiply-add chains) against its FP64
definition, a flat flux against the closed form, the synthetic cross sections, and the
oracle's power iteration (FP32 sweep oracle + source update, flat sources, vacuum
boundaries) on a small traced lattice. The reference kernel stops at the tallies, so
there is no reference iteration to pin against."""
import numpy as np
import pytest

import mocatt
import oracle


def small_case(M=4, G=8, R=30, I=5, seed=3):
    xs = mocatt.synth_xs(M, G, seed=seed)
    rng = np.random.default_rng(seed)
    mat = rng.integers(0, M, R).astype(np.int32)
    vol = rng.uniform(0.5, 2.0, R * I)
    tally = np.zeros((R * I, xs.Gs), np.float32)
    tally[:, :G] = rng.uniform(0.1, 3.0, (R * I, G)) * vol[:, None]
    return xs, mat, vol, tally


def test_synthetic_cross_sections():
    xs = mocatt.synth_xs(4, 16, seed=1)
    again = mocatt.synth_xs(4, 16, seed=1)
    for n in ("sigT", "scatter", "nu_fission", "chi"):
        np.testing.assert_array_equal(getattr(xs, n), getattr(again, n))
    G = xs.G
    out = xs.scatter[:, :, :G].sum(axis=2)          # scattering out of each group
    assert np.all(out < xs.sigT[:, :G])               # absorption > 0
    np.testing.assert_allclose(out[0] / xs.sigT[0, :G], 0.9, rtol=1e-5)
    assert not xs.nu_fission[0].any() and not xs.chi[0].any()
    np.testing.assert_allclose(xs.chi[1:, :G].sum(axis=1), 1.0, rtol=1e-6)
    assert not xs.scatter[:, :, G:].any() and not xs.sigT[:, G:].any()


@pytest.mark.parametrize("G", [1, 8, 33])
def test_source_update_fp32_against_fp64(G):
    xs, mat, vol, tally = small_case(G=G)
    s32, f32 = oracle.source_update(xs, mat, 30, 5, vol, tally, 1.1)
    s64, f64 = oracle.source_update(xs, mat, 30, 5, vol, tally.astype(np.float64), 1.1,
                                    fp64=True)
    np.testing.assert_allclose(s32[:, :G], s64[:, :G], rtol=2e-6 * max(G, 4), atol=0)
    assert not s32[:, G:].any()
    assert abs(f32 - f64) <= 1e-6 * f64


def test_flat_flux_closed_form():
    """phi = 1 in every cell and group: q[g] = (sum_g' S[g'][g] + chi[g] sum nu_f / k)/4pi,
    and the fission total is sum_c V[c] sum_g nu_f[m][g]."""
    xs, mat, vol, _ = small_case(G=12)
    G, R, I, k = xs.G, 30, 5, 0.93
    tally = np.zeros((R * I, xs.Gs))
    tally[:, :G] = vol[:, None]
    s64, f64 = oracle.source_update(xs, mat, R, I, vol, tally, k, fp64=True)
    m = np.repeat(mat, I)
    S = xs.scatter.astype(np.float64)[m][:, :, :G].sum(axis=1)
    nuf = xs.nu_fission.astype(np.float64)[m][:, :G].sum(axis=1)
    want = (S + xs.chi.astype(np.float64)[m][:, :G] * (nuf / k)[:, None]) / (4 * np.pi)
    np.testing.assert_allclose(s64[:, :G], want, rtol=1e-13)
    np.testing.assert_allclose(f64, (vol * nuf).sum(), rtol=1e-13)


def test_invalid_source_update_inputs():
    xs, mat, vol, tally = small_case()
    bad = mat.copy()
    bad[4] = xs.M
    with pytest.raises(ValueError):
        oracle.source_update(xs, bad, 30, 5, vol, tally, 1.0)
    with pytest.raises(ValueError):
        oracle.source_update(xs, mat, 30, 5, vol, tally, 0.0)


def traced_lattice(G=8, M=4):
    xs = mocatt.synth_xs(M, G)
    g = mocatt.geometry(nx=2, ny=2, n_rings=3, n_axial=2, n_intervals=5, height=10.0)
    q = mocatt.quadrature(n_azim=4, n_polar=4, spacing=0.1, axial_spacing=0.5,
                          both_directions=1)
    plan = mocatt.tracks_plan(g, q)
    off, reg, itv, ds = oracle.trace(g, plan)
    hp, mat, vol = mocatt.problem_from_tracks(g, off, reg, itv, ds, xs)
    opts = mocatt.default_opts(weight=mocatt.tracks_weight(q), zin=0.0, mu=0.0, mu2=0.0)
    return g, q, plan, xs, hp, mat, vol, opts


def test_oracle_power_iteration_converges():
    *_, xs, hp, mat, vol, opts = traced_lattice()
    ks = oracle.power_iteration(hp, opts, xs, mat, vol, 1.0, 40)
    assert all(0.0 < k < 2.0 for k in ks)
    assert abs(ks[-1] - ks[-2]) < 1e-4 * ks[-1]
    assert np.all(hp.fine_flux[:, :xs.G] > 0)
    assert np.all(hp.source[:, :xs.G] >= 0)
