"""Track generation (include/moc_tracks.h) without a GPU: libmocatt's plan against the
oracle's restatement, bit for bit, and properties of the oracle's segments that any
correct ray tracer has: lengths add up to the track, a reversed track mirrors its
forward twin, cell volumes add up to the box, and the track-length estimate of every
region's volume converges to it. The reference draws its segments at random
(src/cpu/kernel.c:47-50) and has no tracer to pin against."""
import ctypes as C

import numpy as np
import pytest

import mocatt
import oracle

CONFIGS = {
    "3x2_both": (dict(nx=3, ny=2, n_axial=2, height=10.0),
                 dict(n_azim=4, n_polar=4, spacing=0.3, axial_spacing=1.0, both_directions=1)),
    "1x1_8rings": (dict(nx=1, ny=1, n_rings=8, n_axial=1, n_intervals=2, pitch=1.0,
                        fuel_radius=0.44, height=3.0),
                   dict(n_azim=2, n_polar=2, spacing=0.05, axial_spacing=0.3,
                        both_directions=1)),
    "5x7_thin": (dict(nx=5, ny=7, n_rings=1, n_axial=3, n_intervals=7, pitch=2.0,
                      fuel_radius=0.1, height=13.0),
                 dict(n_azim=6, n_polar=8, spacing=0.17, axial_spacing=0.7,
                      both_directions=1)),
    "17x17": (dict(nx=17, ny=17, n_axial=4, height=20.0),
              dict(n_azim=8, n_polar=4, spacing=0.1, axial_spacing=1.0)),
}


def config(name):
    g, q = CONFIGS[name]
    return mocatt.geometry(**g), mocatt.quadrature(**q)


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_plan_matches_oracle(name):
    g, q = config(name)
    a = mocatt.tracks_plan(g, q)
    b = oracle.tracks_plan(g, q)
    assert len(a) > 0
    assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_plan_records(name):
    g, q = config(name)
    a = mocatt.tracks_plan(g, q)
    W, Y = g.nx * g.pitch, g.ny * g.pitch
    assert np.all(np.isfinite(a["tb"])) and np.all(a["tb"] > a["ta"]) and np.all(a["ta"] >= 0)
    np.testing.assert_allclose(a["ux"] ** 2 + a["uy"] ** 2, 1.0, rtol=1e-15)
    assert np.all(a["rsin"] >= 1.0)
    assert np.all((a["x0"] >= 0) & (a["x0"] <= W) & (a["y0"] >= 0) & (a["y0"] <= Y))
    assert np.all((a["za"] >= 0) & (a["za"] <= g.height * (1 + 1e-15)))
    # entry exactly on a face of the lattice
    on_face = (a["x0"] == 0) | (a["x0"] == W) | (a["y0"] == 0)
    assert on_face.all()
    if q.both_directions:
        np.testing.assert_array_equal(a["reversed"], np.arange(len(a)) % 2)
        fwd = a[0::2].copy()
        rev = a[1::2].copy()
        rev["reversed"] = 0
        assert fwd.tobytes() == rev.tobytes()
    # every direction bin is present
    assert set(np.unique(a["azim"])) == set(range(q.n_azim))
    assert set(np.unique(a["polar"])) == set(range(q.n_polar))


@pytest.mark.parametrize("name", ["3x2_both", "1x1_8rings", "5x7_thin"])
def test_oracle_segments_cover_tracks(name):
    g, q = config(name)
    a = mocatt.tracks_plan(g, q)
    off, reg, itv, ds = oracle.trace(g, a)
    R = mocatt.geometry_regions(g)
    assert off[-1] == len(reg) > len(a)
    assert reg.min() >= 0 and reg.max() < R
    assert int(itv.max()) < g.n_intervals
    assert np.all(ds > 0)
    per_track = np.add.reduceat(ds.astype(np.float64), off[:-1])
    np.testing.assert_allclose(per_track, (a["tb"] - a["ta"]) * a["rsin"], rtol=2e-6)
    if q.both_directions:
        for t in range(0, min(len(a), 400), 2):
            f = slice(off[t], off[t + 1])
            r = slice(off[t + 1], off[t + 2])
            np.testing.assert_array_equal(reg[f][::-1], reg[r])
            np.testing.assert_array_equal(itv[f][::-1], itv[r])
            np.testing.assert_array_equal(ds[f][::-1], ds[r])


def test_volumes_add_up():
    g, _ = config("5x7_thin")
    v = mocatt.geometry_volumes(g)
    assert len(v) == mocatt.geometry_regions(g) * g.n_intervals
    np.testing.assert_allclose(v.sum(), g.nx * g.ny * g.pitch ** 2 * g.height, rtol=1e-12)
    K, I = g.n_rings, g.n_intervals
    rings = v.reshape(g.nx * g.ny, K + 1, g.n_axial, I)
    np.testing.assert_allclose(rings[:, :K].sum(axis=(0, 2, 3)),
                               np.pi * g.fuel_radius ** 2 * g.nx * g.ny * g.height / K,
                               rtol=1e-12)


def test_track_length_estimate_of_volumes():
    """sum over tracks of weight * (length inside a region) -> 4 pi V for every region as
    the spacings shrink (each direction bin's tracks tile the box)."""
    g = mocatt.geometry(nx=2, ny=2, n_rings=2, n_axial=2, n_intervals=2, pitch=1.26,
                        fuel_radius=0.54, height=4.0)
    q = mocatt.quadrature(n_azim=8, n_polar=6, spacing=0.02, axial_spacing=0.05,
                          both_directions=1)
    a = mocatt.tracks_plan(g, q)
    off, reg, itv, ds = oracle.trace(g, a)
    w = mocatt.tracks_weight(q)
    R = mocatt.geometry_regions(g)
    est = np.bincount(reg, weights=w * ds.astype(np.float64), minlength=R)
    vol = mocatt.geometry_volumes(g).reshape(R, g.n_intervals).sum(axis=1)
    rel = est / (4 * np.pi * vol) - 1.0
    assert np.abs(rel).max() < 2e-3, rel


def test_invalid_inputs():
    L = mocatt.lib()
    n = C.c_int64()
    for bad in (dict(fuel_radius=0.6), dict(n_rings=0), dict(n_rings=9), dict(n_intervals=1),
                dict(height=0.0), dict(nx=0)):
        g = mocatt.geometry(**bad)
        q = mocatt.quadrature()
        assert L.moc_tracks_plan(C.byref(g), C.byref(q), None, 0, C.byref(n)) == \
            mocatt.MOC_ERR_INVALID_ARG
        assert L.moc_geometry_regions(C.byref(g)) == 0
    g = mocatt.geometry()
    for bad in (dict(n_azim=3), dict(n_polar=5), dict(spacing=0.0), dict(both_directions=2)):
        q = mocatt.quadrature(**bad)
        assert L.moc_tracks_plan(C.byref(g), C.byref(q), None, 0, C.byref(n)) == \
            mocatt.MOC_ERR_INVALID_ARG
        assert L.moc_tracks_weight(C.byref(q)) == 0.0
    # a capacity smaller than the plan: the count is still reported, nothing overflows
    q = mocatt.quadrature(n_azim=2, n_polar=2, spacing=1.0, axial_spacing=10.0)
    full = mocatt.tracks_plan(g, q)
    part = np.zeros(3, mocatt.TRACK_DTYPE)
    assert L.moc_tracks_plan(C.byref(g), C.byref(q), part.ctypes.data, 3, C.byref(n)) == 0
    assert n.value == len(full) and part.tobytes() == full[:3].tobytes()
