"""The seeded input generator: reproducible, correctly laid out, right distributions."""
import os

import numpy as np

import mocatt

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_reproduces_golden_inputs():
    for name, wl, over in (
        ("synth_uniform", "sweep_1M_g64", dict(regions=20, tracks=16, segments=500)),
        ("synth_widetau", "widetau_50M_g128", dict(regions=8, tracks=8, segments=300)),
    ):
        z = np.load(os.path.join(GOLDEN, name + ".npz"))
        hp = mocatt.generate(mocatt.WORKLOADS[wl].with_(**over))
        for k in ("track_offsets", "seg_region", "seg_interval", "seg_ds", "source", "psi"):
            np.testing.assert_array_equal(getattr(hp, k), z[k], err_msg=k)
        if name == "synth_uniform":
            np.testing.assert_array_equal(hp.sigT, z["sigT"])
        else:  # logU uses libm exp/log: allow an ulp across hosts
            np.testing.assert_allclose(hp.sigT, z["sigT"], rtol=2 ** -22)


def test_lognormal_lengths_golden():
    z = np.load(os.path.join(GOLDEN, "synth_lognormal_lengths.npz"))
    spec = mocatt.WORKLOADS["batch_20k_g70"].spec()
    off = np.zeros(spec.n_tracks + 1, np.int64)
    S = mocatt.synth_lib().moc_synth_track_offsets(mocatt.C.byref(spec), off.ctypes.data)
    lens = np.diff(off)
    # Box-Muller goes through libm: a track may differ by one segment across hosts
    assert np.mean(lens == z["lengths"]) > 0.999
    assert abs(S - int(z["lengths"].sum())) < 100
    assert lens.min() >= 1 and lens.max() <= 5000
    assert 5.5e6 < S < 6.5e6                      # about 6M segments
    assert abs(np.median(lens) - 200) < 10        # median 200


def test_csr_is_stable_counting_sort():
    w = mocatt.WORKLOADS["sweep_1M_g64"].with_(regions=30, tracks=50, segments=5000)
    hp = mocatt.generate(w)
    off = hp.track_offsets
    assert off[0] == 0 and off[-1] == hp.S and np.all(np.diff(off) >= 0)
    assert hp.seg_region.min() >= 0 and hp.seg_region.max() < hp.R
    assert hp.seg_interval.max() < hp.I
    assert hp.seg_ds.min() >= 0.01 and hp.seg_ds.max() < 1.0
    # uniform track assignment: lengths near S/T
    lens = np.diff(off)
    assert abs(lens.mean() - 100) < 1e-9 and lens.std() < 30


def test_distributions_and_padding():
    w = mocatt.WORKLOADS["sweep_1M_g64"].with_(groups=70, regions=100, tracks=10, segments=10)
    hp = mocatt.generate(w)
    assert hp.Gs == 72
    s = hp.sigT[:, :70]
    assert s.min() >= 0.1 and s.max() < 2.0 and abs(s.mean() - 1.05) < 0.02
    assert np.all(hp.sigT[:, 70:] == 1.0)       # padding stays finite
    assert np.all(hp.source[:, 70:] == 0.0) and np.all(hp.psi[:, 70:] == 0.0)
    assert 0.45 < hp.source[:, :70].mean() < 0.55
    wide = mocatt.generate(mocatt.WORKLOADS["widetau_50M_g128"].with_(regions=200, tracks=4,
                                                                       segments=20000))
    ls = np.log(wide.sigT[:, :128])
    assert ls.min() >= np.log(1e-3) - 1e-6 and ls.max() < np.log(20.0) + 1e-6
    assert wide.seg_ds.min() >= 1e-3 and wide.seg_ds.max() < 2.0


def test_draws_are_independent_of_batching():
    a = mocatt.synth_uniform(5, 9, 1000, 0.0, 1.0)
    b = mocatt.synth_uniform(5, 9, 10, 0.0, 1.0)
    np.testing.assert_array_equal(a[:10], b)
    n = mocatt.synth_normal(5, 10, 20000)
    assert abs(n.mean()) < 0.03 and abs(n.std() - 1) < 0.03
    r = mocatt.synth_randint(5, 11, 5000, 7)
    assert r.min() == 0 and r.max() == 6


def test_invalid_specs_rejected():
    spec = mocatt.WORKLOADS["sweep_1M_g64"].spec()
    spec.n_intervals = 1
    off = np.zeros(spec.n_tracks + 1, np.int64)
    assert mocatt.synth_lib().moc_synth_track_offsets(mocatt.C.byref(spec), off.ctypes.data) == -1
