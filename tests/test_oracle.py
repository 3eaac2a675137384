"""The oracle itself: pinned against the reference, then checked for its own accuracy.

1. Golden fixtures (tests/golden, made by make_golden.py from the reference's own
   attenuate_segment) reproduce through the oracle's FP32 restatement bit for bit.
2. Where the reference sources are present, the pin is re-run live on fresh seeds.
3. The FP64 oracle and its error-magnitude companion bound the FP32 restatement.
4. The FP64 adjoint agrees with FP64 central differences.
5. What the 16-bit storage of the precision forms does to the problem itself (the storage
   term, reported apart from the forms' arithmetic error).
"""
import os
import platform

import numpy as np
import pytest

import mocatt
import oracle
import parity

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
EXACT_HOST = platform.machine() == "x86_64"  # the fixtures were made on x86_64


def load_problem(path):
    z = np.load(path)
    hp = mocatt.HostProblem(int(z["R"]), int(z["I"]), int(z["G"]), int(z["Gs"]), int(z["T"]),
                            int(z["S"]), z["track_offsets"], z["seg_region"],
                            z["seg_interval"], z["seg_ds"], z["sigT"], z["source"],
                            z["fine_flux"], z["psi"])
    return hp, z


@pytest.mark.parametrize("name", ["pin_exp_g64", "pin_table_g64", "pin_exp_g16_i3",
                                  "pin_exp_g128_i7"])
def test_golden_reference_outputs(name):
    hp, z = load_problem(os.path.join(GOLDEN, name + ".npz"))
    opts = mocatt.default_opts()
    if str(z["mode"]) == "table":
        t = np.load(os.path.join(GOLDEN, "table_ref.npz"))
        opts = mocatt.default_opts(exp_mode=mocatt.MOC_EXP_TABLE, table_points=int(t["n"]),
                                   table_max=float(t["max_val"]))
    psi, ff = oracle.fwd_fp32(hp, opts)
    if EXACT_HOST:
        np.testing.assert_array_equal(psi, z["out_psi"])
        np.testing.assert_array_equal(ff, z["out_ff"])
    else:  # another libm's expf may differ by an ulp: hold to the FP32 tolerance
        ref = oracle.fwd_fp64(hp, opts)
        parity.check_plain(z["out_psi"], z["out_ff"], ref, hp.G)
        parity.check_plain(psi, ff, ref, hp.G)


def test_golden_reference_table():
    t = np.load(os.path.join(GOLDEN, "table_ref.npz"))
    assert int(t["n"]) == 353  # (int)(10 * sqrt(1 / (8 * 0.01 * 0.01)))
    vals, dx, lk = oracle.table(int(t["n"]), float(t["max_val"]))
    if EXACT_HOST:
        np.testing.assert_array_equal(vals, t["values"])
    else:
        np.testing.assert_allclose(vals, t["values"], rtol=2 ** -23, atol=2 ** -24)
    assert dx == float(t["dx"]) and lk == float(t["lookup_max"])
    # the reference's slope sign: values[2n] = -exp(-n dx) (the tangent would be +)
    assert np.all(vals[2::2] < 0)
    # matches 1 - exp(-x) only at grid points
    x = np.float32(5 * dx)
    assert abs(oracle.lib().oracle_table_lookup(vals.ctypes.data, dx, lk, x) -
               (1 - np.exp(-float(x)))) < 1e-6


needs_ref = pytest.mark.skipif(not oracle.pinref_available(),
                               reason="reference sources not mounted here")


@needs_ref
@pytest.mark.parametrize("seed,G,I", [(21, 64, 5), (22, 128, 5), (23, 8, 2), (24, 36, 9)])
def test_live_pin_exp(seed, G, I):
    w = mocatt.WORKLOADS["sweep_1M_g64"].with_(seed=seed, groups=G, intervals=I,
                                                regions=25, tracks=20, segments=2000)
    hp = mocatt.generate(w, group_stride=G if G % 4 == 0 else None)
    hp.seg_ds[:] = np.float32(0.7)
    a = oracle.fwd_fp32(hp)
    b = oracle.pinref_sweep(hp)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


@needs_ref
@pytest.mark.parametrize("precision,maxv", [(0.01, 10.0), (0.001, 10.0), (0.05, 4.0)])
def test_live_pin_table(precision, maxv):
    vals, n, dx, lk = oracle.pinref_table(precision, maxv)
    mine, mdx, mlk = oracle.table(n, maxv)
    np.testing.assert_array_equal(vals, mine)
    assert (dx, lk) == (mdx, mlk)
    # and the library's own builder
    lv, ldx, llk = mocatt.build_exp_table(n, maxv)
    np.testing.assert_array_equal(vals, lv)
    assert (ldx, llk) == (dx, lk)
    hp = mocatt.generate(mocatt.WORKLOADS["sweep_1M_g64"].with_(seed=31, regions=25,
                                                                 tracks=20, segments=2000))
    hp.seg_ds[:] = np.float32(0.7)
    opts = mocatt.default_opts(exp_mode=mocatt.MOC_EXP_TABLE, table_points=n, table_max=maxv)
    a = oracle.fwd_fp32(hp, opts)
    b = oracle.pinref_sweep(hp, vals, dx, lk)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("wl,over", [
    ("sweep_1M_g64", dict(regions=60, tracks=30, segments=6000)),
    ("widetau_50M_g128", dict(regions=20, tracks=10, segments=2000, groups=32)),
])
def test_fp64_companion_bounds_fp32(wl, over):
    """The FP32 restatement stays inside the plain tolerance of the FP64 oracle, in both
    exp modes, also where tau spans [1e-6, 40] and the reference formula cancels."""
    hp = mocatt.generate(mocatt.WORKLOADS[wl].with_(**over))
    for opts in (mocatt.default_opts(),
                 mocatt.default_opts(exp_mode=mocatt.MOC_EXP_TABLE, table_points=10000)):
        psi, ff = oracle.fwd_fp32(hp, opts)
        ref = oracle.fwd_fp64(hp, opts)
        parity.check_plain(psi, ff, ref, hp.G, k=4.0)


def test_fp64_series_branch_continuity():
    """tau - e and the cubic switch from series to direct at tau = 1: the oracle's output
    is smooth across the switch."""
    base = mocatt.WORKLOADS["sweep_1M_g64"].with_(regions=4, tracks=1, segments=1, groups=4)
    hp = mocatt.generate(base)
    outs = []
    for ds in (np.nextafter(np.float32(1.0), np.float32(0)), np.float32(1.0)):
        q = hp.copy()
        q.sigT[:] = 1.0
        q.seg_ds[:] = ds
        outs.append(oracle.fwd_fp64(q)["psi"][0, :4])
    np.testing.assert_allclose(outs[0], outs[1], rtol=1e-6)


@pytest.mark.parametrize("prec,u", [(mocatt.MOC_PREC_BF16, 2.0 ** -9),
                                     (mocatt.MOC_PREC_FP16, 2.0 ** -11)])
def test_storage_rounding_effect(prec, u):
    """What 16-bit storage does to the problem itself, apart from any arithmetic: the FP64
    oracle on the cell blocks as a 16-bit form stores them (sigT and the FP32 axial
    coefficients rounded to nearest) against the FP64 oracle on the FP32 inputs, on the
    wide-tau inputs the forms are graded on. The forms' own arithmetic error is measured
    against the first of these (on the GPU); this is the separate storage term. Normwise,
    the outputs move by about the storage format's unit roundoff u, between u / 8 and 4 u:
    BF16 storage shifts psi and fine_flux by ~4e-3, FP16 by ~5e-4, far above 1e-5."""
    hp = mocatt.generate(mocatt.WORKLOADS["widetau_50M_g128"].with_(
        regions=400, tracks=400, segments=200_000))
    ref = oracle.fwd_fp64(hp)
    qp, coef = oracle.quantized_inputs(hp, prec)
    q = oracle.fwd_fp64_coef(qp, coef)
    G = hp.G
    out = {}
    for k in ("psi", "ff"):
        d = q[k][:, :G] - ref[k][:, :G]
        out[k] = float(np.linalg.norm(d) / np.linalg.norm(ref[k][:, :G]))
        assert u / 8 <= out[k] <= 4 * u, (k, out[k], u)
    print("storage rounding, normwise:", out)
    # the FP32 fit of the coefficients alone (what FP32 storage stores) is ~1e-7
    qp, coef = oracle.quantized_inputs(hp, mocatt.MOC_PREC_FP32_STABLE)
    q = oracle.fwd_fp64_coef(qp, coef)
    for k in ("psi", "ff"):
        d = q[k][:, :G] - ref[k][:, :G]
        assert np.linalg.norm(d) / np.linalg.norm(ref[k][:, :G]) <= 1e-6


def test_fp32_omp_matches_sequential():
    hp = mocatt.generate(mocatt.WORKLOADS["sweep_1M_g64"].with_(regions=50, tracks=40,
                                                                 segments=8000))
    p1, f1 = oracle.fwd_fp32(hp)
    p2, f2 = oracle.fwd_fp32(hp, threads=4)
    np.testing.assert_array_equal(p1, p2)
    # tallies are added in another order: both sums stay inside the FP32 tolerance
    ref = oracle.fwd_fp64(hp)
    parity.check_plain(p1, f1, ref, hp.G)
    parity.check_plain(p2, f2, ref, hp.G)


def test_fp64_adjoint_vs_central_differences():
    """FP64 adjoint vs FP64 central differences (h = 1e-6) on random parameters."""
    w = mocatt.WORKLOADS["adjoint_2M_g64"].with_(tracks=12, regions=10, groups=8,
                                                  lognormal=(40.0, 0.9005, 1, 200))
    hp = mocatt.generate(w)
    rng = np.random.default_rng(5)
    wgt = np.zeros((hp.R * hp.I, hp.Gs)); wgt[:, :hp.G] = rng.standard_normal((hp.R * hp.I, hp.G))
    v = np.zeros((hp.T, hp.Gs)); v[:, :hp.G] = rng.standard_normal((hp.T, hp.G))
    adj = oracle.adj_fp64(hp, wgt, v)
    sig = hp.sigT.astype(np.float64)
    src = hp.source.astype(np.float64)
    psi = hp.psi.astype(np.float64)
    h = 1e-6
    checks = []
    for kind, arr, grad in (("sigT", sig, adj["d_sigT"]), ("source", src, adj["d_source"]),
                            ("psi", psi, adj["d_psi_in"])):
        for _ in range(8):
            i = rng.integers(arr.shape[0]); g = int(rng.integers(hp.G))
            a_p, a_m = arr.copy(), arr.copy()
            a_p[i, g] += h
            a_m[i, g] -= h
            args_p = {"sigT": sig, "source": src, "psi": psi}
            args_m = dict(args_p)
            args_p[kind], args_m[kind] = a_p, a_m
            lp = oracle.loss_fp64(hp, args_p["sigT"], args_p["source"], args_p["psi"], wgt, v, g)
            lm = oracle.loss_fp64(hp, args_m["sigT"], args_m["source"], args_m["psi"], wgt, v, g)
            fd = (lp - lm) / (2 * h)
            checks.append((kind, fd, grad[i, g]))
            # truncation O(h^2) plus the rounding of L itself amplified by 1/h
            tol = 1e-6 * max(1.0, abs(fd)) + 64 * 2.0 ** -52 * max(abs(lp), abs(lm)) / h
            assert abs(fd - grad[i, g]) <= tol, (kind, i, g, fd, grad[i, g], lp)
    assert len(checks) == 24
