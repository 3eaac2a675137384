"""Seeded random configurations of the forward sweep against the FP64 oracle: small
problems with random group counts, track-length distributions, chunk lengths, groups per
lane, warps per block, prefetch, exp modes, precision forms and tally forms, so that the
combinations of the branch-free loop, the checked loop (G not a multiple of VEC), long-
track cuts and group-chunk-major items are all exercised together. Every case must sit
inside the FP32 tolerance of the formula (the oracle run on the values the form stores)."""
import numpy as np
import pytest

import mocatt
import oracle
import parity

pytestmark = pytest.mark.gpu

N_CASES = 120


def case(k: int):
    rng = np.random.default_rng(1000 + k)
    G = int(rng.choice([1, 2, 3, 5, 16, 31, 32, 33, 64, 65, 96, 127, 128, 130]))
    if rng.random() < 0.5:
        w = mocatt.WORKLOADS["adjoint_2M_g64"].with_(
            regions=int(rng.integers(3, 200)), groups=G, tracks=int(rng.integers(1, 300)),
            lognormal=(float(rng.uniform(20, 400)), 0.9, 0, int(rng.integers(50, 3000))))
    else:
        w = mocatt.WORKLOADS["sweep_1M_g64"].with_(
            regions=int(rng.integers(3, 200)), groups=G, tracks=int(rng.integers(1, 200)),
            segments=int(rng.integers(0, 60_000)))
    prec = int(rng.choice([mocatt.MOC_PREC_FP32, mocatt.MOC_PREC_FP32, mocatt.MOC_PREC_BF16,
                           mocatt.MOC_PREC_FP16, mocatt.MOC_PREC_FP32_STABLE]))
    opts = dict(
        precision=prec,
        track_chunk=int(rng.choice([0, 0, -1, 32, 64, 200])),
        vec=int(rng.choice([0, 1, 2, 4])),
        warps_per_block=int(rng.choice([0, 1, 4, 8, 16])),
    )
    if prec == mocatt.MOC_PREC_FP32:
        if rng.random() < 0.3:
            opts.update(exp_mode=mocatt.MOC_EXP_TABLE,
                        table_points=int(rng.choice([50, 353, 10_000])), table_max=10.0)
        if rng.random() < 0.2 and opts.get("exp_mode", 0) == 0:
            # the prefetch ring takes 16 KB of shared memory per warp at VEC = 4
            opts.update(prefetch=8, warps_per_block=min(opts["warps_per_block"], 8))
    else:
        opts.update(tally=int(rng.choice([mocatt.MOC_TALLY_ATOMIC_FP32,
                                          mocatt.MOC_TALLY_COMPENSATED,
                                          mocatt.MOC_TALLY_FP64])))
    return w, opts


@pytest.mark.parametrize("k", range(N_CASES))
def test_random_configuration(handle, k):
    w, kw = case(k)
    hp = mocatt.generate(w)
    opts = mocatt.default_opts(**kw)
    dp = mocatt.DeviceProblem(hp)
    handle.fwd(dp, opts)
    st = handle.synchronize()
    assert st == 0, (kw, mocatt.lib().moc_status_string(st))
    psi, ff = dp.to_host("psi"), dp.to_host("fine_flux")
    if kw["precision"] == mocatt.MOC_PREC_FP32:
        ref = oracle.fwd_fp64(hp, opts)
    else:
        qp, coef = oracle.quantized_inputs(hp, kw["precision"])
        ref = oracle.fwd_fp64_coef(qp, coef)
    res = parity.check_plain(psi, ff, ref, hp.G)
    # padding groups are never written
    if hp.Gs > hp.G:
        assert not ff[:, hp.G:].any()
        np.testing.assert_array_equal(psi[:, hp.G:], hp.psi[:, hp.G:])
    print(k, hp.S, hp.T, hp.G, kw, res)


def _rel(a, b, floor_frac=1e-3):
    d = np.abs(a.astype(np.float64) - b)
    den = np.maximum(np.abs(b), floor_frac * np.sqrt(np.mean(b * b)) + 1e-300)
    r = d / den
    return float(r.max()), float(np.sqrt(np.mean(r * r)))


@pytest.mark.parametrize("k", range(30))
def test_random_adjoint(handle, k):
    """The adjoint on random small problems (group counts, lengths, chunk lengths, groups
    per lane) against the FP64 CPU adjoint."""
    import torch

    rng = np.random.default_rng(5000 + k)
    G = int(rng.choice([1, 3, 16, 33, 64, 70, 128]))
    w = mocatt.WORKLOADS["adjoint_2M_g64"].with_(
        regions=int(rng.integers(3, 100)), groups=G, tracks=int(rng.integers(1, 150)),
        lognormal=(float(rng.uniform(20, 300)), 0.9, 0, int(rng.integers(50, 2000))))
    hp = mocatt.generate(w)
    opts = mocatt.default_opts(track_chunk=int(rng.choice([0, -1, 32, 100])),
                               vec=int(rng.choice([0, 1, 2, 4])))
    wt = np.zeros((hp.R * hp.I, hp.Gs), np.float32)
    vt = np.zeros((hp.T, hp.Gs), np.float32)
    wt[:, :G] = rng.standard_normal((hp.R * hp.I, G))
    vt[:, :G] = rng.standard_normal((hp.T, G))
    dp = mocatt.DeviceProblem(hp)
    ds, dsrc, dpsi = handle.adj(dp, torch.from_numpy(wt).cuda(), torch.from_numpy(vt).cuda(),
                                opts)
    assert handle.synchronize() == 0
    ref = oracle.adj_fp64(hp, wt.astype(np.float64), vt.astype(np.float64))
    for name, got, r in (("sigT", ds, "d_sigT"), ("source", dsrc, "d_source"),
                         ("psi_in", dpsi, "d_psi_in")):
        got = got.cpu().numpy()[:, :G]
        want = ref[r][:, :G]
        if not np.any(want):
            continue
        mx, rms = _rel(got, want)
        assert rms <= 1e-4 and mx <= 1e-2, (k, name, mx, rms, G, hp.S, hp.T)


@pytest.mark.parametrize("k", range(15))
def test_random_batch(handle, k):
    """Random sets of one to four problems (mixed group counts and track lengths) swept by
    the batching form, each problem against the FP64 oracle."""
    import ctypes as C

    import torch

    rng = np.random.default_rng(7000 + k)
    hps = []
    for p in range(int(rng.integers(1, 5))):
        G = int(rng.choice([1, 5, 16, 32, 33, 70, 128]))
        w = mocatt.WORKLOADS["batch_20k_g16"].with_(
            regions=int(rng.integers(3, 100)), groups=G, tracks=int(rng.integers(1, 400)),
            seed=100 * k + p,
            lognormal=(float(rng.uniform(20, 300)), 0.9, 0, int(rng.integers(50, 3000))))
        hps.append(mocatt.generate(w))
    dps = [mocatt.DeviceProblem(hp) for hp in hps]
    arr = (mocatt.MocProblem * len(dps))(*[dp.c_struct() for dp in dps])
    opts = mocatt.default_opts(track_chunk=int(rng.choice([0, -1, 32])),
                               vec=int(rng.choice([0, 1, 2])))
    handle.check(mocatt.lib().moc_attenuate_fwd_batch(
        handle.ptr, arr, len(dps), C.byref(opts),
        C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    assert handle.synchronize() == 0
    for hp, dp in zip(hps, dps):
        parity.check_plain(dp.to_host("psi"), dp.to_host("fine_flux"), oracle.fwd_fp64(hp),
                           hp.G)
