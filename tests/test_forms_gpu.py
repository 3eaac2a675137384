"""The precision forms beside the plain sweep: stable small-tau math, FP32 / BF16 / FP16
storage, FP32 / compensated / FP64 tallies. Each is checked against the FP64 oracle run on
exactly the values the form stores (the rounding of storage is a separate, reported
effect). Printed per form: max and RMS relative error (floor 1e-6 of the RMS), normwise
relative error, and the worst ratio to the FP32 error bound of the oracle's companion."""
import numpy as np
import pytest

import mocatt
import oracle
import parity

pytestmark = pytest.mark.gpu

PRECISIONS = {"fp32s": mocatt.MOC_PREC_FP32_STABLE, "bf16": mocatt.MOC_PREC_BF16,
              "fp16": mocatt.MOC_PREC_FP16}
TALLIES = {"f32": mocatt.MOC_TALLY_ATOMIC_FP32, "comp": mocatt.MOC_TALLY_COMPENSATED,
           "f64": mocatt.MOC_TALLY_FP64}


def run(handle, hp, opts):
    dp = mocatt.DeviceProblem(hp)
    handle.fwd(dp, opts)
    assert handle.synchronize() == 0
    return dp.to_host("psi"), dp.to_host("fine_flux")


def report(hp, psi, ff, ref):
    G = hp.G
    out = {}
    for name, x, r in (("psi", psi, ref["psi"]), ("ff", ff, ref["ff"])):
        mx, rms = parity.rel_err(x[:, :G], r[:, :G])
        d = x[:, :G].astype(np.float64) - r[:, :G]
        out[name] = (mx, rms, float(np.linalg.norm(d) / np.linalg.norm(r[:, :G])))
    return out


def widetau():
    # tau over ~[1e-6, 40]: sigT ~ logU(1e-3, 20), ds ~ U(1e-3, 2)
    return mocatt.generate(mocatt.WORKLOADS["widetau_50M_g128"].with_(
        regions=400, tracks=400, segments=200_000))


@pytest.mark.parametrize("prec", list(PRECISIONS))
@pytest.mark.parametrize("tally", list(TALLIES))
def test_form_on_widetau(handle, prec, tally):
    """The stable math stays inside the FP32 error bound of the formula where the
    reference's expressions cancel (tau down to 1e-6)."""
    hp = widetau()
    opts = mocatt.default_opts(precision=PRECISIONS[prec], tally=TALLIES[tally])
    psi, ff = run(handle, hp, opts)
    qp, coef = oracle.quantized_inputs(hp, PRECISIONS[prec])
    ref = oracle.fwd_fp64_coef(qp, coef)
    rep = report(hp, psi, ff, ref)
    res = parity.check_plain(psi, ff, ref, hp.G)
    print(f"{prec}/{tally}: {rep} bound ratios {res}")
    assert rep["psi"][1] <= 1e-5 and rep["psi"][2] <= 1e-6
    assert rep["ff"][1] <= 1e-4 and rep["ff"][2] <= 1e-6


def test_stable_math_fixes_small_tau_cancellation(handle):
    """On the wide-tau inputs the plain form (the reference's expressions) loses the small-tau
    terms; the stable form keeps them. Both against the same FP64 oracle."""
    hp = widetau()
    ref = oracle.fwd_fp64(hp)
    psi_p, ff_p = run(handle, hp, mocatt.default_opts())
    psi_s, ff_s = run(handle, hp, mocatt.default_opts(precision=mocatt.MOC_PREC_FP32_STABLE))
    rp, rs = report(hp, psi_p, ff_p, ref), report(hp, psi_s, ff_s, ref)
    print("plain", rp, "stable", rs)
    assert rs["psi"][1] < rp["psi"][1] / 10
    # and the plain form is still inside its own (cancellation-aware) tolerance
    parity.check_plain(psi_p, ff_p, ref, hp.G)


def test_compensated_tally_is_correctly_rounded():
    """100,000 positive tallies into each of a few cells (a constant source makes
    q1 = q2 = 0): FP32 atomics drift by ~sqrt(n) units, the compensated and FP64 tallies
    stay at the per-tally arithmetic error."""
    import torch

    h = mocatt.Handle(0)
    hp = mocatt.generate(mocatt.WORKLOADS["sweep_1M_g64"].with_(regions=2, intervals=2,
                                                                 tracks=512, segments=400_000))
    hp.source[:] = 0.5
    ref = oracle.fwd_fp64_coef(hp, oracle.fit_fp32(hp))
    out = {}
    for tally in ("f32", "comp", "f64"):
        opts = mocatt.default_opts(precision=mocatt.MOC_PREC_FP32_STABLE, tally=TALLIES[tally])
        _, ff = run(h, hp, opts)
        out[tally] = parity.rel_err(ff[:, :hp.G], ref["ff"][:, :hp.G])[0]
    h.close()
    torch.cuda.synchronize()
    print(out)
    assert out["comp"] <= 2e-6 and out["f64"] <= 2e-6
    assert out["comp"] < out["f32"] / 4


REPORT_FORMS = {
    "plain_fp32": (mocatt.MOC_PREC_FP32, mocatt.MOC_TALLY_ATOMIC_FP32),
    "fp32_stable": (mocatt.MOC_PREC_FP32_STABLE, mocatt.MOC_TALLY_ATOMIC_FP32),
    "fp32_stable_compensated": (mocatt.MOC_PREC_FP32_STABLE, mocatt.MOC_TALLY_COMPENSATED),
    "fp32_stable_fp64": (mocatt.MOC_PREC_FP32_STABLE, mocatt.MOC_TALLY_FP64),
    "bf16_stable": (mocatt.MOC_PREC_BF16, mocatt.MOC_TALLY_ATOMIC_FP32),
    "bf16_stable_compensated": (mocatt.MOC_PREC_BF16, mocatt.MOC_TALLY_COMPENSATED),
    "fp16_stable": (mocatt.MOC_PREC_FP16, mocatt.MOC_TALLY_ATOMIC_FP32),
}
# The accuracy rule of the precision forms: normwise relative error <= 1e-5 for psi and for
# fine_flux against the FP64 oracle on the values the form stores. RMS and maximum relative
# errors are printed beside it, not part of it: single outputs that are sums which cancel
# (psi near zero after a long track, tallies of opposite-signed terms) can exceed 1e-5 while
# staying inside the FP32 companion bound, which every form must meet.
NORMWISE_TOL = 1e-5


def test_forms_accuracy_report(handle):
    """Error of every form bench.py times, on the wide-tau inputs, against the FP64 oracle
    on the values the form stores. With MOC_FORMS_REPORT=<path> the numbers are written
    there as JSON (bench.py reports them beside its timings)."""
    import json
    import os

    hp = widetau()
    report_all = {}
    for name, (prec, tally) in REPORT_FORMS.items():
        psi, ff = run(handle, hp, mocatt.default_opts(precision=prec, tally=tally))
        if prec == mocatt.MOC_PREC_FP32:
            ref = oracle.fwd_fp64(hp)
        else:
            qp, coef = oracle.quantized_inputs(hp, prec)
            ref = oracle.fwd_fp64_coef(qp, coef)
        rep = report(hp, psi, ff, ref)
        report_all[name] = {k: {"max_rel": v[0], "rms_rel": v[1], "normwise": v[2]}
                            for k, v in (("psi", rep["psi"]), ("fine_flux", rep["ff"]))}
    report_all["inputs"] = ("widetau_50M_g128 shapes cut to 200,000 segments, 400 tracks, "
                            "400 regions (sigT ~ logU(1e-3, 20), ds ~ U(1e-3, 2)); FP64 oracle "
                            "on the stored (rounded) sigT and coefficients; relative error "
                            "floor 1e-6 of the RMS")
    print(json.dumps(report_all, indent=1))
    path = os.environ.get("MOC_FORMS_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(report_all, f, indent=1)
    assert report_all["fp32_stable"]["psi"]["rms_rel"] < report_all["plain_fp32"]["psi"]["rms_rel"]


def test_precision_forms_reject_table_mode(handle):
    hp = mocatt.generate(mocatt.WORKLOADS["sweep_1M_g64"].with_(regions=20, tracks=4,
                                                                 segments=100))
    dp = mocatt.DeviceProblem(hp)
    o = mocatt.default_opts(precision=mocatt.MOC_PREC_BF16, exp_mode=mocatt.MOC_EXP_TABLE)
    st = mocatt.lib().moc_attenuate_fwd(handle.ptr, mocatt.C.byref(dp.c_struct()),
                                        mocatt.C.byref(o), None)
    assert st == mocatt.MOC_ERR_UNSUPPORTED
    o = mocatt.default_opts(tally=mocatt.MOC_TALLY_FP64)  # plain form: FP32 atomics only
    st = mocatt.lib().moc_attenuate_fwd(handle.ptr, mocatt.C.byref(dp.c_struct()),
                                        mocatt.C.byref(o), None)
    assert st == mocatt.MOC_ERR_UNSUPPORTED


def test_forms_widetau_50M_g128_full_size(cuda):
    """Every precision form on the wide-tau workload at its stated size (50,000,000
    segments x 128 groups, 100,000 tracks, 10,000 regions; sigT ~ logU(1e-3, 20),
    ds ~ U(1e-3, 2)), against the FP64 oracle on the values each form stores (one oracle
    run per storage kind). Prints max, RMS and normwise relative errors of psi and
    fine_flux; the stable forms must meet the normwise rule, every form the FP32
    companion bound. With MOC_FORMS_REPORT=<path> the numbers are written there as JSON."""
    import json
    import os

    import torch

    h = mocatt.Handle(0)
    hp = mocatt.generate(mocatt.WORKLOADS["widetau_50M_g128"])
    dp = mocatt.DeviceProblem(hp)
    psi0 = dp.psi.clone()
    threads = os.cpu_count() or 1
    outs = {}
    for name, (prec, tally) in REPORT_FORMS.items():
        dp.psi.copy_(psi0)
        dp.fine_flux.zero_()
        h.fwd(dp, mocatt.default_opts(precision=prec, tally=tally))
        assert h.synchronize() == 0, name
        outs[name] = (dp.to_host("psi"), dp.to_host("fine_flux"))
    h.close()
    del dp
    torch.cuda.empty_cache()
    storage = {mocatt.MOC_PREC_FP32: "fp32", mocatt.MOC_PREC_FP32_STABLE: "fp32",
               mocatt.MOC_PREC_BF16: "bf16", mocatt.MOC_PREC_FP16: "fp16"}
    report_all = {}
    for kind, prec in (("fp32", mocatt.MOC_PREC_FP32_STABLE), ("bf16", mocatt.MOC_PREC_BF16),
                       ("fp16", mocatt.MOC_PREC_FP16)):
        qp, coef = oracle.quantized_inputs(hp, prec)
        ref = oracle.fwd_fp64_coef(qp, coef, threads=threads)
        for name, (p_, _) in REPORT_FORMS.items():
            if storage[p_] != kind:
                continue
            psi, ff = outs.pop(name)
            rep = report(hp, psi, ff, ref)
            res = parity.check_plain(psi, ff, ref, hp.G)
            report_all[name] = {k: {"max_rel": v[0], "rms_rel": v[1], "normwise": v[2]}
                                for k, v in (("psi", rep["psi"]), ("fine_flux", rep["ff"]))}
            report_all[name]["bound_ratio"] = res
        del ref
    report_all["inputs"] = ("widetau_50M_g128 at full size: 50,000,000 segments x 128 groups, "
                            "100,000 tracks, 10,000 regions x 5 intervals, sigT ~ logU(1e-3, 20), "
                            "ds ~ U(1e-3, 2), seed 2; FP64 oracle on the stored (rounded) sigT "
                            "and coefficients; relative error floor 1e-6 of the RMS")
    print(json.dumps(report_all, indent=1))
    path = os.environ.get("MOC_FORMS_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(report_all, f, indent=1)
    for name, (prec, _) in REPORT_FORMS.items():
        if prec == mocatt.MOC_PREC_FP32:
            continue
        r = report_all[name]
        assert r["psi"]["normwise"] <= NORMWISE_TOL, (name, r)
        assert r["fine_flux"]["normwise"] <= NORMWISE_TOL, (name, r)
        # and no drift on the RMS either (measured 8e-6 to 3e-5 on this workload)
        assert r["psi"]["rms_rel"] <= 1e-4, (name, r)
    # the reference's expressions fail the rule on these inputs; the stable ones meet it
    assert report_all["plain_fp32"]["psi"]["rms_rel"] > 10 * report_all["fp32_stable"]["psi"]["rms_rel"]
