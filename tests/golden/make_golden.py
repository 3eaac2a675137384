"""Regenerate the golden fixtures in this folder.

Run from the repository root, in a checkout where the reference sources are mounted
(the pinned reference is built from them by oracle/Makefile):

    python tests/golden/make_golden.py /path/to/SimpleMOC-kernel

Fixtures:
  pin_*.npz      seeded inputs with every ds = 0.7 (the reference hard-codes it,
                 src/cpu/kernel.c:104) and the outputs of the reference's own, unmodified
                 attenuate_segment (src/cpu/kernel.c:75-333) swept over the tracks in CSR
                 order: psi and fine_flux after the sweep.
  table_ref.npz  the reference's buildExponentialTable(0.01, 10.0) (src/cpu/init.c:81-117).
  synth_*.npz    generator outputs, to pin the input generator across hosts.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "simplemoc-kernel_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import mocatt  # noqa: E402
import mocatt_build  # noqa: E402
import oracle  # noqa: E402

# (fixture name, workload, overrides, exp mode)
PIN_CASES = [
    ("pin_exp_g64", "sweep_1M_g64", dict(regions=40, tracks=24, segments=2400), "exp"),
    ("pin_table_g64", "sweep_1M_g64", dict(regions=40, tracks=24, segments=2400), "table"),
    ("pin_exp_g16_i3", "sweep_1M_g64",
     dict(seed=11, regions=30, intervals=3, groups=16, tracks=10, segments=1500), "exp"),
    ("pin_exp_g128_i7", "sweep_50M_g128",
     dict(seed=12, regions=16, intervals=7, tracks=6, segments=900), "exp"),
]


def save_problem(path, hp, **extra):
    np.savez_compressed(
        path, R=hp.R, I=hp.I, G=hp.G, Gs=hp.Gs, T=hp.T, S=hp.S,
        track_offsets=hp.track_offsets, seg_region=hp.seg_region,
        seg_interval=hp.seg_interval, seg_ds=hp.seg_ds, sigT=hp.sigT, source=hp.source,
        fine_flux=hp.fine_flux, psi=hp.psi, **extra)


def main(reference_root):
    mocatt_build.build()
    oracle.build(reference_root)
    if not oracle.pinref_available():
        raise SystemExit("the pinned reference did not build")
    vals, n, dx, lk = oracle.pinref_table(0.01, 10.0)
    np.savez_compressed(os.path.join(HERE, "table_ref.npz"), values=vals, n=n, dx=dx,
                        lookup_max=lk, precision=0.01, max_val=10.0)
    for name, wl, over, mode in PIN_CASES:
        hp = mocatt.generate(mocatt.WORKLOADS[wl].with_(**over))
        hp.seg_ds[:] = np.float32(0.7)
        # a non-zero starting tally, as the reference's initialize_sources makes one
        hp.fine_flux[:, :hp.G] = mocatt.synth_uniform(99, 7, hp.R * hp.I * hp.G, 0.0, 1.0) \
            .reshape(hp.R * hp.I, hp.G)
        if mode == "table":
            psi, ff = oracle.pinref_sweep(hp, vals, dx, lk)
        else:
            psi, ff = oracle.pinref_sweep(hp)
        save_problem(os.path.join(HERE, name + ".npz"), hp, out_psi=psi, out_ff=ff,
                     mode=mode)
        print(name, hp.S, "segments")
    # generator pins
    hp = mocatt.generate(mocatt.WORKLOADS["sweep_1M_g64"].with_(regions=20, tracks=16,
                                                                  segments=500))
    save_problem(os.path.join(HERE, "synth_uniform.npz"), hp)
    hp = mocatt.generate(mocatt.WORKLOADS["widetau_50M_g128"].with_(regions=8, tracks=8,
                                                                      segments=300))
    save_problem(os.path.join(HERE, "synth_widetau.npz"), hp)
    spec = mocatt.WORKLOADS["batch_20k_g70"].spec()
    off = np.zeros(spec.n_tracks + 1, np.int64)
    mocatt.synth_lib().moc_synth_track_offsets(mocatt.C.byref(spec), off.ctypes.data)
    np.savez_compressed(os.path.join(HERE, "synth_lognormal_lengths.npz"),
                        lengths=np.diff(off).astype(np.int32))
    print("lognormal total", off[-1])


if __name__ == "__main__":
    # the reference's sources: the argument, MOC_REFERENCE_SOURCES, or a "reference"
    # directory beside this repository
    default = os.environ.get("MOC_REFERENCE_SOURCES") or os.path.join(
        os.path.dirname(ROOT), "reference")
    main(sys.argv[1] if len(sys.argv) > 1 else default)
