"""Tolerances for comparing the GPU sweep with the oracle (test infrastructure only).

The FP64 oracle returns, for every output x, an error-magnitude companion A (oracle.h):
the reference formula evaluated on magnitudes, with 1 - exp(-tau) counted as carrying
an absolute error of one unit. An FP32 evaluation of the reference formula satisfies
|x_fp32 - x| <= c * 2^-24 * A for a small operation count c; fine_flux sums add
hits * 2^-24 * sum|tally| for the order of the additions. Where no cancellation happens
A ~ |x| and the bound is a relative one; where the reference formula cancels, A keeps
the bound meaningful instead of dividing by a near-zero result.

The stated FP32 tolerance of the plain GPU sweep is K_PLAIN units of 2^-24 * A.
"""
from __future__ import annotations

import numpy as np

U32 = 2.0 ** -24
K_PLAIN = 8.0


def bound_psi(ref64: dict, G: int, k: float = K_PLAIN) -> np.ndarray:
    return k * U32 * ref64["a_psi"][:, :G]


def bound_ff(ref64: dict, G: int, k: float = K_PLAIN) -> np.ndarray:
    return U32 * (k * ref64["a_ff"][:, :G] + ref64["hits"][:, None] * ref64["abs_tally"][:, :G])


def ratio(x: np.ndarray, ref: np.ndarray, bound: np.ndarray) -> np.ndarray:
    """|x - ref| / bound, elementwise (0 where both are 0)."""
    d = np.abs(x.astype(np.float64) - ref)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(bound > 0, d / bound, np.where(d > 0, np.inf, 0.0))
    return r


def rel_err(x: np.ndarray, ref: np.ndarray, floor_frac: float = 1e-6) -> tuple[float, float]:
    """Max and RMS relative error with a floor: |x - ref| / max(|ref|, floor_frac * rms(ref))."""
    ref = np.asarray(ref, np.float64)
    d = np.abs(np.asarray(x, np.float64) - ref)
    rms_ref = float(np.sqrt(np.mean(ref * ref))) if ref.size else 0.0
    den = np.maximum(np.abs(ref), floor_frac * rms_ref)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(den > 0, d / den, 0.0)
    return float(r.max()) if r.size else 0.0, float(np.sqrt(np.mean(r * r))) if r.size else 0.0


def check_plain(psi: np.ndarray, ff: np.ndarray, ref64: dict, G: int,
                k: float = K_PLAIN) -> dict:
    """Check GPU (or FP32 oracle) outputs against the FP64 oracle with the plain
    tolerance. Returns the worst ratios; raises AssertionError on a violation."""
    rp = ratio(psi[:, :G], ref64["psi"][:, :G], bound_psi(ref64, G, k))
    rf = ratio(ff[:, :G], ref64["ff"][:, :G], bound_ff(ref64, G, k))
    out = {"psi_ratio_max": float(rp.max()) if rp.size else 0.0,
           "ff_ratio_max": float(rf.max()) if rf.size else 0.0}
    if rp.size and not np.all(rp <= 1.0):
        i = np.unravel_index(np.argmax(rp), rp.shape)
        raise AssertionError(f"psi outside tolerance at {i}: got {psi[i]}, oracle "
                             f"{ref64['psi'][i]}, ratio {rp[i]:.3g} ({out})")
    if rf.size and not np.all(rf <= 1.0):
        i = np.unravel_index(np.argmax(rf), rf.shape)
        raise AssertionError(f"fine_flux outside tolerance at {i}: got {ff[i]}, oracle "
                             f"{ref64['ff'][i]}, ratio {rf[i]:.3g} ({out})")
    return out
