"""ctypes bindings of the CPU oracle (oracle/oracle.h) and of the pinned reference.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg, as the checker or the timed CPU reference arm. The product never
imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "simplemoc-kernel_gb300"))
import mocatt  # noqa: E402  (struct definitions and the input generator)

LIB = os.path.join(HERE, "_build", "liboracle.so")
CPU_BENCH = os.path.join(HERE, "_build", "cpu_bench")
REF_DIR = os.path.join(HERE, "_ref")

_P = C.c_void_p
_PP = C.POINTER(mocatt.MocProblem)
_PO = C.POINTER(mocatt.MocFwdOpts)
_SIGS = {
    "oracle_build_table": (None, [C.c_int32, C.c_float, _P, C.POINTER(C.c_float),
                                  C.POINTER(C.c_float)]),
    "oracle_table_lookup": (C.c_float, [_P, C.c_float, C.c_float, C.c_float]),
    "oracle_fwd_fp32": (C.c_int, [_PP, _PO]),
    "oracle_fwd_fp32_omp": (C.c_int, [_PP, _PO, C.c_int]),
    "oracle_fwd_fp64": (C.c_int, [_PP, _PO, _P, _P, _P, _P, _P, _P, C.c_int]),
    "oracle_adj_fp64": (C.c_int, [_PP, _PO, _P, _P, _P, _P, _P, C.c_int]),
    "oracle_fit_fp32": (C.c_int, [_PP, _PO, _P]),
    "oracle_fwd_fp64_coef": (C.c_int, [_PP, _PO, _P, _P, _P, _P, _P, _P, _P, C.c_int]),
    "oracle_loss_fp64": (C.c_double, [_PP, _PO, _P, _P, _P, _P, _P, C.c_int32]),
    "oracle_tracks_plan": (C.c_int64, [C.POINTER(mocatt.MocGeometry),
                                       C.POINTER(mocatt.MocQuadrature), _P, C.c_int64]),
    "oracle_trace": (C.c_int64, [C.POINTER(mocatt.MocGeometry), _P, C.c_int64, _P, _P, _P,
                                 _P, C.c_int64]),
    "oracle_trace_omp": (C.c_int64, [C.POINTER(mocatt.MocGeometry), _P, C.c_int64, C.c_int]),
    "oracle_source_update_fp32": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _P, _P, _P, _P,
                                            C.c_int32, C.c_int32, _P, _P, C.c_double, _P,
                                            C.POINTER(C.c_double)]),
    "oracle_source_update_fp64": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _P, _P, _P, _P,
                                            C.c_int32, C.c_int32, _P, _P, C.c_double, _P,
                                            C.POINTER(C.c_double)]),
}

_lib = None


def build(reference_root: str | None = None) -> None:
    """make -C oracle (and the pinned reference when its sources are given)."""
    cmd = ["make", "-s", "-C", HERE, "all"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    if reference_root and os.path.isdir(os.path.join(reference_root, "src", "cpu")):
        r = subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={reference_root}"],
                           capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"reference pin build failed:\n{r.stdout}\n{r.stderr}")


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = C.CDLL(LIB)
        for n, (res, args) in _SIGS.items():
            f = getattr(_lib, n)
            f.restype = res
            f.argtypes = args
    return _lib


def table(n_points: int, max_val: float):
    vals = np.zeros(2 * n_points, np.float32)
    dx, lk = C.c_float(), C.c_float()
    lib().oracle_build_table(n_points, max_val, vals.ctypes.data, C.byref(dx), C.byref(lk))
    return vals, dx.value, lk.value


def fwd_fp32(hp: "mocatt.HostProblem", opts=None, threads: int | None = None):
    """Restated reference sweep in FP32 on a copy; returns (psi, fine_flux). threads=None
    runs the deterministic sequential sweep, else the OpenMP/lock version."""
    opts = opts or mocatt.default_opts()
    q = hp.copy()
    prob = q.c_struct()
    if threads is None:
        rc = lib().oracle_fwd_fp32(C.byref(prob), C.byref(opts))
    else:
        rc = lib().oracle_fwd_fp32_omp(C.byref(prob), C.byref(opts), threads)
    if rc:
        raise ValueError("oracle rejected the problem")
    return q.psi, q.fine_flux


def fwd_fp64(hp: "mocatt.HostProblem", opts=None, threads: int = 0) -> dict:
    """FP64 oracle with error-magnitude companions (see oracle.h)."""
    opts = opts or mocatt.default_opts()
    prob = hp.c_struct()
    ncell = hp.R * hp.I
    out = {k: np.zeros(shape, np.float64) for k, shape in (
        ("psi", (hp.T, hp.Gs)), ("ff", (ncell, hp.Gs)), ("a_psi", (hp.T, hp.Gs)),
        ("a_ff", (ncell, hp.Gs)), ("abs_tally", (ncell, hp.Gs)))}
    out["hits"] = np.zeros(ncell, np.int64)
    rc = lib().oracle_fwd_fp64(C.byref(prob), C.byref(opts), out["psi"].ctypes.data,
                               out["ff"].ctypes.data, out["a_psi"].ctypes.data,
                               out["a_ff"].ctypes.data, out["abs_tally"].ctypes.data,
                               out["hits"].ctypes.data, threads)
    if rc:
        raise ValueError("oracle rejected the problem")
    return out


def fit_fp32(hp, opts=None) -> np.ndarray:
    """The reference's FP32 axial coefficients (q0, q1*mu, q2*mu2), [R*I, 3, Gs]."""
    opts = opts or mocatt.default_opts()
    coef = np.zeros((hp.R * hp.I, 3, hp.Gs), np.float32)
    if lib().oracle_fit_fp32(C.byref(hp.c_struct()), C.byref(opts), coef.ctypes.data):
        raise ValueError("oracle rejected the problem")
    return coef


def round_bf16(x: np.ndarray) -> np.ndarray:
    """float32 values rounded to bfloat16, to nearest even, returned as float32."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def round_fp16(x: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(x, np.float32).astype(np.float16).astype(np.float32)


def quantized_inputs(hp, precision: int, opts=None):
    """(problem with sigT as the form stores it, coefficients as the form stores them):
    what a precision form computes from, for its FP64 reference."""
    coef = fit_fp32(hp, opts)
    q = hp.copy()
    if precision == mocatt.MOC_PREC_BF16:
        rnd = round_bf16
    elif precision == mocatt.MOC_PREC_FP16:
        rnd = round_fp16
    else:
        return q, coef
    q.sigT = rnd(hp.sigT).reshape(hp.sigT.shape)
    return q, rnd(coef).reshape(coef.shape)


def fwd_fp64_coef(hp, coef, opts=None, threads: int = 0) -> dict:
    """FP64 oracle on given coefficients (see oracle_fwd_fp64_coef)."""
    opts = opts or mocatt.default_opts()
    prob = hp.c_struct()
    coef = np.ascontiguousarray(coef, np.float32)
    ncell = hp.R * hp.I
    out = {k: np.zeros(shape, np.float64) for k, shape in (
        ("psi", (hp.T, hp.Gs)), ("ff", (ncell, hp.Gs)), ("a_psi", (hp.T, hp.Gs)),
        ("a_ff", (ncell, hp.Gs)), ("abs_tally", (ncell, hp.Gs)))}
    out["hits"] = np.zeros(ncell, np.int64)
    rc = lib().oracle_fwd_fp64_coef(C.byref(prob), C.byref(opts), coef.ctypes.data,
                                    out["psi"].ctypes.data, out["ff"].ctypes.data,
                                    out["a_psi"].ctypes.data, out["a_ff"].ctypes.data,
                                    out["abs_tally"].ctypes.data, out["hits"].ctypes.data,
                                    threads)
    if rc:
        raise ValueError("oracle rejected the problem")
    return out


def adj_fp64(hp, w, v, opts=None, threads: int = 0) -> dict:
    opts = opts or mocatt.default_opts()
    prob = hp.c_struct()
    w = np.ascontiguousarray(w, np.float64)
    v = np.ascontiguousarray(v, np.float64)
    out = {"d_sigT": np.zeros((hp.R, hp.Gs)), "d_source": np.zeros((hp.R * hp.I, hp.Gs)),
           "d_psi_in": np.zeros((hp.T, hp.Gs))}
    rc = lib().oracle_adj_fp64(C.byref(prob), C.byref(opts), w.ctypes.data, v.ctypes.data,
                               out["d_sigT"].ctypes.data, out["d_source"].ctypes.data,
                               out["d_psi_in"].ctypes.data, threads)
    if rc:
        raise ValueError("oracle rejected the problem")
    return out


def loss_fp64(hp, sigT, source, psi_in, w, v, group: int = -1, opts=None) -> float:
    opts = opts or mocatt.default_opts()
    prob = hp.c_struct()
    arrs = [np.ascontiguousarray(a, np.float64) for a in (sigT, source, psi_in, w, v)]
    return lib().oracle_loss_fp64(C.byref(prob), C.byref(opts),
                                  *[a.ctypes.data for a in arrs], group)


# ------------------------------------------------------------------------------------
# The pinned reference (oracle/_ref, built only where the reference sources exist)
# ------------------------------------------------------------------------------------
def pinref_available() -> bool:
    return all(os.path.exists(os.path.join(REF_DIR, f))
               for f in ("libpinref.so", "libpinref_table.so"))


def _pinlib(table_mode: bool):
    name = "libpinref_table.so" if table_mode else "libpinref.so"
    lib_ = C.CDLL(os.path.join(REF_DIR, name))
    lib_.pinref_sweep.restype = C.c_int
    lib_.pinref_sweep.argtypes = [_PP, _P, C.c_int32, C.c_float, C.c_float]
    lib_.pinref_build_table.restype = C.c_int
    lib_.pinref_build_table.argtypes = [C.c_float, C.c_float, _P, C.c_int32,
                                        C.POINTER(C.c_int32), C.POINTER(C.c_float),
                                        C.POINTER(C.c_float)]
    return lib_


def pinref_table(precision: float, max_val: float):
    """The reference's own buildExponentialTable(precision, maxVal)."""
    cap = 1 << 22
    vals = np.zeros(cap, np.float32)
    n, dx, lk = C.c_int32(), C.c_float(), C.c_float()
    if _pinlib(False).pinref_build_table(precision, max_val, vals.ctypes.data, cap,
                                         C.byref(n), C.byref(dx), C.byref(lk)):
        raise ValueError("table too large")
    return vals[:2 * n.value].copy(), n.value, dx.value, lk.value


def pinref_sweep(hp, table_values=None, table_dx=0.0, table_lookup=0.0):
    """The reference's attenuate_segment over every track (ds fixed at 0.7 by the
    reference); returns (psi, fine_flux) of a copy."""
    q = hp.copy()
    prob = q.c_struct()
    tm = table_values is not None
    tv = np.ascontiguousarray(table_values, np.float32) if tm else None
    rc = _pinlib(tm).pinref_sweep(C.byref(prob), tv.ctypes.data if tm else None,
                                  len(tv) // 2 if tm else 0, table_dx, table_lookup)
    if rc:
        raise ValueError("pinref rejected the problem")
    return q.psi, q.fine_flux


# ---- track generation ------------------------------------------------------------------

def tracks_plan(g, q) -> np.ndarray:
    """The oracle's restatement of moc_tracks_plan (TRACK_DTYPE array)."""
    L = lib()
    n = L.oracle_tracks_plan(C.byref(g), C.byref(q), None, 0)
    if n < 0:
        raise ValueError("invalid geometry or quadrature")
    out = np.zeros(n, mocatt.TRACK_DTYPE)
    if n:
        L.oracle_tracks_plan(C.byref(g), C.byref(q), out.ctypes.data, n)
    return out


def trace(g, tracks: np.ndarray):
    """Segments of every track by sorting all crossings: (offsets, region, interval, ds)."""
    L = lib()
    tracks = np.ascontiguousarray(tracks, mocatt.TRACK_DTYPE)
    T = len(tracks)
    off = np.zeros(T + 1, np.int64)
    tp = tracks.ctypes.data if T else None
    S = L.oracle_trace(C.byref(g), tp, T, off.ctypes.data, None, None, None, 0)
    if S < 0:
        raise ValueError("invalid geometry")
    reg = np.zeros(max(S, 1), np.int32)
    itv = np.zeros(max(S, 1), np.uint8)
    ds = np.zeros(max(S, 1), np.float32)
    L.oracle_trace(C.byref(g), tp, T, off.ctypes.data, reg.ctypes.data, itv.ctypes.data,
                   ds.ctypes.data, S)
    return off, reg[:S], itv[:S], ds[:S]


def trace_count_omp(g, tracks: np.ndarray, nthreads: int = 0) -> int:
    """Total segment count, OpenMP over tracks (the timed CPU arm)."""
    tracks = np.ascontiguousarray(tracks, mocatt.TRACK_DTYPE)
    return int(lib().oracle_trace_omp(C.byref(g), tracks.ctypes.data if len(tracks) else None,
                                      len(tracks), nthreads))


# ---- source update and power iteration ---------------------------------------------------

def source_update(xs, material, R, I, volume, tally, k, fp64=False):
    """The oracle's source update. xs: mocatt.HostXS; tally float32 [R*I, Gs] (float64 for
    fp64). Returns (source, fission total)."""
    L = lib()
    material = np.ascontiguousarray(material, np.int32)
    volume = np.ascontiguousarray(volume, np.float64)
    fis = C.c_double()
    if fp64:
        tally = np.ascontiguousarray(tally, np.float64)
        out = np.zeros(tally.shape, np.float64)
        fn = L.oracle_source_update_fp64
    else:
        tally = np.ascontiguousarray(tally, np.float32)
        out = np.zeros(tally.shape, np.float32)
        fn = L.oracle_source_update_fp32
    st = fn(xs.M, xs.G, xs.Gs, xs.scatter.ctypes.data, xs.nu_fission.ctypes.data,
            xs.chi.ctypes.data, material.ctypes.data, R, I, volume.ctypes.data,
            tally.ctypes.data, float(k), out.ctypes.data, C.byref(fis))
    if st:
        raise ValueError("invalid source update input")
    return out, fis.value


def power_iteration(hp, opts, xs, material, volume, k, iterations):
    """moc_power_iteration restated: the FP32 sweep oracle (oracle_fwd_fp32) and the FP32
    source update, vacuum boundaries. hp: mocatt.HostProblem whose fine_flux holds the
    starting tallies and whose sigT is the materials'; updated in place. Returns the
    eigenvalue after each iteration."""
    src, F_prev = source_update(xs, material, hp.R, hp.I, volume, hp.fine_flux, k)
    hp.source[:] = src
    ks = []
    for _ in range(iterations):
        hp.psi[:] = 0
        hp.fine_flux[:] = 0
        psi, ff = fwd_fp32(hp, opts)
        hp.psi[:] = psi
        hp.fine_flux[:] = ff
        src, F = source_update(xs, material, hp.R, hp.I, volume, hp.fine_flux, k)
        hp.source[:] = src
        k = k * F / F_prev
        F_prev = F
        ks.append(k)
    return ks


# ---- the on-disk track format (include/moc_trackfile.h), restated ------------------------

TRACKFILE_MAGIC = b"MOCTRK01"


def _fnv64_words(payload: bytes) -> int:
    """FNV-1a over little-endian 64-bit words, the last one zero-padded."""
    pad = (-len(payload)) % 8
    words = np.frombuffer(payload + b"\0" * pad, dtype="<u8")
    h = 14695981039346656037
    for w in words.tolist():
        h = ((h ^ w) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def trackfile_bytes(R, I, off, reg, itv, ds, cells=None, compact=False) -> bytes:
    """A track file's bytes from the header's layout; cells overrides region * I +
    interval (to make files with bad indices and a valid checksum). compact: version 2,
    lengths as IEEE half (numpy's float16 conversion, round to nearest even)."""
    import struct

    off = np.ascontiguousarray(off, "<i8")
    if cells is None:
        cells = np.asarray(reg, np.uint64) * I + np.asarray(itv, np.uint64)
    lengths = (np.ascontiguousarray(ds, np.float32).astype("<f2") if compact else
               np.ascontiguousarray(ds, "<f4"))
    payload = off.tobytes() + np.ascontiguousarray(cells, "<u4").tobytes() + lengths.tobytes()
    head = TRACKFILE_MAGIC + struct.pack("<IIqqiiQ", 2 if compact else 1, 48, len(off) - 1,
                                         len(ds), R, I, _fnv64_words(payload))
    return head + payload


def trackfile_parse(data: bytes):
    """(R, I, offsets, region, interval, ds) of a track file's bytes (either version; half
    lengths widened to float32); ValueError if the header, the length or the checksum is
    wrong."""
    import struct

    if len(data) < 48 or data[:8] != TRACKFILE_MAGIC:
        raise ValueError("not a track file")
    version, hbytes, T, S, R, I, cs = struct.unpack("<IIqqiiQ", data[8:48])
    per = {1: 8, 2: 6}.get(version)
    if per is None or hbytes != 48 or len(data) != 48 + 8 * (T + 1) + per * S:
        raise ValueError("bad header or length")
    payload = data[48:]
    if _fnv64_words(payload) != cs:
        raise ValueError("checksum")
    off = np.frombuffer(payload, "<i8", T + 1)
    cells = np.frombuffer(payload, "<u4", S, 8 * (T + 1))
    if version == 1:
        ds = np.frombuffer(payload, "<f4", S, 8 * (T + 1) + 4 * S).copy()
    else:
        ds = np.frombuffer(payload, "<f2", S, 8 * (T + 1) + 4 * S).astype(np.float32)
    return R, I, off.copy(), (cells // I).astype(np.int32), (cells % I).astype(np.uint8), ds
