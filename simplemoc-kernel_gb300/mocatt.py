"""Python binding of the GB300 segment-attenuation library (ctypes over the C ABI).

This is glue for tests and the bench: the product is libmocatt.so and its C ABI
(include/moc_attenuate.h). Every compute call goes through that ABI; there is no Python
or CPU compute path here, and loading fails loudly if the library was not built.

Workloads are named by what they are: the reference's CPU-sized sweep
(`sweep_1M_g64`, the reference's `-s 1000000 -e 64`), the 50M x 128 sweep
(`sweep_50M_g128`, the reference's default problem size), the wide-tau precision
workload, the lognormal-track batch, and the adjoint workload.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")

# ------------------------------------------------------------------------------------
# C structs (must match include/moc_attenuate.h and include/moc_synth.h)
# ------------------------------------------------------------------------------------
MOC_OK = 0
MOC_ERR_INVALID_ARG = 1
MOC_ERR_MISALIGNED = 2
MOC_ERR_UNSUPPORTED = 3
MOC_ERR_CUDA = 4
MOC_ERR_NO_DEVICE = 5
MOC_ERR_OUT_OF_MEMORY = 6
MOC_ERR_BAD_INDEX = 7
MOC_ERR_DEVICE_TIMEOUT = 8
MOC_ERR_TOO_LARGE = 9
MOC_ERR_BAD_TRACK = 10
MOC_ERR_IO = 11

MOC_EXP_FULL = 0
MOC_EXP_TABLE = 1
MOC_PREC_FP32 = 0
MOC_PREC_BF16 = 1
MOC_PREC_FP16 = 2
MOC_PREC_FP32_STABLE = 3
MOC_TALLY_ATOMIC_FP32 = 0
MOC_TALLY_COMPENSATED = 1
MOC_TALLY_FP64 = 2


class MocProblem(C.Structure):
    _fields_ = [
        ("n_regions", C.c_int32), ("n_intervals", C.c_int32), ("n_groups", C.c_int32),
        ("group_stride", C.c_int32), ("n_tracks", C.c_int32), ("reserved0", C.c_int32),
        ("n_segments", C.c_int64),
        ("track_offsets", C.c_void_p), ("seg_region", C.c_void_p),
        ("seg_interval", C.c_void_p), ("seg_ds", C.c_void_p),
        ("sigT", C.c_void_p), ("source", C.c_void_p), ("fine_flux", C.c_void_p),
        ("psi", C.c_void_p),
    ]


class MocFwdOpts(C.Structure):
    _fields_ = [
        ("exp_mode", C.c_int), ("table_points", C.c_int32), ("table_max", C.c_float),
        ("precision", C.c_int), ("tally", C.c_int),
        ("dz", C.c_float), ("zin", C.c_float), ("weight", C.c_float), ("mu", C.c_float),
        ("mu2", C.c_float), ("checked", C.c_int32), ("vec", C.c_int32),
        ("warps_per_block", C.c_int32), ("profile", C.c_int32),
        ("prefetch", C.c_int32), ("track_chunk", C.c_int32), ("reserved", C.c_int32),
    ]


class MocCompactSegments(C.Structure):
    """moc_compact_segments_t (include/moc_attenuate.h)."""
    _fields_ = [("seg_cell", C.c_void_p), ("seg_ds_half", C.c_void_p)]


class MocTimings(C.Structure):
    _fields_ = [("prep_ms", C.c_float), ("sweep_ms", C.c_float), ("finish_ms", C.c_float),
                ("launches", C.c_int32), ("split_ms", C.c_float)]


class MocTuneResult(C.Structure):
    _fields_ = [("vec", C.c_int32), ("warps_per_block", C.c_int32),
                ("tracks_per_block", C.c_int32), ("best_ms", C.c_float),
                ("n_candidates", C.c_int32), ("candidate_vec", C.c_int32 * 48),
                ("candidate_warps", C.c_int32 * 48), ("candidate_ms", C.c_float * 48)]


class MocGeometry(C.Structure):
    """moc_geometry_t (include/moc_tracks.h)."""
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("n_rings", C.c_int32),
                ("n_axial", C.c_int32), ("n_intervals", C.c_int32), ("reserved", C.c_int32),
                ("pitch", C.c_double), ("fuel_radius", C.c_double), ("height", C.c_double)]


class MocQuadrature(C.Structure):
    """moc_quadrature_t (include/moc_tracks.h)."""
    _fields_ = [("n_azim", C.c_int32), ("n_polar", C.c_int32),
                ("both_directions", C.c_int32), ("reserved", C.c_int32),
                ("spacing", C.c_double), ("axial_spacing", C.c_double)]


class MocXS(C.Structure):
    """moc_xs_t (include/moc_transport.h)."""
    _fields_ = [("n_materials", C.c_int32), ("n_groups", C.c_int32),
                ("group_stride", C.c_int32), ("reserved", C.c_int32),
                ("sigT", C.c_void_p), ("scatter", C.c_void_p), ("nu_fission", C.c_void_p),
                ("chi", C.c_void_p)]


class MocEigenOpts(C.Structure):
    """moc_eigen_opts_t (include/moc_transport.h)."""
    _fields_ = [("max_iterations", C.c_int32), ("reserved", C.c_int32),
                ("tolerance", C.c_double)]


class MocTrackfileInfo(C.Structure):
    """moc_trackfile_info_t (include/moc_trackfile.h)."""
    _fields_ = [("n_tracks", C.c_int64), ("n_segments", C.c_int64), ("n_regions", C.c_int32),
                ("n_intervals", C.c_int32), ("checksum", C.c_uint64), ("version", C.c_int32),
                ("bytes_per_segment", C.c_int32)]


# moc_track_t as a numpy record (112 bytes)
TRACK_DTYPE = np.dtype([(n, np.float64) for n in (
    "x0", "y0", "ux", "uy", "rux", "ruy", "ta", "tb", "za", "cot", "rcot", "rsin")] +
    [(n, np.int32) for n in ("azim", "polar", "reversed", "reserved")])
assert TRACK_DTYPE.itemsize == 112


class SynthSpec(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64), ("n_regions", C.c_int32), ("n_intervals", C.c_int32),
        ("n_groups", C.c_int32), ("group_stride", C.c_int32), ("n_tracks", C.c_int32),
        ("n_segments", C.c_int64), ("track_mode", C.c_int32), ("len_median", C.c_float),
        ("len_sigma", C.c_float), ("len_min", C.c_int32), ("len_max", C.c_int32),
        ("sigT_mode", C.c_int32), ("sigT_lo", C.c_float), ("sigT_hi", C.c_float),
        ("ds_lo", C.c_float), ("ds_hi", C.c_float),
    ]


# Symbols the C ABI exports (include/moc_attenuate.h), with ctypes signatures.
_P = C.c_void_p
ABI = {
    "moc_fwd_opts_default": (None, [C.POINTER(MocFwdOpts)]),
    "moc_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "moc_destroy": (C.c_int, [_P]),
    "moc_attenuate_fwd": (C.c_int, [_P, C.POINTER(MocProblem), C.POINTER(MocFwdOpts), _P]),
    "moc_attenuate_fwd_compact": (C.c_int, [_P, C.POINTER(MocProblem),
                                            C.POINTER(MocCompactSegments),
                                            C.POINTER(MocFwdOpts), _P]),
    "moc_attenuate_fwd_host": (C.c_int, [_P, C.POINTER(MocProblem), C.POINTER(MocFwdOpts)]),
    "moc_synchronize": (C.c_int, [_P, _P]),
    "moc_build_exp_table": (C.c_int, [C.c_int32, C.c_float, _P, C.POINTER(C.c_float),
                                      C.POINTER(C.c_float)]),
    "moc_last_timings": (C.c_int, [_P, C.POINTER(MocTimings)]),
    "moc_attenuate_fwd_noalloc": (C.c_int, [C.POINTER(MocProblem), C.POINTER(MocFwdOpts), _P]),
    "moc_attenuate_adj": (C.c_int, [_P, C.POINTER(MocProblem), C.POINTER(MocFwdOpts), _P, _P,
                                    _P, _P, _P, _P]),
    "moc_attenuate_fwd_batch": (C.c_int, [_P, C.POINTER(MocProblem), C.c_int32,
                                          C.POINTER(MocFwdOpts), _P]),
    "moc_autotune_batch": (C.c_int, [_P, C.POINTER(MocProblem), C.c_int32,
                                     C.POINTER(MocFwdOpts), _P, C.POINTER(MocTuneResult)]),
    "moc_status_string": (C.c_char_p, [C.c_int]),
    "moc_last_error": (C.c_char_p, [_P]),
    "moc_abi_version": (C.c_int32, []),
    "moc_geometry_regions": (C.c_int32, [C.POINTER(MocGeometry)]),
    "moc_geometry_volumes": (C.c_int, [C.POINTER(MocGeometry), _P]),
    "moc_tracks_plan": (C.c_int, [C.POINTER(MocGeometry), C.POINTER(MocQuadrature), _P,
                                  C.c_int64, C.POINTER(C.c_int64)]),
    "moc_tracks_weight": (C.c_double, [C.POINTER(MocQuadrature)]),
    "moc_trace_count": (C.c_int, [_P, C.POINTER(MocGeometry), _P, C.c_int64, _P,
                                  C.POINTER(C.c_int64), _P]),
    "moc_trace_segments": (C.c_int, [_P, C.POINTER(MocGeometry), _P, C.c_int64, _P, _P,
                                     _P, _P, _P]),
    "moc_trackfile_write": (C.c_int, [C.c_char_p, C.c_int64, C.c_int64, C.c_int32, C.c_int32,
                                      _P, _P, _P, _P]),
    "moc_trackfile_write_compact": (C.c_int, [C.c_char_p, C.c_int64, C.c_int64, C.c_int32,
                                              C.c_int32, _P, _P, _P, _P]),
    "moc_trackfile_info": (C.c_int, [C.c_char_p, C.POINTER(MocTrackfileInfo)]),
    "moc_trackfile_read": (C.c_int, [C.c_char_p, _P, _P, _P, _P]),
    "moc_region_sigT": (C.c_int, [_P, C.POINTER(MocXS), _P, C.c_int32, _P, _P]),
    "moc_source_update": (C.c_int, [_P, C.POINTER(MocXS), _P, C.c_int32, C.c_int32, _P, _P,
                                    C.c_double, _P, _P, _P]),
    "moc_power_iteration": (C.c_int, [_P, C.POINTER(MocProblem), C.POINTER(MocFwdOpts),
                                      C.POINTER(MocXS), _P, _P, C.POINTER(MocEigenOpts),
                                      C.POINTER(C.c_double), C.POINTER(C.c_int32), _P]),
}
SYNTH_ABI = {
    "moc_synth_spec_init": (None, [C.POINTER(SynthSpec), C.c_uint64, C.c_int32, C.c_int32,
                                   C.c_int32, C.c_int32, C.c_int64]),
    "moc_synth_track_offsets": (C.c_int64, [C.POINTER(SynthSpec), _P]),
    "moc_synth_fill": (C.c_int, [C.POINTER(SynthSpec), _P, _P, _P, _P, _P, _P, _P]),
    "moc_synth_uniform": (None, [C.c_uint64, C.c_uint64, C.c_int64, C.c_float, C.c_float, _P]),
    "moc_synth_normal": (None, [C.c_uint64, C.c_uint64, C.c_int64, _P]),
    "moc_synth_randint": (None, [C.c_uint64, C.c_uint64, C.c_int64, C.c_int64, _P]),
}

_lib = None
_synth = None


def _bind(path: str, table: dict):
    if not os.path.exists(path):
        raise RuntimeError(f"{os.path.basename(path)} is not built ({path}); run "
                           "__graft_entry__.build() first")
    lib = C.CDLL(path)
    for name, (res, args) in table.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def lib():
    """The loaded libmocatt.so (raises if it is missing)."""
    global _lib
    if _lib is None:
        _lib = _bind(os.path.join(BUILD, "libmocatt.so"), ABI)
    return _lib


def synth_lib():
    global _synth
    if _synth is None:
        _synth = _bind(os.path.join(BUILD, "libmocsynth.so"), SYNTH_ABI)
    return _synth


class MocError(RuntimeError):
    def __init__(self, status: int, detail: str = ""):
        self.status = status
        msg = lib().moc_status_string(status).decode()
        super().__init__(f"moc status {status} ({msg}){': ' + detail if detail else ''}")


def default_opts(**kw) -> MocFwdOpts:
    o = MocFwdOpts()
    lib().moc_fwd_opts_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def build_exp_table(n_points: int, max_val: float):
    vals = np.zeros(2 * n_points, np.float32)
    dx, lk = C.c_float(), C.c_float()
    st = lib().moc_build_exp_table(n_points, max_val, vals.ctypes.data, C.byref(dx), C.byref(lk))
    if st:
        raise MocError(st)
    return vals, dx.value, lk.value


# ------------------------------------------------------------------------------------
# Workloads
# ------------------------------------------------------------------------------------
@dataclasses.dataclass(frozen=True)
class Workload:
    name: str
    seed: int
    regions: int
    intervals: int
    groups: int
    tracks: int
    segments: int = 0            # uniform track assignment (0 with lognormal lengths)
    lognormal: tuple | None = None   # (median, sigma, min, max)
    logsigt: tuple | None = None     # sigT ~ logU(lo, hi)
    ds: tuple = (0.01, 1.0)

    def with_(self, **kw) -> "Workload":
        return dataclasses.replace(self, **kw)

    def spec(self) -> SynthSpec:
        s = SynthSpec()
        synth_lib().moc_synth_spec_init(C.byref(s), self.seed, self.regions, self.intervals,
                                        self.groups, self.tracks, self.segments)
        if self.lognormal:
            s.track_mode = 1
            s.len_median, s.len_sigma, s.len_min, s.len_max = self.lognormal
        if self.logsigt:
            s.sigT_mode = 1
            s.sigT_lo, s.sigT_hi = self.logsigt
        s.ds_lo, s.ds_hi = self.ds
        return s

    def cpu_bench_args(self) -> list[str]:
        a = ["--seed", str(self.seed), "--regions", str(self.regions), "--intervals",
             str(self.intervals), "--groups", str(self.groups), "--tracks", str(self.tracks),
             "--segments", str(self.segments), "--ds", str(self.ds[0]), str(self.ds[1])]
        if self.lognormal:
            a += ["--lognormal"] + [str(x) for x in self.lognormal]
        if self.logsigt:
            a += ["--logsigt"] + [str(x) for x in self.logsigt]
        return a


# lognormal track lengths: median 200, sigma = sqrt(2 ln 1.5) so the mean is 300
LOGN_BATCH = (200.0, 0.9005, 1, 5000)
# 5,000 tracks, about 2,000,000 segments: same sigma, median 400 / exp(sigma^2 / 2)
LOGN_ADJ = (267.0, 0.9005, 1, 5000)

WORKLOADS = {
    # the reference's CPU-sized run (-s 1000000 -e 64), 1,000 tracks, 2,000 regions
    "sweep_1M_g64": Workload("sweep_1M_g64", 1, 2000, 5, 64, 1000, 1_000_000),
    # the reference's default size (-s 50000000 -e 128), 100,000 tracks, 10,000 regions
    "sweep_50M_g128": Workload("sweep_50M_g128", 2, 10000, 5, 128, 100_000, 50_000_000),
    # same shapes, tau spread over ~[1e-6, 40] for the precision form
    "widetau_50M_g128": Workload("widetau_50M_g128", 2, 10000, 5, 128, 100_000, 50_000_000,
                                 logsigt=(1e-3, 20.0), ds=(1e-3, 2.0)),
    # three problems of 20,000 lognormal tracks (about 6M segments each)
    "batch_20k_g16": Workload("batch_20k_g16", 3, 2000, 5, 16, 20_000, 0, LOGN_BATCH),
    "batch_20k_g70": Workload("batch_20k_g70", 3, 2000, 5, 70, 20_000, 0, LOGN_BATCH),
    "batch_20k_g128": Workload("batch_20k_g128", 3, 2000, 5, 128, 20_000, 0, LOGN_BATCH),
    # adjoint: 5,000 lognormal tracks, about 2M segments, G=64
    "adjoint_2M_g64": Workload("adjoint_2M_g64", 4, 2000, 5, 64, 5000, 0, LOGN_ADJ),
}


@dataclasses.dataclass
class HostProblem:
    """A problem's arrays in host memory (numpy), in the C ABI's layout."""
    R: int
    I: int
    G: int
    Gs: int
    T: int
    S: int
    track_offsets: np.ndarray   # int64 [T+1]
    seg_region: np.ndarray      # int32 [S]
    seg_interval: np.ndarray    # uint8 [S]
    seg_ds: np.ndarray          # float32 [S]
    sigT: np.ndarray            # float32 [R, Gs]
    source: np.ndarray          # float32 [R*I, Gs]
    fine_flux: np.ndarray       # float32 [R*I, Gs]
    psi: np.ndarray             # float32 [T, Gs]

    def copy(self) -> "HostProblem":
        return dataclasses.replace(self, **{f.name: getattr(self, f.name).copy()
                                            for f in dataclasses.fields(self)
                                            if isinstance(getattr(self, f.name), np.ndarray)})

    def c_struct(self) -> MocProblem:
        """C struct pointing at these (host) arrays; keep self alive while it is used."""
        for name in ("track_offsets", "seg_region", "seg_interval", "seg_ds", "sigT",
                     "source", "fine_flux", "psi"):
            a = getattr(self, name)
            assert a.flags["C_CONTIGUOUS"], name
        return MocProblem(self.R, self.I, self.G, self.Gs, self.T, 0, self.S,
                          self.track_offsets.ctypes.data, self.seg_region.ctypes.data,
                          self.seg_interval.ctypes.data, self.seg_ds.ctypes.data,
                          self.sigT.ctypes.data, self.source.ctypes.data,
                          self.fine_flux.ctypes.data, self.psi.ctypes.data)

    def subset_tracks(self, tracks) -> "HostProblem":
        """A problem with only the given tracks (same tables, fresh zero tallies). psi of a
        track depends only on its own segments, so this reproduces those tracks exactly."""
        tracks = np.asarray(tracks, np.int64)
        lens = self.track_offsets[tracks + 1] - self.track_offsets[tracks]
        off = np.zeros(len(tracks) + 1, np.int64)
        off[1:] = np.cumsum(lens)
        idx = np.concatenate([np.arange(self.track_offsets[t], self.track_offsets[t + 1])
                              for t in tracks]) if len(tracks) else np.zeros(0, np.int64)
        return HostProblem(self.R, self.I, self.G, self.Gs, len(tracks), int(off[-1]), off,
                           self.seg_region[idx].copy(), self.seg_interval[idx].copy(),
                           self.seg_ds[idx].copy(), self.sigT, self.source,
                           np.zeros_like(self.fine_flux), self.psi[tracks].copy())

    def with_lengths(self, lens) -> "HostProblem":
        """The first sum(lens) segments regrouped into tracks of the given lengths (same
        tables, zero tallies); track t takes psi row t mod T."""
        lens = np.asarray(lens, np.int64)
        off = np.zeros(len(lens) + 1, np.int64)
        off[1:] = np.cumsum(lens)
        S = int(off[-1])
        assert S <= self.S, "not enough segments"
        rows = np.arange(len(lens)) % max(self.T, 1)
        return HostProblem(self.R, self.I, self.G, self.Gs, len(lens), S, off,
                           self.seg_region[:S].copy(), self.seg_interval[:S].copy(),
                           self.seg_ds[:S].copy(), self.sigT, self.source,
                           np.zeros_like(self.fine_flux), self.psi[rows].copy())


def _aligned_empty(shape, dtype, align=64):
    """numpy array with 64-byte aligned data (the ABI wants 16-byte aligned rows)."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    buf = np.empty(n + align, np.uint8)
    off = (-buf.ctypes.data) % align
    return buf[off:off + n].view(dtype).reshape(shape)


def generate(w: Workload, group_stride: int | None = None) -> HostProblem:
    """Seeded inputs of a workload (moc_synth.h), fine_flux zeroed."""
    sl = synth_lib()
    spec = w.spec()
    if group_stride is not None:
        spec.group_stride = group_stride
    T, Gs, R, I = w.tracks, spec.group_stride, w.regions, w.intervals
    off = np.zeros(T + 1, np.int64)
    S = sl.moc_synth_track_offsets(C.byref(spec), off.ctypes.data)
    if S < 0:
        raise ValueError(f"invalid workload {w}")
    psi = _aligned_empty((T, Gs), np.float32)
    sig = _aligned_empty((R, Gs), np.float32)
    src = _aligned_empty((R * I, Gs), np.float32)
    reg = np.empty(S, np.int32)
    itv = np.empty(S, np.uint8)
    ds = np.empty(S, np.float32)
    if sl.moc_synth_fill(C.byref(spec), off.ctypes.data, psi.ctypes.data, sig.ctypes.data,
                         src.ctypes.data, reg.ctypes.data, itv.ctypes.data, ds.ctypes.data):
        raise ValueError("moc_synth_fill failed")
    ff = _aligned_empty((R * I, Gs), np.float32)
    ff[:] = 0
    return HostProblem(R, I, w.groups, Gs, T, int(S), off, reg, itv, ds, sig, src, ff, psi)


def synth_normal(seed: int, tag: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float32)
    synth_lib().moc_synth_normal(seed, tag, n, out.ctypes.data)
    return out


def synth_uniform(seed: int, tag: int, n: int, lo: float, hi: float) -> np.ndarray:
    out = np.empty(n, np.float32)
    synth_lib().moc_synth_uniform(seed, tag, n, lo, hi, out.ctypes.data)
    return out


def synth_randint(seed: int, tag: int, n: int, bound: int) -> np.ndarray:
    out = np.empty(n, np.int64)
    synth_lib().moc_synth_randint(seed, tag, n, bound, out.ctypes.data)
    return out


# ------------------------------------------------------------------------------------
# Device side (torch is only the allocator and stream provider here)
# ------------------------------------------------------------------------------------
# ---- track generation (include/moc_tracks.h) -------------------------------------------

def geometry(nx=17, ny=17, n_rings=3, n_axial=40, n_intervals=5, pitch=1.26,
             fuel_radius=0.54, height=200.0) -> MocGeometry:
    """A pin lattice (defaults: a 17 x 17 assembly, 1.26 cm pitch, 200 cm tall)."""
    return MocGeometry(nx, ny, n_rings, n_axial, n_intervals, 0, pitch, fuel_radius, height)


def quadrature(n_azim=8, n_polar=4, spacing=0.1, axial_spacing=1.0,
               both_directions=0) -> MocQuadrature:
    return MocQuadrature(n_azim, n_polar, both_directions, 0, spacing, axial_spacing)


def geometry_regions(g: MocGeometry) -> int:
    return int(lib().moc_geometry_regions(C.byref(g)))


def geometry_volumes(g: MocGeometry) -> np.ndarray:
    """Volume of every (region, interval) cell, [n_regions * n_intervals] float64."""
    v = np.empty(geometry_regions(g) * g.n_intervals, np.float64)
    st = lib().moc_geometry_volumes(C.byref(g), v.ctypes.data)
    if st:
        raise MocError(st)
    return v


def tracks_plan(g: MocGeometry, q: MocQuadrature) -> np.ndarray:
    """moc_tracks_plan: the tracks as a TRACK_DTYPE array (host)."""
    n = C.c_int64()
    L = lib()
    st = L.moc_tracks_plan(C.byref(g), C.byref(q), None, 0, C.byref(n))
    if st:
        raise MocError(st)
    out = np.zeros(n.value, TRACK_DTYPE)
    st = L.moc_tracks_plan(C.byref(g), C.byref(q), out.ctypes.data if n.value else None,
                           n.value, C.byref(n))
    if st:
        raise MocError(st)
    return out


def tracks_weight(q: MocQuadrature) -> float:
    return float(lib().moc_tracks_weight(C.byref(q)))


# ---- cross sections (include/moc_transport.h) ---------------------------------------------

@dataclasses.dataclass
class HostXS:
    """Multigroup cross sections of M materials in moc_xs_t's layout (host, float32)."""
    M: int
    G: int
    Gs: int
    sigT: np.ndarray        # [M, Gs]
    scatter: np.ndarray     # [M, G, Gs]: from group g' (axis 1) into group g (axis 2)
    nu_fission: np.ndarray  # [M, Gs]
    chi: np.ndarray         # [M, Gs]


def synth_xs(M: int, G: int, seed: int = 7, fissile=None) -> HostXS:
    """Seeded synthetic cross sections: material 0 a scatterer (scattering ratio ~0.9,
    no fission), the others fissile (~0.5, nu_fission ~1.6 x absorption); total cross
    sections rising with the group index (fast to thermal), scattering mostly into the
    same and lower-energy groups with some up-scattering in the last quarter, and chi
    over the first third of the groups, normalised."""
    rng = np.random.default_rng(seed)
    Gs = (G + 3) & ~3
    fissile = set(range(1, M)) if fissile is None else set(fissile)
    sig = _aligned_empty((M, Gs), np.float32)
    sc = _aligned_empty((M, G, Gs), np.float32)
    nuf = _aligned_empty((M, Gs), np.float32)
    chi = _aligned_empty((M, Gs), np.float32)
    for a in (sig, sc, nuf, chi):
        a[:] = 0
    gg = np.arange(G)
    for m in range(M):
        st = 0.25 + 1.2 * gg / max(G - 1, 1) + 0.05 * rng.random(G)
        ratio = 0.9 if m not in fissile else 0.5
        w = rng.random((G, G)) + 0.05
        down = gg[None, :] >= gg[:, None]                 # g >= g'
        up = (gg[:, None] >= 3 * G // 4) & (gg[None, :] >= 3 * G // 4)
        w = np.where(down | up, w, 0.0)
        w /= w.sum(axis=1, keepdims=True)
        sig[m, :G] = st
        sc[m, :, :G] = (ratio * st)[:, None] * w
        if m in fissile:
            nuf[m, :G] = 1.6 * (1.0 - ratio) * st
            c = np.where(gg < max(1, G // 3), rng.random(G) + 0.1, 0.0)
            chi[m, :G] = c / c.sum()
    return HostXS(M, G, Gs, sig, sc, nuf, chi)


def geometry_materials(g) -> np.ndarray:
    """Material of every region of a traced geometry (include/moc_tracks.h numbering):
    moderator 0, fuel ring k material 1 + k."""
    R = geometry_regions(g)
    ring = (np.arange(R) // g.n_axial) % (g.n_rings + 1)
    return np.where(ring == g.n_rings, 0, 1 + ring).astype(np.int32)


def write_trackfile(path: str, R: int, I: int, off, reg, itv, ds, compact: bool = False) -> None:
    """moc_trackfile_write (or, compact, moc_trackfile_write_compact: half lengths) of CSR
    descriptors (host arrays)."""
    off = np.ascontiguousarray(off, np.int64)
    reg = np.ascontiguousarray(reg, np.int32)
    itv = np.ascontiguousarray(itv, np.uint8)
    ds = np.ascontiguousarray(ds, np.float32)
    fn = lib().moc_trackfile_write_compact if compact else lib().moc_trackfile_write
    st = fn(os.fsencode(path), len(off) - 1, len(reg), R, I, off.ctypes.data, reg.ctypes.data,
            itv.ctypes.data, ds.ctypes.data)
    if st:
        raise MocError(st)


def read_trackfile(path: str):
    """moc_trackfile_info + moc_trackfile_read: (R, I, offsets, region, interval, ds)."""
    info = MocTrackfileInfo()
    L = lib()
    st = L.moc_trackfile_info(os.fsencode(path), C.byref(info))
    if st:
        raise MocError(st)
    T, S = info.n_tracks, info.n_segments
    off = np.empty(T + 1, np.int64)
    reg = np.empty(max(S, 1), np.int32)
    itv = np.empty(max(S, 1), np.uint8)
    ds = np.empty(max(S, 1), np.float32)
    st = L.moc_trackfile_read(os.fsencode(path), off.ctypes.data, reg.ctypes.data,
                              itv.ctypes.data, ds.ctypes.data)
    if st:
        raise MocError(st)
    return info.n_regions, info.n_intervals, off, reg[:S], itv[:S], ds[:S]


def problem_from_tracks(g, off, reg, itv, ds, xs: HostXS):
    """A host problem on traced descriptors (int64 offsets, int32 regions, uint8
    intervals, float32 lengths) of geometry g with the materials' sigT, a zero source and
    psi, and fine_flux = the cell volumes in every group (the starting tallies of a flat
    flux phi = 1). Returns (problem, material [R] int32, volume [R*I] float64)."""
    R, I = geometry_regions(g), g.n_intervals
    T = len(off) - 1
    mat = geometry_materials(g)
    vol = geometry_volumes(g)
    sig = _aligned_empty((R, xs.Gs), np.float32)
    sig[:] = xs.sigT[mat]
    src = _aligned_empty((R * I, xs.Gs), np.float32)
    src[:] = 0
    ff = _aligned_empty((R * I, xs.Gs), np.float32)
    ff[:] = 0
    ff[:, :xs.G] = vol[:, None].astype(np.float32)
    psi = _aligned_empty((T, xs.Gs), np.float32)
    psi[:] = 0
    hp = HostProblem(R, I, xs.G, xs.Gs, T, int(off[-1]), np.ascontiguousarray(off, np.int64),
                     np.ascontiguousarray(reg, np.int32), np.ascontiguousarray(itv, np.uint8),
                     np.ascontiguousarray(ds, np.float32), sig, src, ff, psi)
    return hp, mat, vol


class DeviceXS:
    """HostXS on the GPU and its moc_xs_t."""

    def __init__(self, xs: HostXS, device="cuda:0"):
        import torch
        self.M, self.G, self.Gs = xs.M, xs.G, xs.Gs
        for n in ("sigT", "scatter", "nu_fission", "chi"):
            setattr(self, n, torch.from_numpy(np.ascontiguousarray(getattr(xs, n))).to(device))

    def c_struct(self) -> MocXS:
        return MocXS(self.M, self.G, self.Gs, 0, self.sigT.data_ptr(), self.scatter.data_ptr(),
                     self.nu_fission.data_ptr(), self.chi.data_ptr())


class DeviceProblem:
    """A problem resident on the GPU (torch tensors), and its C struct."""

    NAMES = ("track_offsets", "seg_region", "seg_interval", "seg_ds", "sigT", "source",
             "fine_flux", "psi")

    def __init__(self, hp: HostProblem, device="cuda:0"):
        import torch
        self.R, self.I, self.G, self.Gs, self.T, self.S = hp.R, hp.I, hp.G, hp.Gs, hp.T, hp.S
        for n in self.NAMES:
            a = getattr(hp, n)
            t = torch.from_numpy(np.ascontiguousarray(a)).to(device) if a.size else \
                torch.empty(max(1, a.size), dtype=torch.from_numpy(a).dtype, device=device)
            setattr(self, n, t)

    @classmethod
    def from_tensors(cls, R, I, G, Gs, T, S, **tensors) -> "DeviceProblem":
        """A device problem over existing device tensors (e.g. traced descriptors), one
        per name of NAMES."""
        dp = cls.__new__(cls)
        dp.R, dp.I, dp.G, dp.Gs, dp.T, dp.S = R, I, G, Gs, T, S
        for n in cls.NAMES:
            setattr(dp, n, tensors[n])
        return dp

    def c_struct(self) -> MocProblem:
        return MocProblem(self.R, self.I, self.G, self.Gs, self.T, 0, self.S,
                          *[getattr(self, n).data_ptr() for n in self.NAMES])

    def to_host(self, name):
        return getattr(self, name).cpu().numpy()


class Handle:
    """Owns a moc_handle_t."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        st = lib().moc_create(C.byref(self._h), device)
        if st:
            raise MocError(st)

    @property
    def ptr(self):
        return self._h

    def check(self, st: int):
        if st:
            raise MocError(st, lib().moc_last_error(self._h).decode())

    def fwd(self, dp: DeviceProblem, opts: MocFwdOpts | None = None, stream=None):
        """moc_attenuate_fwd on the device problem, on `stream` (a torch stream or None
        for torch's current stream)."""
        import torch
        opts = opts or default_opts()
        s = stream if stream is not None else torch.cuda.current_stream()
        prob = dp.c_struct()
        self.check(lib().moc_attenuate_fwd(self._h, C.byref(prob), C.byref(opts),
                                           C.c_void_p(s.cuda_stream)))

    def fwd_compact(self, dp: DeviceProblem, cell, ds_half, opts: MocFwdOpts | None = None,
                    stream=None):
        """moc_attenuate_fwd_compact: dp's tables, offsets, psi and fine_flux with the
        segments given as device tensors of 32-bit cells (region * I + interval) and half
        lengths (int16/uint16 bit patterns or float16)."""
        import torch
        opts = opts or default_opts()
        s = stream if stream is not None else torch.cuda.current_stream()
        prob = dp.c_struct()
        segs = MocCompactSegments(cell.data_ptr(), ds_half.data_ptr())
        self.check(lib().moc_attenuate_fwd_compact(self._h, C.byref(prob), C.byref(segs),
                                                   C.byref(opts), C.c_void_p(s.cuda_stream)))

    def adj(self, dp: DeviceProblem, w, v, opts: MocFwdOpts | None = None, stream=None):
        """moc_attenuate_adj: gradients of L = sum w . fine_flux_out + sum v . psi_out with
        respect to sigT, source and the incoming psi (dp.psi, which is not modified).
        w, v: device float32 tensors shaped like fine_flux and psi. Returns torch tensors
        (d_sigT, d_source, d_psi_in)."""
        import torch
        opts = opts or default_opts()
        s = stream if stream is not None else torch.cuda.current_stream()
        d_sig = torch.zeros_like(dp.sigT)
        d_src = torch.zeros_like(dp.source)
        d_psi = torch.zeros_like(dp.psi)
        prob = dp.c_struct()
        self.check(lib().moc_attenuate_adj(self._h, C.byref(prob), C.byref(opts),
                                           w.data_ptr(), v.data_ptr(), d_sig.data_ptr(),
                                           d_src.data_ptr(), d_psi.data_ptr(),
                                           C.c_void_p(s.cuda_stream)))
        return d_sig, d_src, d_psi

    def trace(self, g: MocGeometry, d_tracks, n_tracks: int, stream=None):
        """moc_trace_count + moc_trace_segments: the CSR descriptors of the tracks
        (d_tracks: a device tensor holding n_tracks moc_track_t records). Returns device
        tensors (track_offsets int64 [T+1], seg_region int32, seg_interval uint8,
        seg_ds float32)."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        dev = d_tracks.device
        off = torch.empty(n_tracks + 1, dtype=torch.int64, device=dev)
        S = C.c_int64()
        L = lib()
        self.check(L.moc_trace_count(self._h, C.byref(g), d_tracks.data_ptr(), n_tracks,
                                     off.data_ptr(), C.byref(S), C.c_void_p(s.cuda_stream)))
        n = S.value
        reg = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        itv = torch.empty(max(n, 1), dtype=torch.uint8, device=dev)
        ds = torch.empty(max(n, 1), dtype=torch.float32, device=dev)
        self.check(L.moc_trace_segments(self._h, C.byref(g), d_tracks.data_ptr(), n_tracks,
                                        off.data_ptr(), reg.data_ptr(), itv.data_ptr(),
                                        ds.data_ptr(), C.c_void_p(s.cuda_stream)))
        return off, reg[:n], itv[:n], ds[:n]

    def region_sigT(self, xs: DeviceXS, material, stream=None):
        """moc_region_sigT: the regions' sigT [R, Gs] from their materials (device)."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        R = material.numel()
        out = torch.empty((R, xs.Gs), dtype=torch.float32, device=material.device)
        xc = xs.c_struct()
        self.check(lib().moc_region_sigT(self._h, C.byref(xc), material.data_ptr(), R,
                                         out.data_ptr(), C.c_void_p(s.cuda_stream)))
        return out

    def source_update(self, xs: DeviceXS, material, I: int, volume, tally, k: float,
                      stream=None):
        """moc_source_update: returns (source [R*I, Gs] device tensor, fission total)."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        src = torch.zeros_like(tally)
        fis = torch.zeros(1, dtype=torch.float64, device=tally.device)
        xc = xs.c_struct()
        self.check(lib().moc_source_update(self._h, C.byref(xc), material.data_ptr(),
                                           material.numel(), I, volume.data_ptr(),
                                           tally.data_ptr(), float(k), src.data_ptr(),
                                           fis.data_ptr(), C.c_void_p(s.cuda_stream)))
        return src, fis

    def power_iteration(self, dp: "DeviceProblem", opts: MocFwdOpts, xs: DeviceXS, material,
                        volume, k: float, max_iterations: int, tolerance: float = 0.0,
                        stream=None):
        """moc_power_iteration on dp (its fine_flux the starting tallies). Returns
        (k, iterations)."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        kk = C.c_double(k)
        it = C.c_int32()
        eo = MocEigenOpts(max_iterations, 0, tolerance)
        prob = dp.c_struct()
        xc = xs.c_struct()
        self.check(lib().moc_power_iteration(self._h, C.byref(prob), C.byref(opts), C.byref(xc),
                                             material.data_ptr(), volume.data_ptr(),
                                             C.byref(eo), C.byref(kk), C.byref(it),
                                             C.c_void_p(s.cuda_stream)))
        return kk.value, it.value

    def fwd_host(self, hp: HostProblem, opts: MocFwdOpts | None = None):
        opts = opts or default_opts()
        prob = hp.c_struct()
        self.check(lib().moc_attenuate_fwd_host(self._h, C.byref(prob), C.byref(opts)))

    def timings(self) -> MocTimings:
        t = MocTimings()
        self.check(lib().moc_last_timings(self._h, C.byref(t)))
        return t

    def synchronize(self, stream=None) -> int:
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        return lib().moc_synchronize(self._h, C.c_void_p(s.cuda_stream))

    def close(self):
        if self._h:
            lib().moc_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
