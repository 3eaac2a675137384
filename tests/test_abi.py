"""The C-ABI library without a GPU: it loads, exports every declared symbol, and its
host-only entry points behave."""
import os
import re
import subprocess

import numpy as np

import mocatt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_functions(header):
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(moc_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def exported(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True,
                         text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_every_declared_symbol_is_exported():
    syms = exported(os.path.join(mocatt.BUILD, "libmocatt.so"))
    decl = (declared_functions("moc_attenuate.h") + declared_functions("moc_tracks.h") +
            declared_functions("moc_transport.h") + declared_functions("moc_trackfile.h"))
    assert decl, "no declarations found"
    missing = [n for n in decl if n not in syms]
    assert not missing, missing
    # the Python binding names every one of them too
    assert set(decl) <= set(mocatt.ABI), set(decl) - set(mocatt.ABI)
    ssyms = exported(os.path.join(mocatt.BUILD, "libmocsynth.so"))
    sdecl = declared_functions("moc_synth.h")
    assert not [n for n in sdecl if n not in ssyms]


def test_library_loads_and_reports_version():
    L = mocatt.lib()
    assert L.moc_abi_version() == 4
    assert L.moc_status_string(mocatt.MOC_ERR_BAD_INDEX).decode().startswith("segment")
    assert L.moc_status_string(999) == b"unknown status"


def test_defaults_are_the_reference_constants():
    o = mocatt.default_opts()
    # src/cpu/kernel.c:99-103 and the table of src/cpu/main.c:33 (0.01 -> N = 353, 10.0)
    assert (o.dz, o.zin, o.weight, o.mu, o.mu2) == tuple(
        float(np.float32(x)) for x in (0.1, 0.3, 0.5, 0.9, 0.3))
    assert (o.table_points, o.table_max) == (353, 10.0)
    assert o.exp_mode == mocatt.MOC_EXP_FULL and o.precision == mocatt.MOC_PREC_FP32


def test_exp_table_builder_matches_oracle():
    import oracle

    for n, mx in ((353, 10.0), (10_000, 10.0), (7, 1.5)):
        a, dx, lk = mocatt.build_exp_table(n, mx)
        b, dx2, lk2 = oracle.table(n, mx)
        np.testing.assert_array_equal(a, b)
        assert (dx, lk) == (dx2, lk2)
    L = mocatt.lib()
    buf = np.zeros(4, np.float32)
    f = mocatt.C.c_float()
    assert L.moc_build_exp_table(1, 10.0, buf.ctypes.data, mocatt.C.byref(f),
                                 mocatt.C.byref(f)) == mocatt.MOC_ERR_INVALID_ARG


def test_null_handle_and_no_device_paths():
    L = mocatt.lib()
    o = mocatt.default_opts()
    p = mocatt.MocProblem()
    assert L.moc_attenuate_fwd(None, mocatt.C.byref(p), mocatt.C.byref(o), None) == \
        mocatt.MOC_ERR_INVALID_ARG
    assert L.moc_attenuate_fwd_host(None, mocatt.C.byref(p), mocatt.C.byref(o)) == \
        mocatt.MOC_ERR_INVALID_ARG
    assert L.moc_destroy(None) == 0
    assert L.moc_create(None, 0) == mocatt.MOC_ERR_INVALID_ARG
    import torch

    if not torch.cuda.is_available():
        h = mocatt.C.c_void_p()
        assert L.moc_create(mocatt.C.byref(h), 0) == mocatt.MOC_ERR_NO_DEVICE
        assert not h.value
