"""The Python mirror of the C ABI (mocatt's ctypes structures, record dtypes and
constants) against the headers themselves: a probe compiled with gcc from include/*.h
prints every structure's size and field offsets and every enumerator and limit, and each
must equal what the Python side assumes. A field added, moved or retyped on one side only
would otherwise pass arguments the library reads at other offsets."""
import ctypes as C
import json
import os
import re
import subprocess

import numpy as np
import pytest

import mocatt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
HEADERS = ["moc_attenuate.h", "moc_synth.h", "moc_tracks.h", "moc_transport.h",
           "moc_trackfile.h"]

# C type name -> the ctypes structure that mirrors it
STRUCTS = {
    "moc_problem_t": mocatt.MocProblem,
    "moc_fwd_opts_t": mocatt.MocFwdOpts,
    "moc_timings_t": mocatt.MocTimings,
    "moc_tune_result_t": mocatt.MocTuneResult,
    "moc_synth_spec_t": mocatt.SynthSpec,
    "moc_geometry_t": mocatt.MocGeometry,
    "moc_quadrature_t": mocatt.MocQuadrature,
    "moc_xs_t": mocatt.MocXS,
    "moc_eigen_opts_t": mocatt.MocEigenOpts,
    "moc_trackfile_info_t": mocatt.MocTrackfileInfo,
    "moc_compact_segments_t": mocatt.MocCompactSegments,
}
# C type name -> the numpy record dtype that mirrors it
RECORDS = {"moc_track_t": mocatt.TRACK_DTYPE}


def header_text():
    text = "\n".join(open(os.path.join(INCLUDE, h)).read() for h in HEADERS)
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def enumerators():
    return sorted(set(re.findall(r"\b(MOC_[A-Z0-9_]+)\s*=", header_text())))


def defines():
    return sorted(n for n in set(re.findall(r"#define\s+(MOC_[A-Z0-9_]+)\s+\S", header_text()))
                  if not n.endswith("_H"))


def c_fields(ctype):
    """Field names of a ctypes structure or numpy record (arrays by their name)."""
    if isinstance(ctype, np.dtype):
        return list(ctype.names)
    return [f[0] for f in ctype._fields_]


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    d = tmp_path_factory.mktemp("layout")
    lines = ["#include <stddef.h>", "#include <stdio.h>"]
    lines += [f'#include "{h}"' for h in HEADERS]
    lines += ["int main(void) {", '  printf("{\\"sizes\\": {");']
    types = list(STRUCTS) + list(RECORDS)
    for i, t in enumerate(types):
        sep = "," if i + 1 < len(types) else ""
        lines.append(f'  printf("\\"{t}\\": %zu{sep}", sizeof({t}));')
    lines.append('  printf("}, \\"offsets\\": {");')
    all_types = [(t, c_fields(STRUCTS[t])) for t in STRUCTS]
    all_types += [(t, c_fields(RECORDS[t])) for t in RECORDS]
    for i, (t, fields) in enumerate(all_types):
        lines.append(f'  printf("\\"{t}\\": [");')
        for j, f in enumerate(fields):
            sep = "," if j + 1 < len(fields) else ""
            lines.append(f'  printf("%zu{sep}", offsetof({t}, {f}));')
        sep = "," if i + 1 < len(all_types) else ""
        lines.append(f'  printf("]{sep}");')
    lines.append('  printf("}, \\"values\\": {");')
    names = enumerators() + defines()
    for i, n in enumerate(names):
        sep = "," if i + 1 < len(names) else ""
        lines.append(f'  printf("\\"{n}\\": %lld{sep}", (long long)({n}));')
    lines += ['  printf("}}\\n");', "  return 0;", "}"]
    src = d / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "probe"
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", INCLUDE, str(src), "-o",
                    str(exe)], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return json.loads(out)


@pytest.mark.parametrize("name", sorted(STRUCTS))
def test_structure_layout(probe, name):
    ct = STRUCTS[name]
    assert C.sizeof(ct) == probe["sizes"][name], name
    got = [getattr(ct, f).offset for f in c_fields(ct)]
    assert got == probe["offsets"][name], name


@pytest.mark.parametrize("name", sorted(RECORDS))
def test_record_layout(probe, name):
    dt = RECORDS[name]
    assert dt.itemsize == probe["sizes"][name]
    got = [dt.fields[f][1] for f in dt.names]
    assert got == probe["offsets"][name]


def test_constants(probe):
    vals = probe["values"]
    # every status code, exp mode, precision and tally enumerator has its Python twin
    needed = [n for n in vals if re.match(r"MOC_(OK|ERR_|EXP_|PREC_|TALLY_)", n)]
    assert len(needed) >= 20
    for n in needed:
        assert getattr(mocatt, n) == vals[n], n
    # and any other constant the Python side names agrees with the header
    for n, v in vals.items():
        if hasattr(mocatt, n):
            assert getattr(mocatt, n) == v, n
    assert vals["MOC_ABI_VERSION"] == mocatt.lib().moc_abi_version()
