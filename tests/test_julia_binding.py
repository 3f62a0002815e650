"""The Julia backend (julia/GaugefieldsGB300.jl) against the C header it binds.

No Julia toolchain exists where these tests run, so the Julia file is checked
as text: its mirror of gf_md_params has the header's field order and C types,
its constants equal the header's #defines, and every symbol it ccalls is
declared in include/gaugefields_gb300.h and exported by libgfgb300.so (the
ccall argument lists follow the declarations).
"""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JL = os.path.join(ROOT, "julia", "GaugefieldsGB300.jl")
HEADER = os.path.join(ROOT, "include", "gaugefields_gb300.h")

C_TO_JULIA = {"double": "Cdouble", "int": "Cint"}


def _julia_struct(src, name):
    m = re.search(r"struct %s\s*\n(.*?)\nend" % name, src, re.S)
    assert m, name
    fields = []
    for line in m.group(1).splitlines():
        line = line.split("#")[0].strip()
        if line:
            f, t = line.split("::")
            fields.append((f.strip(), t.strip()))
    return fields


def _c_struct(src, name):
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, re.S)
    assert m, name
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        mm = re.match(r"(\w+)\s+(\w+)(\[(\w+)\])?$", decl)
        assert mm, decl
        ctype, fname, arr = mm.group(1), mm.group(2), mm.group(4)
        jt = C_TO_JULIA[ctype]
        if arr:
            n = re.search(r"#define %s (\d+)" % arr, src).group(1)
            jt = "NTuple{%s,%s}" % (n, jt)
        fields.append((fname, jt))
    return fields


def test_md_params_mirror_matches_the_header():
    jl = open(JL).read()
    h = open(HEADER).read()
    assert _julia_struct(jl, "GB300MDParams") == _c_struct(h, "gf_md_params")


def test_constants_match_the_header():
    jl = open(JL).read()
    h = open(HEADER).read()
    defines = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define (GF_\w+) \(?(-?\d+)\)?", h)}
    for m in re.finditer(r"const ((?:GF_\w+(?:, )?)+) = ([-\d, ]+)\n", jl):
        names = [x.strip() for x in m.group(1).split(",")]
        vals = [int(x) for x in m.group(2).split(",")]
        assert len(names) == len(vals)
        for n, v in zip(names, vals):
            assert defines[n] == v, n


def _ccalls(jl):
    return sorted(set(re.findall(r"ccall\(\(:(\w+), libgf\)", jl)))


def test_every_ccall_is_declared_in_the_header():
    jl = open(JL).read()
    h = open(HEADER).read()
    calls = _ccalls(jl)
    assert "gf_md_trajectory" in calls and "gf_stout_backward" in calls and "gf_stout_param_derivatives" in calls
    for name in calls:
        assert re.search(r"\b%s\(" % name, h), name


def test_ccall_argument_counts_match_the_declarations():
    jl = open(JL).read()
    h = open(HEADER).read()
    for m in re.finditer(r"ccall\(\(:(\w+), libgf\), \w+, \((.*?)\),", jl, re.S):
        name, types = m.group(1), m.group(2)
        n_jl = len([t for t in types.split(",") if t.strip()])
        d = re.search(r"^(?:const )?\w+\*? ?\*?%s\(([^)]*)\);" % name, h, re.M)
        n_c = len([a for a in d.group(1).split(",") if a.strip() and a.strip() != "void"])
        assert n_jl == n_c, (name, n_jl, n_c)


def test_every_ccall_is_exported_by_the_library(pkg):
    lib = os.path.join(ROOT, "gaugefields.jl_gb300", "libgfgb300.so")
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("nm not available")
    exported = set(line.split()[-1] for line in out.stdout.splitlines() if line.strip())
    for name in _ccalls(open(JL).read()):
        assert name in exported, name


def test_md_methods_are_typed_on_the_driver():
    """The MD steps are specialised on MDDriver (as the reference's methods at
    src/molecular_dynamics.jl:494-730 are), so calls are not ambiguous, and
    md_force! has one method."""
    jl = open(JL).read()
    for fn in ("md_hamiltonian", "update_momenta!", "update_gaugefields!", "md_trajectory!"):
        for m in re.finditer(r"function %s\((.*?)\)" % re.escape(fn), jl, re.S):
            assert "driver::Gaugefields.MDDriver" in m.group(1), fn
    assert len(re.findall(r"function md_force!\(", jl)) == 1
    # the backend is a positional selector: the reference's keyword method is not redefined
    assert re.search(r"function gauge_configuration\(lattice::NTuple\{4,<:Integer\}, backend::GB300Backend;", jl)


def test_configuration_accessors_are_defined():
    """measure_plaquette(U) and the accessors of src/API.jl:262-295 reach the
    backend through size, gauge_backend and gauge_halo_width of a direction."""
    jl = open(JL).read()
    assert re.search(r"Base\.size\(u::Gaugefields_4D_GB300\) = \(u\.NC, u\.NC, u\.NX, u\.NY, u\.NZ, u\.NT\)", jl)
    assert "Gaugefields.gauge_backend(u::Gaugefields_4D_GB300)" in jl
    assert "Gaugefields.gauge_halo_width(::Gaugefields_4D_GB300)" in jl
    assert re.search(r"function copy_configuration!\(destination::GB300Config, source::GB300Config\)", jl)


def test_configuration_files_go_through_the_reference_writers():
    """save_configuration / load_configuration! of a device configuration run
    the reference's own readers and writers (portable JLD2, ILDG, Bridge++) on
    a LegacyBackend host copy (src/API.jl:711-826)."""
    jl = open(JL).read()
    assert re.search(r"save_configuration\(filename, U::GB300Config; kwargs\.\.\.\) =\s*save_configuration\(filename, "
                     r"host_configuration\(U\); kwargs\.\.\.\)", jl)
    assert re.search(r"function load_configuration!\(U::GB300Config, filename; format::Symbol=:jld2\)", jl)
    assert "backend=Gaugefields.LegacyBackend()" in jl

