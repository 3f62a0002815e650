"""CPU-side checks of the C-ABI library: it builds for sm_103a, loads, exports
every entry point declared in include/gaugefields_gb300.h, and rejects bad
arguments with the reference's ArgumentError behaviour before any GPU work."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gaugefields_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(gf_\w+)\s*\(", text, re.M)))


def test_header_declares_the_abi():
    syms = declared_symbols()
    for s in ("gf_ctx_create", "gf_plaquette", "gf_md_trajectory", "gf_stout_backward", "gf_flow", "gf_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol(pkg):
    lib = ctypes.CDLL(os.path.join(ROOT, "gaugefields.jl_gb300", "libgfgb300.so"))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol(pkg):
    from gaugefields_gb300 import _lib
    assert sorted(declared_symbols()) == sorted(_lib.exported_symbols())


def test_library_is_built_for_sm_103a(pkg):
    from gaugefields_gb300 import _nvcc_build
    assert "arch=compute_103a,code=sm_103a" in " ".join(_nvcc_build.NVCC_FLAGS)
    assert _nvcc_build.up_to_date()


def test_ctx_create_rejects_bad_extents_before_touching_the_gpu(pkg):
    from gaugefields_gb300 import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    for L in ((3, 4, 4, 4), (4, 4, 4, 0), (4, 5, 4, 4)):
        arr = (ctypes.c_int * 4)(*L)
        assert lib.gf_ctx_create(arr, 0, ctypes.byref(h)) == _lib.GF_EINVAL
        assert b"even" in lib.gf_last_error(None)
    assert lib.gf_ctx_create(None, 0, ctypes.byref(h)) == _lib.GF_EINVAL


def test_null_arguments_are_rejected(pkg):
    from gaugefields_gb300 import _lib
    lib = _lib.load()
    out = ctypes.c_double()
    assert lib.gf_plaquette(None, None, ctypes.byref(out)) == _lib.GF_EINVAL
    assert lib.gf_md_trajectory(None, None, None, None, None) == _lib.GF_EINVAL
    assert lib.gf_flow(None, None, ctypes.c_double(0.01), 1) == _lib.GF_EINVAL
    prm = _lib.MDParams()
    assert lib.gf_md_mom_update(None, None, None, ctypes.c_double(0.1), ctypes.byref(prm)) == _lib.GF_EINVAL
    assert lib.gf_md_link_update(None, None, None, ctypes.c_double(0.1), ctypes.byref(prm)) == _lib.GF_EINVAL
    assert lib.gf_stout_create(None, 2, None, _lib.GF_DFLOAT, 1, None) == _lib.GF_EINVAL
    assert lib.gf_rectangle(None, None, ctypes.byref(out)) == _lib.GF_EINVAL
    assert lib.gf_mom_scale(None, None, ctypes.c_double(0.5)) == _lib.GF_EINVAL
    assert lib.gf_action_loops(None, None, ctypes.c_double(1.0), ctypes.c_double(0.1), ctypes.byref(out)) == \
        _lib.GF_EINVAL
    assert lib.gf_force_loops(None, None, ctypes.c_double(1.0), ctypes.c_double(0.1), None) == _lib.GF_EINVAL
    assert lib.gf_flow_loops(None, None, ctypes.c_double(0.01), 1, ctypes.c_double(1.0), ctypes.c_double(0.1)) == \
        _lib.GF_EINVAL
    assert lib.gf_field_free(None) == _lib.GF_OK
    assert lib.gf_ctx_destroy(None) == _lib.GF_OK


def test_python_errors_map_to_argument_errors(pkg):
    from gaugefields_gb300 import _lib
    with pytest.raises(ValueError):
        _lib.call("gf_plaquette", None, None, None)


class _FakeU:
    """Stands in for a configuration in host-side validation tests."""

    def __len__(self):
        return 4


def test_md_driver_argument_validation(pkg):
    U = _FakeU()
    action = pkg.GaugeAction(U)
    pkg.push_(action, 3.0, "plaquette")
    with pytest.raises(ValueError):
        pkg.md_driver(U, action, steps=0)
    with pytest.raises(ValueError):
        pkg.md_driver(U, action, steps=10, trajectory_length=0.0)
    with pytest.raises(ValueError):
        pkg.md_driver(U, action, steps=10, trajectory_length=float("inf"))
    # an integrator without md_step! fails when it steps (test/md_driver.jl:309-320)
    odd = pkg.md_driver(U, action, steps=10, integrator=object())
    with pytest.raises(ValueError, match="md_step! is not implemented"):
        pkg.md_trajectory_(U, None, odd, diagnostics=False)
    with pytest.raises(ValueError):
        pkg.md_driver(U, pkg.GaugeAction(U), steps=10)  # empty action
    drv = pkg.md_driver(U, action, steps=10, trajectory_length=-1.0, integrator=pkg.PQP())
    assert pkg.md_step_size(drv) == -0.1
    p = drv.params()
    assert p.beta == 6.0 and p.steps == 10 and p.integrator == 1 and p.nstout == 0


def test_md_driver_with_smearing_params(pkg):
    U = _FakeU()
    action = pkg.GaugeAction(U)
    pkg.push_(action, 3.0, "plaquette")
    net = pkg.stout_smearing(U, rho=0.1)
    pkg.push_(net, pkg.STOUT_Layer("plaquette", 0.12))
    drv = pkg.md_driver(U, action, steps=20, smearing=net, precision="mixed")
    p = drv.params()
    assert p.nstout == 2 and list(p.rho)[:2] == [0.1, 0.12] and p.precision == 1
    assert pkg.md_driver(U, action, steps=20, smearing=net, precision="dfloat").params().precision == 2
    with pytest.raises(ValueError):
        pkg.md_driver(U, action, steps=20, smearing=net, precision="fp32")


def test_api_argument_validation(pkg):
    with pytest.raises(ValueError):
        pkg.gauge_configuration((4, 4, 4, 4), colors=2)
    with pytest.raises(ValueError):
        pkg.gauge_configuration((4, 4, 4, 4), start="warm")
    with pytest.raises(ValueError):
        pkg.gauge_configuration((4, 4, 4))
    with pytest.raises(ValueError):
        pkg.STOUT_Layer("rectangular", 0.1)
    with pytest.raises(ValueError):
        pkg.gradient_flow(None, steps=0)
    with pytest.raises(ValueError):
        pkg.gradient_flow(None, step_size=-0.1)


def test_md_params_layout_matches_the_header(pkg, tmp_path):
    """The ctypes mirror of gf_md_params has the header's size and offsets."""
    import shutil
    import subprocess
    from gaugefields_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f for f, _ in _lib.MDParams._fields_]
    cnames = {"lam": "lambda"}
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gaugefields_gb300.h"', "int main(void) {",
             '  printf("size %zu\\n", sizeof(gf_md_params));']
    for f in fields:
        lines.append('  printf("%s %%zu\\n", offsetof(gf_md_params, %s));' % (f, cnames.get(f, f)))
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n") if l)
    assert int(out["size"]) == ctypes.sizeof(_lib.MDParams)
    for f in fields:
        assert int(out[f]) == getattr(_lib.MDParams, f).offset, f


def _df_tables():
    """The double-float operation tables of gf_stout.cu: {name: [10-tuples]}."""
    src = open(os.path.join(ROOT, "gaugefields.jl_gb300", "csrc", "gf_stout.cu")).read()
    tables = {}
    for m in re.finditer(r"__constant__ DfOp (c_\w+)\[(\d+)\] = \{(.*?)\n\};", src, re.S):
        body = re.sub(r"//[^\n]*", "", m.group(3))
        rows = [tuple(int(x) for x in r.split(",")) for r in re.findall(r"\{([^{}]*)\}", body)]
        assert len(rows) == int(m.group(2)), m.group(1)
        tables[m.group(1)] = rows
    return src, tables


def test_double_float_op_tables_stay_in_bounds():
    """Every operand and result of the table-driven double-float kernels names
    a field, a site, a direction or a shared-memory slot that the kernel has:
    a slot index beyond the allocation would address shared memory out of
    bounds."""
    src, tables = _df_tables()
    assert set(tables) == {"c_gather_ops", "c_stout_ops", "c_local_ops"}
    nslots = {"c_gather_ops": 2, "c_stout_ops": 2,
              "c_local_ops": int(re.search(r"#define GF_LOCAL_SLOTS (\d+)", src).group(1))}
    # the static shared arrays of the two-slot kernels (forward, gather) hold
    # two slots of 36 floats per thread, 16-byte aligned for the float4 slot
    # accesses
    assert src.count("__shared__ __align__(16) float sm[2 * 36 * 128];") == 2
    for name, rows in tables.items():
        placeholders = {14, 15} if name == "c_local_ops" else set()
        for r in rows:
            assert len(r) == 10, (name, r)
            a_src, a_dir, a_site, a_dag, b_src, b_dir, b_site, b_dag, out, acc = r
            for src_, dir_, site, dag in ((a_src, a_dir, a_site, a_dag), (b_src, b_dir, b_site, b_dag)):
                assert src_ in placeholders or 0 <= src_ < 3 + nslots[name], (name, r)
                assert dir_ in (0, 1) and dag in (0, 1) and 0 <= site <= 4, (name, r)
            assert 0 <= out < nslots[name] and acc in (0, 1), (name, r)
    # the placeholders resolve to fields 1, 2 or slots 4, 5 (src 7, 8)
    assert "recompute ? 8 : 2" in src and "TOP ? 7 : 1" in src
    assert nslots["c_local_ops"] >= 6
    # the local adjoint's shared memory is sized per launch: 4 slots below the
    # top level with stored C, 5 at the top level, all 6 when C is recomputed.
    # The ops such a launch executes (0-11 only when recomputing, 12-23 only
    # at the top level) and their resolved operands stay inside those slots.
    assert "const int nslots = Cst == nullptr ? GF_LOCAL_SLOTS : (top ? 5 : 4);" in src
    rows = tables["c_local_ops"]
    for top, recompute, limit in ((False, False, 4), (True, False, 5), (False, True, 6), (True, True, 6)):
        for q, r in enumerate(rows):
            if (q < 12 and not recompute) or (12 <= q < 24 and not top):
                continue
            a_src, b_src, out = r[0], r[4], r[8]
            srcs = [{14: 8 if recompute else 2, 15: 7 if top else 1}.get(x, x) for x in (a_src, b_src)]
            for x in srcs:
                assert x < 3 or x - 3 < limit, (top, recompute, q, r)
            assert out < limit, (top, recompute, q, r)
        # the hooks between table entries write slots 0-3, plus 4 (top) and 5 (recompute)
        assert limit >= 4


def test_gaussian_momenta_sigma_scales_the_unit_draws(pkg, monkeypatch):
    """gaussian_momenta!(P; sigma): the unit-variance draws of (seed, sweep),
    then P <- sigma P (gf_mom_scale); sigma = 1 makes no second call."""
    import gaugefields_gb300.api as api
    from types import SimpleNamespace
    P = SimpleNamespace(ctx=SimpleNamespace(h="ctx"), field=SimpleNamespace(h="P"))
    seen = []
    monkeypatch.setattr(api, "call", lambda name, *args, ctx=None: seen.append((name, args)))
    pkg.gaussian_momenta_(P, sigma=0.5, seed=7, sweep=3)
    assert [n for n, _ in seen] == ["gf_gaussian_momenta", "gf_mom_scale"]
    assert (seen[0][1][2].value, seen[0][1][3].value) == (7, 3) and seen[1][1][2].value == 0.5
    seen.clear()
    pkg.gaussian_momenta_(P, seed=7, sweep=3)
    assert [n for n, _ in seen] == ["gf_gaussian_momenta"]
    with pytest.raises(ValueError):
        pkg.gaussian_momenta_(P, sigma=float("nan"), seed=7)
    with pytest.raises(ValueError):
        pkg.gaussian_momenta_(P, sweep=-1, seed=7)
