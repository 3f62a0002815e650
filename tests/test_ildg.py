"""ILDG and Bridge++ configuration files (save_configuration /
load_configuration! with format=:ildg or :bridge; src/API.jl:711-826,
src/output/ildg_format.jl, src/output/bridge_format.jl) on the host
layout, against links from the oracle's Haar generator. CPU only, except the
last test, which goes through a device configuration."""
import struct

import numpy as np
import pytest

import __graft_entry__ as entry

L4 = (4, 4, 4, 4)
L_MIXED = (4, 2, 6, 2)


@pytest.fixture(scope="module")
def io():
    entry.load_package()
    from gaugefields_gb300 import ildg as mod
    return mod


def _links(oracle, L, seed):
    return oracle.hot_start(list(L), seed)


def test_round_trip_fp64_is_exact(io, oracle, tmp_path):
    U = _links(oracle, L_MIXED, 3)
    f = tmp_path / "a.ildg"
    io.write(str(f), U, L_MIXED, 64)
    V, h = io.read(str(f), L=L_MIXED)
    assert np.array_equal(V, U)
    assert h["L"] == L_MIXED and h["precision"] == 64 and h["NC"] == 3


def test_round_trip_fp32(io, oracle, tmp_path):
    U = _links(oracle, L4, 4)
    f = tmp_path / "b.ildg"
    io.write(str(f), U, L4, 32)
    V, h = io.read(str(f))
    assert h["precision"] == 32
    assert np.abs(V - U).max() < 1.2e-7
    assert np.array_equal(V, U.astype(np.complex64).astype(np.complex128))


def test_lime_structure_and_header(io, oracle, tmp_path):
    U = _links(oracle, L_MIXED, 5)
    f = tmp_path / "c.ildg"
    io.write(str(f), U, L_MIXED, 64)
    recs = io.read_records(str(f))
    assert [r["type"] for r in recs] == ["ildg-format", "ildg-binary-data"]
    assert recs[0]["mb"] and not recs[0]["me"] and not recs[1]["mb"] and recs[1]["me"]
    assert all(r["message"] == 1 for r in recs) and [r["record"] for r in recs] == [1, 2]
    raw = f.read_bytes()
    assert len(raw) % 8 == 0
    assert struct.unpack(">I", raw[:4])[0] == 0x456789AB
    xml = raw[recs[0]["offset"]:recs[0]["offset"] + recs[0]["length"]].decode()
    for tag, val in (("field", "su3gauge"), ("precision", "64"), ("lx", "4"), ("ly", "2"), ("lz", "6"), ("lt", "2")):
        assert "<%s>%s</%s>" % (tag, val, tag) in xml
    assert 'xmlns="http://www.lqcd.org/ildg"' in xml
    V = int(np.prod(L_MIXED))
    assert recs[1]["length"] == V * 4 * 9 * 16


def test_payload_order_is_site_direction_row_column(io, oracle, tmp_path):
    """x fastest over the sites, then directions x, y, z, t, then each matrix
    row by row, real before imaginary, big-endian (ildg_format.jl:697-745)."""
    U = _links(oracle, L_MIXED, 6)
    f = tmp_path / "d.ildg"
    io.write(str(f), U, L_MIXED, 64)
    rec = io.read_records(str(f))[1]
    raw = f.read_bytes()[rec["offset"]:rec["offset"] + rec["length"]]
    NX, NY, NZ, NT = L_MIXED
    for (x, y, z, t, mu, row, col) in ((0, 0, 0, 0, 0, 0, 0), (1, 0, 0, 0, 2, 1, 2), (3, 1, 5, 1, 3, 2, 0)):
        lex = x + NX * (y + NY * (z + NZ * t))
        k = (((lex * 4 + mu) * 3 + row) * 3 + col) * 2
        re, im = struct.unpack(">dd", raw[8 * k:8 * k + 16])
        # host layout: [mu, lex] holds the matrix column by column
        assert (re, im) == (U[mu, lex, col, row].real, U[mu, lex, col, row].imag)


def test_several_configurations_in_one_file(io, oracle, tmp_path):
    A, B = _links(oracle, L4, 7), _links(oracle, L4, 8)
    f = tmp_path / "e.ildg"
    io.write(str(f), A, L4, 64)
    io.write(str(f), B, L4, 32, append=True)
    hs = io.headers(str(f))
    assert [h["precision"] for h in hs] == [64, 32] and [h["message"] for h in hs] == [1, 2]
    assert np.array_equal(io.read(str(f), index=1)[0], A)
    assert np.abs(io.read(str(f), index=2)[0] - B).max() < 1.2e-7
    with pytest.raises(ValueError):
        io.read(str(f), index=3)


def test_missing_precision_element_means_32(io, oracle, tmp_path):
    """The reference's reader assumes precision 32 without the element."""
    U = _links(oracle, L4, 9)
    xml = io.format_xml(L4, 32).replace("  <precision>32</precision>\n", "").encode()
    ordered = np.ascontiguousarray(np.transpose(np.swapaxes(U, -1, -2), (1, 0, 2, 3)))
    payload = ordered.view(np.float64).reshape(-1).astype(">f4").tobytes()
    f = tmp_path / "f.ildg"
    with open(f, "wb") as fp:
        io.write_records(fp, [("ildg-format", xml), ("ildg-binary-data", payload)])
    V, h = io.read(str(f))
    assert h["precision"] == 32 and np.abs(V - U).max() < 1.2e-7


def test_header_rules_of_the_reference_reader(io, oracle, tmp_path):
    """extract_info_fromdict (ildg_format.jl:1100-1206): the precision carries
    over between header records; a second binary record keeps the header of
    the first; a scidac-private-file-xml record gives the lattice; a binary
    record with no header is read at precision 64 on the caller's lattice
    (load_gaugefield!, ildg_format.jl:917-921)."""
    A, B = _links(oracle, L4, 13), _links(oracle, L4, 14)

    def payload(U, dt):
        ordered = np.ascontiguousarray(np.transpose(np.swapaxes(U, -1, -2), (1, 0, 2, 3)))
        return ordered.view(np.float64).reshape(-1).astype(dt).tobytes()

    f = tmp_path / "carry.ildg"
    no_prec = io.format_xml(L4, 64).replace("  <precision>64</precision>\n", "").encode()
    with open(f, "wb") as fp:
        io.write_records(fp, [("ildg-format", io.format_xml(L4, 64).encode()), ("ildg-binary-data", payload(A, ">f8"))])
        io.write_records(fp, [("ildg-format", no_prec), ("ildg-binary-data", payload(B, ">f8")),
                              ("ildg-binary-data", payload(A, ">f8"))])
    hs = io.headers(str(f))
    assert [h["precision"] for h in hs] == [64, 64, 64] and [h["message"] for h in hs] == [1, 2, 2]
    assert np.array_equal(io.read(str(f), index=2)[0], B) and np.array_equal(io.read(str(f), index=3)[0], A)

    g = tmp_path / "scidac.ildg"
    scidac = b"<?xml version=\"1.0\"?><scidacFile><version>1.1</version><spacetime>4</spacetime>" \
             b"<dims>4 4 4 4 </dims><volfmt>0</volfmt></scidacFile>"
    with open(g, "wb") as fp:
        io.write_records(fp, [("scidac-private-file-xml", scidac), ("ildg-binary-data", payload(A, ">f4"))])
    V, h = io.read(str(g), L=L4)
    assert h["L"] == L4 and h["precision"] == 32 and np.abs(V - A).max() < 1.2e-7

    n = tmp_path / "bare.ildg"
    with open(n, "wb") as fp:
        io.write_records(fp, [("ildg-binary-data", payload(B, ">f8"))])
    assert io.headers(str(n))[0]["L"] is None
    with pytest.raises(ValueError):
        io.read(str(n))                            # no header and no lattice
    V, h = io.read(str(n), L=L4)
    assert np.array_equal(V, B) and h["precision"] == 64 and h["L"] == L4 and h["NC"] == 3
    with pytest.raises(ValueError):
        io.read(str(n), L=(4, 4, 4, 2))            # payload size of another lattice


def _pin():
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "ildg_reference_pin", os.path.join(os.path.dirname(__file__), "golden", "ildg_reference_pin.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_reference_ildg_files_pin_the_payload_order(io):
    """The reference's own SU(2) test file has the plaquette that its test
    set expects (test/init.jl:407-425) in the reader's payload order and not
    with the matrices transposed. The record was made by
    tests/golden/ildg_reference_pin.py; where the reference tree is present,
    the files are read again and must give the recorded numbers bit for bit."""
    import json
    import os
    pin = _pin()
    with open(pin.RECORD) as fp:
        record = json.load(fp)["reference_files"]
    assert set(record) == set(pin.FIXTURES)
    pinned = 0
    for name, e in record.items():
        assert e["precision"] == 64 and [r["type"] for r in e["records"]] == ["ildg-binary-data"]
        assert e["max_unitarity_error"] < 1e-14
        if e["golden_plaquette"] is not None:
            g = e["golden_plaquette"]
            assert abs(e["plaquette"] - g) <= 1e-13 * abs(g) and abs(e["plaquette"] - g) <= e["golden_rtol"] * abs(g)
            assert abs(e["plaquette_transposed"] - g) > 0.5 * abs(g)
            pinned += 1
    assert pinned == 1
    root = pin.reference_root()
    if root is None:
        pytest.skip("GF_REFERENCE_ROOT not set; checked the record only")
    present = [n for n in record if os.path.exists(os.path.join(root, n))]
    if not present:
        pytest.skip("reference test files not present; checked the record only")
    for name in present:
        again = pin.derive(root, name, pin.FIXTURES[name], io)
        for key in ("sha256", "bytes", "records", "precision", "plaquette", "plaquette_transposed"):
            assert again[key] == record[name][key], (name, key)


def test_su2_plaquette_helper_on_a_cold_field():
    pin = _pin()
    cold = np.broadcast_to(np.eye(2, dtype=np.complex128), (4, 4 ** 4, 2, 2))
    assert pin.plaquette(cold, (4, 4, 4, 4), 2) == 1.0


def test_rejections(io, oracle, tmp_path):
    U = _links(oracle, L4, 10)
    f = tmp_path / "g.ildg"
    io.write(str(f), U, L4, 64)
    with pytest.raises(ValueError):
        io.read(str(f), L=(4, 4, 4, 2))           # lattice mismatch
    bad = tmp_path / "h.ildg"
    bad.write_bytes(b"\0" * 144)
    with pytest.raises(ValueError):
        io.read(str(bad))                          # not LIME
    nofmt = tmp_path / "i.ildg"
    with open(nofmt, "wb") as fp:
        io.write_records(fp, [("ildg-binary-data", b"\0" * 16)])
    with pytest.raises(ValueError):
        io.read(str(nofmt))                        # no ildg-format record
    short = tmp_path / "j.ildg"
    with open(short, "wb") as fp:
        io.write_records(fp, [("ildg-format", io.format_xml(L4, 64).encode()), ("ildg-binary-data", b"\0" * 64)])
    with pytest.raises(ValueError):
        io.read(str(short))                        # payload of the wrong size
    with pytest.raises(ValueError):
        io.write(str(f), U, L4, 16)                # precision


def test_read_configuration_has_the_oracle_plaquette(io, oracle, tmp_path):
    U = _links(oracle, L_MIXED, 11)
    f = tmp_path / "k.ildg"
    io.write(str(f), U, L_MIXED, 64)
    V, _ = io.read(str(f))
    assert oracle.plaquette(list(L_MIXED), V) == oracle.plaquette(list(L_MIXED), U)


def test_bridge_text_round_trip_and_layout(oracle, tmp_path):
    """Bridge++ text (bridge_format.jl:201-297): one real per line, sites with
    x fastest, then direction, row, column, real before imaginary."""
    entry.load_package()
    from gaugefields_gb300 import bridge
    U = _links(oracle, L_MIXED, 12)
    f = tmp_path / "conf.txt"
    bridge.write(str(f), U, L_MIXED)
    lines = f.read_text().split("\n")[:-1]
    V = int(np.prod(L_MIXED))
    assert len(lines) == 4 * 9 * 2 * V
    NX, NY, NZ, NT = L_MIXED
    x, y, z, t, mu, row, col = 3, 1, 5, 1, 2, 0, 2
    lex = x + NX * (y + NY * (z + NZ * t))
    k = (((lex * 4 + mu) * 3 + row) * 3 + col) * 2
    assert float(lines[k]) == U[mu, lex, col, row].real and float(lines[k + 1]) == U[mu, lex, col, row].imag
    assert np.array_equal(bridge.read(str(f), L_MIXED), U)
    # the notation Julia's println uses reads back too
    g = tmp_path / "julia.txt"
    g.write_text("\n".join(("%.17e" % float(v)).replace("e-0", "e-").replace("e+0", "e") for v in lines) + "\n")
    assert np.array_equal(bridge.read(str(g), L_MIXED), U)
    with pytest.raises(ValueError):
        bridge.read(str(f), (4, 4, 4, 4))         # line count of another lattice


def test_package_exports_the_configuration_io(pkg):
    assert callable(pkg.save_configuration) and callable(pkg.load_configuration_)
    with pytest.raises(ValueError):
        pkg.save_configuration("x.ildg", None, format="jld2")
    with pytest.raises(ValueError):
        pkg.load_configuration_(None, "x.ildg", format="jld2")


@pytest.mark.gpu
def test_save_and_load_through_the_device(pkg, tmp_path):
    U = pkg.gauge_configuration(L_MIXED, start="hot", seed=21)
    f = str(tmp_path / "dev.ildg")
    pkg.save_configuration(f, U, format="ildg")
    W = pkg.gauge_configuration(L_MIXED, start="cold")
    pkg.load_configuration_(W, f, format="ildg")
    assert np.array_equal(W.to_host(), U.to_host())
    assert pkg.measure_plaquette(W) == pkg.measure_plaquette(U)
    with pytest.raises(ValueError):
        pkg.load_configuration_(pkg.gauge_configuration(L4, start="cold"), f, format="ildg")
    with pytest.raises(ValueError):
        pkg.save_configuration(f, U, format="jld2")
    t = str(tmp_path / "dev.txt")
    pkg.save_configuration(t, U, format="bridge")
    X = pkg.gauge_configuration(L_MIXED, start="cold")
    pkg.load_configuration_(X, t, format="bridge")
    assert np.array_equal(X.to_host(), U.to_host())
