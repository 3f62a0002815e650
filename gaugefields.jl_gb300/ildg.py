"""ILDG gauge-configuration files (save_configuration / load_configuration!
with format=:ildg, src/API.jl:711-826 and src/output/ildg_format.jl).

The file is a LIME container (the USQCD LIME record format: a 144-byte
big-endian header per record - magic 0x456789ab, version 1, message-begin and
message-end flags, data length, a 128-byte type string - then the data padded
with zeros to a multiple of 8 bytes). A configuration is one message of two
records, as the reference writes it through lime_pack
(ildg_format.jl:50-65):

* "ildg-format": the XML header with version, field su3gauge, precision and
  lx, ly, lz, lt (ildg_format.jl:34-48);
* "ildg-binary-data": the links as big-endian reals (precision 64 or 32), the
  sites in lexicographic order with x fastest, per site the four directions
  x, y, z, t, per direction the 3x3 matrix row by row, each entry real then
  imaginary (ildg_format.jl:697-745, :862-887).

A file may hold several configurations; reading takes the one at `index`
(the reference's ildg[i], ildg_format.jl:902). The header rules follow the
reference's reader: the precision comes from the header, 32 when no header
has given one (ildg_format.jl:1111), and a binary record without any header
record, as in the reference's own test files, is read at precision 64 on
the caller's lattice (ildg_format.jl:917-921).

The functions here work on host arrays in this package's host layout, the
reference's per-direction (3, 3, NX, NY, NZ, NT) arrays: a complex128 array of
shape (4, V, 3, 3) whose [mu, lex] block holds the matrix column by column.
"""
import os
import re
import struct

import numpy as np

LIME_MAGIC = 0x456789AB
LIME_VERSION = 1
_MB = 1 << 15
_ME = 1 << 14
_HEADER = struct.Struct(">IHHQ128s")  # 144 bytes

ILDG_NAMESPACE = "http://www.lqcd.org/ildg"
ILDG_FORMAT_VERSION = "1.2"


def format_xml(L, precision, colors=3):
    """The ildg-format record (ildg_format.jl:34-48)."""
    if precision not in (32, 64):
        raise ValueError("ILDG precision must be 32 or 64, got %r" % (precision,))
    return ('<?xml version="1.0" encoding="UTF-8"?>\n'
            '<ildgFormat xmlns="%s">\n'
            '  <version>%s</version>\n'
            '  <field>su%dgauge</field>\n'
            '  <precision>%d</precision>\n'
            '  <lx>%d</lx>\n  <ly>%d</ly>\n  <lz>%d</lz>\n  <lt>%d</lt>\n'
            '</ildgFormat>\n' % (ILDG_NAMESPACE, ILDG_FORMAT_VERSION, colors, precision, *L))


def _pad(n):
    return (-n) % 8


def write_records(fp, records):
    """One LIME message of (type, bytes) records."""
    for i, (rtype, data) in enumerate(records):
        t = rtype.encode()
        if len(t) > 128:
            raise ValueError("LIME record type longer than 128 bytes: %r" % rtype)
        flags = (_MB if i == 0 else 0) | (_ME if i == len(records) - 1 else 0)
        fp.write(_HEADER.pack(LIME_MAGIC, LIME_VERSION, flags, len(data), t.ljust(128, b"\0")))
        fp.write(data)
        fp.write(b"\0" * _pad(len(data)))


def read_records(path):
    """All records of a LIME file: a list of dicts with message and record
    numbers (1-based, as lime_contents prints them), type, flags, the data
    offset and length."""
    out = []
    size = os.path.getsize(path)
    with open(path, "rb") as fp:
        pos, message, record = 0, 0, 0
        while pos < size:
            head = fp.read(_HEADER.size)
            if len(head) != _HEADER.size:
                raise ValueError("%s: truncated LIME header at byte %d" % (path, pos))
            magic, version, flags, length, rtype = _HEADER.unpack(head)
            if magic != LIME_MAGIC:
                raise ValueError("%s: not a LIME file (magic 0x%08x at byte %d)" % (path, magic, pos))
            if flags & _MB:
                message += 1
                record = 0
            record += 1
            start = pos + _HEADER.size
            if start + length > size:
                raise ValueError("%s: LIME record %d.%d runs past the end of the file" % (path, message, record))
            out.append({"message": message, "record": record, "type": rtype.rstrip(b"\0").decode(errors="replace"),
                        "mb": bool(flags & _MB), "me": bool(flags & _ME), "offset": start, "length": length,
                        "version": version})
            pos = start + length + _pad(length)
            fp.seek(pos)
    return out


def _xml_int(xml, tag):
    m = re.search(r"<%s>\s*([^<\s]+)\s*</%s>" % (tag, tag), xml)
    return m.group(1) if m else None


def headers(path):
    """The configurations of an ILDG file: for each ildg-binary-data record,
    the lattice, colours and precision of the last header record before it
    and the record's place (extract_info_fromdict, ildg_format.jl:1100-1206).

    As in the reference, a header record is either "ildg-format" (lx..lt,
    field, precision) or "scidac-private-file-xml" (dims); the colour count
    and the precision carry over from one header record to the next, starting
    at 3 and 32, so an ildg-format record without a precision element has the
    previous one's; a binary record after another one keeps the header of the
    first. A binary record with no header record before it has L, NC and
    precision None: the reader then takes the caller's lattice and colours and
    precision 64, as load_gaugefield! does (ildg_format.jl:917-921)."""
    recs = read_records(path)
    out, fmt = [], None
    nc, precision = 3, 32
    with open(path, "rb") as fp:
        for r in recs:
            if r["type"] in ("ildg-format", "scidac-private-file-xml"):
                fp.seek(r["offset"])
                xml = fp.read(r["length"]).decode(errors="replace")
                if r["type"] == "ildg-format":
                    dims = [_xml_int(xml, t) for t in ("lx", "ly", "lz", "lt")]
                    if None in dims:
                        raise ValueError("%s: ildg-format record without lx, ly, lz, lt" % path)
                    field = re.search(r"<field>\s*([^<\s]+)\s*</field>", xml)
                    if field:
                        m = re.fullmatch(r"su(\d+)gauge", field.group(1))
                        if not m:
                            raise ValueError("%s: field %r is not an su(N) gauge field" % (path, field.group(1)))
                        nc = int(m.group(1))
                    prec = _xml_int(xml, "precision")
                    if prec is not None:
                        precision = int(prec)
                else:
                    m = re.search(r"<dims>\s*([^<]*?)\s*</dims>", xml)
                    dims = m.group(1).split() if m else []
                    if len(dims) != 4:
                        raise ValueError("%s: scidac-private-file-xml record without four dims" % path)
                fmt = {"L": tuple(int(d) for d in dims), "NC": nc, "precision": precision}
            elif r["type"] == "ildg-binary-data":
                head = fmt if fmt is not None else {"L": None, "NC": None, "precision": None}
                out.append(dict(head, message=r["message"], record=r["record"], offset=r["offset"],
                                length=r["length"]))
    return out


def _payload_order(links):
    """(4, V, 3, 3) host layout [mu, lex, col, row] -> [lex, mu, row, col]."""
    return np.ascontiguousarray(np.transpose(np.swapaxes(links, -1, -2), (1, 0, 2, 3)))


def write(path, links, L, precision=64, append=False):
    """Write one configuration (host layout, complex) as an ILDG message."""
    L = tuple(int(x) for x in L)
    V = int(np.prod(L))
    links = np.asarray(links)
    if links.shape != (4, V, 3, 3):
        raise ValueError("links have shape %s; expected (4, %d, 3, 3)" % (links.shape, V))
    if precision not in (32, 64):
        raise ValueError("ILDG precision must be 32 or 64, got %r" % (precision,))
    ordered = _payload_order(links.astype(np.complex128, copy=False))
    reals = ordered.view(np.float64).reshape(-1)
    payload = reals.astype(">f8" if precision == 64 else ">f4").tobytes()
    with open(path, "ab" if append else "wb") as fp:
        write_records(fp, [("ildg-format", format_xml(L, precision).encode()), ("ildg-binary-data", payload)])


def read(path, L=None, index=1, NC=3):
    """Read configuration `index` (1-based) into the host layout, a complex
    array of shape (4, V, NC, NC); checks the lattice against L and the colour
    count against NC. L is required when the binary record has no header
    record before it. Returns (links, header) with the header's L, NC and
    precision filled in. The backend's fields take NC = 3; other NC serve
    reading the reference's SU(2) files."""
    hs = headers(path)
    if not hs:
        raise ValueError("%s: no ildg-binary-data record" % path)
    if not 1 <= index <= len(hs):
        raise ValueError("%s holds %d configuration(s); index %d" % (path, len(hs), index))
    h = dict(hs[index - 1])
    if h["L"] is None:
        if L is None:
            raise ValueError("%s: binary record %d.%d has no header record; the lattice must be given"
                             % (path, h["message"], h["record"]))
        h.update(L=tuple(int(x) for x in L), NC=int(NC), precision=64)
    if h["NC"] != NC:
        raise ValueError("%s: su(%d) field; expected su(%d)" % (path, h["NC"], NC))
    if L is not None and tuple(int(x) for x in L) != h["L"]:
        raise ValueError("%s: lattice %s does not match the target %s" % (path, h["L"], tuple(L)))
    if h["precision"] not in (32, 64):
        raise ValueError("%s: ILDG precision must be 32 or 64, got %r" % (path, h["precision"]))
    V = int(np.prod(h["L"]))
    width = 8 if h["precision"] == 64 else 4
    need = V * 4 * NC * NC * 2 * width
    if h["length"] != need:
        raise ValueError("%s: binary record of %d bytes; a %s su(%d) lattice at precision %d needs %d"
                         % (path, h["length"], h["L"], NC, h["precision"], need))
    with open(path, "rb") as fp:
        fp.seek(h["offset"])
        raw = np.frombuffer(fp.read(h["length"]), dtype=">f8" if width == 8 else ">f4")
    ordered = raw.astype(np.float64).view(np.complex128).reshape(V, 4, NC, NC)   # [lex, mu, row, col]
    links = np.ascontiguousarray(np.swapaxes(np.transpose(ordered, (1, 0, 2, 3)), -1, -2))
    return links, h
