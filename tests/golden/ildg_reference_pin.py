"""Pin of the ILDG reader against the reference's own test files.

The reference's test tree holds two LIME files written by the reference
(test/data/conf_00000100_4444_test.ildg and conf_00000100_4444nc2.ildg): 4^4
SU(2) configurations, each a single ildg-binary-data record without a header
record. test/init.jl:407-425 (the "File start" test set) loads the first on a
4^4 SU(2) lattice and expects the plaquette -0.007853743153861798, normalised
by 1/(6 V NC), at the relative tolerance 1e-8 of test/init.jl:255.

This script reads those files through gaugefields_gb300.ildg, computes the
plaquette with numpy, and writes ildg_reference_pin.json beside itself: the
files' SHA-256, their record layout, the plaquette in the payload order the
reader uses and, for contrast, with every matrix transposed. The files are
not copied. tests/test_ildg.py checks the record against the reference's
number and, where the reference tree is present, reads the files again.

    GF_REFERENCE_ROOT=<reference checkout> python tests/golden/ildg_reference_pin.py
    python tests/golden/ildg_reference_pin.py <reference checkout>

The reference root is the argument, else the environment variable
GF_REFERENCE_ROOT; there is no default location.
"""
import hashlib
import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
RECORD = os.path.join(HERE, "ildg_reference_pin.json")

FIXTURES = {
    "test/data/conf_00000100_4444_test.ildg": {
        "L": [4, 4, 4, 4], "NC": 2,
        "golden_plaquette": -0.007853743153861798, "golden_rtol": 1e-8,
        "golden_source": "test/init.jl:407-425 (tolerance test/init.jl:255)",
    },
    "test/data/conf_00000100_4444nc2.ildg": {
        "L": [4, 4, 4, 4], "NC": 2,
        "golden_plaquette": None, "golden_rtol": None, "golden_source": None,
    },
}


def reference_root(argv=()):
    """The reference checkout to read, or None when none was given."""
    if argv:
        return argv[0]
    return os.environ.get("GF_REFERENCE_ROOT") or None


def ildg_module():
    spec = importlib.util.spec_from_file_location("gf_ildg", os.path.join(REPO, "gaugefields.jl_gb300", "ildg.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def plaquette(links, L, NC):
    """Sum over x and mu < nu of Re tr U_mu(x) U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+,
    divided by 6 V NC (calculate_Plaquette times the factor of
    test/init.jl:60-62). links: host layout (4, V, NC, NC), each [mu, lex]
    block the matrix column by column; lex has x fastest."""
    NX, NY, NZ, NT = L
    V = NX * NY * NZ * NT
    # [mu, t, z, y, x, row, col]
    U = np.swapaxes(np.asarray(links), -1, -2).reshape(4, NT, NZ, NY, NX, NC, NC)
    axis = {0: 3, 1: 2, 2: 1, 3: 0}   # direction -> array axis of U[mu]

    def dag(m):
        return np.conj(np.swapaxes(m, -1, -2))

    s = 0.0
    for mu in range(4):
        for nu in range(mu + 1, 4):
            a = U[mu]
            b = np.roll(U[nu], -1, axis=axis[mu])
            c = np.roll(U[mu], -1, axis=axis[nu])
            p = a @ b @ dag(c) @ dag(U[nu])
            s += float(np.trace(p, axis1=-2, axis2=-1).real.sum())
    return s / (6 * V * NC)


def derive(root, name, spec, io=None):
    """Read one reference file and return its record entry."""
    io = io or ildg_module()
    path = os.path.join(root, name)
    with open(path, "rb") as fp:
        digest = hashlib.sha256(fp.read()).hexdigest()
    links, head = io.read(path, L=spec["L"], NC=spec["NC"])
    records = [{k: r[k] for k in ("type", "length", "mb", "me")} for r in io.read_records(path)]
    return {
        "sha256": digest,
        "bytes": os.path.getsize(path),
        "records": records,
        "precision": head["precision"],
        "plaquette": plaquette(links, spec["L"], spec["NC"]),
        "plaquette_transposed": plaquette(np.swapaxes(links, -1, -2), spec["L"], spec["NC"]),
        "max_unitarity_error": float(np.abs(np.swapaxes(links, -1, -2) @ np.conj(links)
                                            - np.eye(spec["NC"])).max()),
    }


def main(argv):
    root = reference_root(argv)
    if root is None:
        sys.exit("give the reference checkout as the argument or in GF_REFERENCE_ROOT")
    out = {"reference_files": {}}
    for name, spec in FIXTURES.items():
        entry = dict(spec)
        entry.update(derive(root, name, spec))
        out["reference_files"][name] = entry
    with open(RECORD, "w") as fp:
        json.dump(out, fp, indent=1, sort_keys=True)
        fp.write("\n")
    for name, e in out["reference_files"].items():
        print(name, e["plaquette"], e["golden_plaquette"])


if __name__ == "__main__":
    main(sys.argv[1:])
