"""Bridge++ text gauge-configuration files (save_configuration /
load_configuration! with format=:bridge; src/API.jl:711-826,
src/output/bridge_format.jl:201-297).

One real per line: the sites in lexicographic order with x fastest, per site
the four directions x, y, z, t, per direction the 3x3 matrix row by row, each
entry its real part then its imaginary part (the loop order of save_textdata
and load_BridgeText!). Values are written as the shortest decimal that reads
back to the same double, so a round trip is exact; reading accepts any
decimal or exponent notation (Julia's println form included). A file whose
line count is not 4 x 9 x 2 x V is rejected, as the reference asserts.

The functions work on the host layout: a complex128 array of shape
(4, V, 3, 3) whose [mu, lex] block holds the matrix column by column.
"""
import numpy as np


def _payload_order(links):
    """[mu, lex, col, row] -> [lex, mu, row, col]."""
    return np.ascontiguousarray(np.transpose(np.swapaxes(links, -1, -2), (1, 0, 2, 3)))


def write(path, links, L):
    L = tuple(int(x) for x in L)
    V = int(np.prod(L))
    links = np.asarray(links)
    if links.shape != (4, V, 3, 3):
        raise ValueError("links have shape %s; expected (4, %d, 3, 3)" % (links.shape, V))
    reals = _payload_order(links.astype(np.complex128, copy=False)).view(np.float64).reshape(-1)
    with open(path, "w") as fp:
        fp.write("\n".join(map(repr, reals.tolist())))
        fp.write("\n")


def read(path, L):
    L = tuple(int(x) for x in L)
    V = int(np.prod(L))
    with open(path) as fp:
        words = fp.read().split()
    if len(words) != 4 * 9 * 2 * V:
        raise ValueError("%s holds %d values; a %s lattice needs %d" % (path, len(words), L, 4 * 9 * 2 * V))
    try:
        reals = np.asarray(words, dtype=np.float64)
    except ValueError as e:
        raise ValueError("%s: not a list of numbers (%s)" % (path, e))
    ordered = reals.view(np.complex128).reshape(V, 4, 3, 3)   # [lex, mu, row, col]
    return np.ascontiguousarray(np.swapaxes(np.transpose(ordered, (1, 0, 2, 3)), -1, -2))
