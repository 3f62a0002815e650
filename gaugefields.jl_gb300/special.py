"""The lattice one-instanton configuration, built on the host
(Oneinstanton / _su2_instanton_link / Oneinstanton_SUN_embedded,
src/AbstractGaugefields.jl:998-1184 and :1495-1581).

For a site with zero-based coordinates x and the instanton centre c (default
L/2 + 1/2 in every direction, so that no site sits on it), n = x - c and
n2 = |n|^2. With s = (i sigma_1, i sigma_2, i sigma_3, 1) and its conjugate
s~ = (-i sigma_1, -i sigma_2, -i sigma_3, 1), the SU(2) link in direction mu is

    U_mu(x) = exp(-R^2 T_mu / (2 n2 (n2 + R^2))),
    T_mu = sum_nu (s~_mu s_nu - s~_nu s_mu) n_nu          (instanton, sign +1)
    T_mu = sum_nu (s_mu s~_nu - s_nu s~_mu) n_nu          (anti-instanton, -1)

with radius R (default NX div 2). T_mu is i times a real combination of the
Pauli matrices, so the exponential has the closed form
cos(t) + sin(t)/t X for X in su(2), t^2 = det X. The SU(N) form places the
SU(2) link in the rows and columns `block` (1-based, i < j) of the identity.

Arrays are in the package's host layout: complex (4, V, NC, NC), each [mu, lex]
block the matrix column by column, lex with x fastest.
"""
import numpy as np

_PAULI = np.array([[[0, 1], [1, 0]], [[0, -1j], [1j, 0]], [[1, 0], [0, -1]]], dtype=np.complex128)
_S = np.concatenate([1j * _PAULI, np.eye(2, dtype=np.complex128)[None]])        # s_nu
_SBAR = np.concatenate([-1j * _PAULI, np.eye(2, dtype=np.complex128)[None]])    # s~_nu


def validate_block(NC, block):
    """_validate_su2_embedding_block (AbstractGaugefields.jl:1095-1106)."""
    if not isinstance(NC, (int, np.integer)) or NC < 2:
        raise ValueError("NC must be an integer of at least 2; got %r" % (NC,))
    if len(block) != 2:
        raise ValueError("block must contain two color indices; got %r" % (block,))
    i, j = block
    if not all(isinstance(b, (int, np.integer)) for b in (i, j)):
        raise ValueError("block indices must be integers; got %r" % (block,))
    if not 1 <= i < j <= NC:
        raise ValueError("block must satisfy 1 <= i < j <= NC; got %r for NC = %d" % (tuple(block), NC))
    return int(i), int(j)


def su2_instanton_links(L, center=None, radius=None, sign=1):
    """The SU(2) instanton links of every site and direction, (4, V, 2, 2)."""
    L = tuple(int(x) for x in L)
    if len(L) != 4:
        raise ValueError("L must contain four lattice extents")
    if sign not in (-1, 1):
        raise ValueError("sign must be +1 or -1")
    c = np.array([x / 2 + 0.5 for x in L] if center is None else center, dtype=np.float64)
    if c.shape != (4,):
        raise ValueError("center must contain four coordinates")
    R = L[0] // 2 if radius is None else radius
    if not R > 0:
        raise ValueError("radius must be positive")
    # zero-based coordinates in lex order (x fastest)
    t, z, y, x = np.meshgrid(*(np.arange(n, dtype=np.float64) for n in L[::-1]), indexing="ij")
    n = np.stack([x.ravel(), y.ravel(), z.ravel(), t.ravel()], axis=1) - c          # (V, 4)
    n2 = np.einsum("vk,vk->v", n, n)
    if not np.all(np.isfinite(n2)):
        raise ValueError("instanton center must contain finite coordinates")
    if np.any(n2 <= 0):
        raise ValueError("instanton center must not coincide with a zero-based lattice site")
    if sign == 1:
        pair = np.einsum("mab,nbc->mnac", _SBAR, _S)       # s~_mu s_nu
    else:
        pair = np.einsum("mab,nbc->mnac", _S, _SBAR)       # s_mu s~_nu
    gen = pair - np.swapaxes(pair, 0, 1)                   # (mu, nu, 2, 2)
    T = np.einsum("mnac,vn->mvac", gen, n)                 # (mu, V, 2, 2)
    X = T * (-(R * R) / (2.0 * n2 * (n2 + R * R)))[None, :, None, None]
    det = (X[..., 0, 0] * X[..., 1, 1] - X[..., 0, 1] * X[..., 1, 0]).real
    theta = np.sqrt(np.maximum(det, 0.0))
    U = np.cos(theta)[..., None, None] * np.eye(2) + np.sinc(theta / np.pi)[..., None, None] * X
    return np.ascontiguousarray(np.swapaxes(U, -1, -2))


def embed_su2(links2, NC=3, block=(1, 2)):
    """_embed_su2_matrix_in_sun! on every link (AbstractGaugefields.jl:1108-1124):
    host-layout SU(2) links (4, V, 2, 2) -> SU(NC) links (4, V, NC, NC)."""
    i, j = validate_block(NC, block)
    links2 = np.asarray(links2)
    out = np.zeros(links2.shape[:2] + (NC, NC), dtype=np.complex128)
    out[..., range(NC), range(NC)] = 1.0
    idx = (i - 1, j - 1)
    for a in range(2):
        for b in range(2):
            out[..., idx[a], idx[b]] = links2[..., a, b]
    return out


def oneinstanton_sun_embedded(NC, L, center=None, radius=None, sign=1, block=(1, 2)):
    """Oneinstanton_SUN_embedded (AbstractGaugefields.jl:1495-1581) on the host."""
    validate_block(NC, block)
    return embed_su2(su2_instanton_links(L, center, radius, sign), NC, block)
