"""The one-instanton configuration (Oneinstanton, Oneinstanton_SUN_embedded;
src/AbstractGaugefields.jl:998-1184, :1495-1581) and the golden plaquette the
reference's tests hold for it.

test/init.jl:351-371 builds Oneinstanton(NC, NX, NY, NZ, NT, Nwing) with
NC = 2, NX = NY = NZ = NT = 4 and Nwing = 1. Against the signature
Oneinstanton(NC, NDW, NN...) those arguments are NDW = 4 and the lattice
(4, 4, 4, 1), and the test expects the plaquette 0.9796864531099871 (relative
tolerance 1e-8, test/init.jl:255). test/sun_embedded_instanton.jl:149 relates
the SU(N) embedding to it: P_SU(N) = (2 P_SU(2) + N - 2) / N. Both give the
oracle's SU(3) plaquette a golden number written by the reference."""
import importlib.util
import os

import numpy as np
import pytest

import __graft_entry__ as entry

GOLDEN_SU2 = 0.9796864531099871          # test/init.jl:369
GOLDEN_L = (4, 4, 4, 1)


@pytest.fixture(scope="module")
def special():
    entry.load_package()
    from gaugefields_gb300 import special as mod
    return mod


def _plaquette(links, L, NC):
    spec = importlib.util.spec_from_file_location(
        "ildg_reference_pin", os.path.join(os.path.dirname(__file__), "golden", "ildg_reference_pin.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.plaquette(links, L, NC)


def _mats(links):
    return np.swapaxes(links, -1, -2)     # host layout -> [mu, lex, row, col]


def test_su2_instanton_has_the_reference_plaquette(special):
    P = _plaquette(special.su2_instanton_links(GOLDEN_L), GOLDEN_L, 2)
    assert abs(P - GOLDEN_SU2) <= 1e-14 * GOLDEN_SU2


def test_oracle_plaquette_of_the_embedded_instanton(special, oracle):
    """The oracle's SU(3) plaquette, on the golden lattice, equals the
    reference's number through the embedding identity, for every block."""
    V = int(np.prod(GOLDEN_L))
    want = (2 * GOLDEN_SU2 + 1) / 3
    for block in ((1, 2), (1, 3), (2, 3)):
        U = special.oneinstanton_sun_embedded(3, GOLDEN_L, block=block)
        got = oracle.plaquette(list(GOLDEN_L), U) / (6 * V * 3)
        assert abs(got - want) <= 1e-14, (block, got, want)
    # and on a 4^4 lattice, against the SU(2) plaquette computed here
    L = (4, 4, 4, 4)
    P2 = _plaquette(special.su2_instanton_links(L), L, 2)
    got = oracle.plaquette(list(L), special.oneinstanton_sun_embedded(3, L)) / (6 * 256 * 3)
    assert abs(got - (2 * P2 + 1) / 3) <= 1e-14


def test_links_are_special_unitary_and_embedded(special):
    """The checks of test/sun_embedded_instanton.jl:63-150: unitarity, unit
    determinant, the SU(2) block in place and the spectator colour 1."""
    L = (4, 4, 4, 4)
    for sign in (1, -1):
        u2 = _mats(special.su2_instanton_links(L, sign=sign))
        assert np.abs(u2 @ np.conj(np.swapaxes(u2, -1, -2)) - np.eye(2)).max() < 1e-15
        assert np.abs(np.linalg.det(u2) - 1).max() < 1e-15
    u2 = _mats(special.su2_instanton_links(L))
    for block in ((1, 2), (1, 3), (2, 3)):
        u3 = _mats(special.oneinstanton_sun_embedded(3, L, block=block))
        i, j = block[0] - 1, block[1] - 1
        k = 3 - i - j
        assert np.array_equal(u3[..., [i, i, j, j], [i, j, i, j]], u2[..., [0, 0, 1, 1], [0, 1, 0, 1]])
        assert np.all(u3[..., k, k] == 1) and np.all(u3[..., k, [i, j]] == 0) and np.all(u3[..., [i, j], k] == 0)
        assert np.abs(np.linalg.det(u3) - 1).max() < 1e-15
    # instanton and anti-instanton differ; both are smooth (plaquette near 1)
    a, b = (_plaquette(special.su2_instanton_links(L, sign=s), L, 2) for s in (1, -1))
    assert 0.9 < a < 1 and 0.9 < b < 1


def test_exponential_closed_form_matches_scipy(special):
    sl = pytest.importorskip("scipy.linalg")
    L = (6, 4, 2, 4)
    U = _mats(special.su2_instanton_links(L, radius=2.5, center=(1.2, 0.7, 3.1, 2.2)))
    # rebuild one link from the generator directly
    x = np.array([5, 3, 1, 2], dtype=float)
    n = x - np.array([1.2, 0.7, 3.1, 2.2])
    n2 = n @ n
    s = [1j * m for m in (np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.array([[1, 0], [0, -1]]))]
    s = s + [np.eye(2)]
    sb = [-m for m in s[:3]] + [np.eye(2)]
    lex = 5 + 6 * (3 + 4 * (1 + 2 * 2))
    for mu in range(4):
        T = sum((sb[mu] @ s[nu] - sb[nu] @ s[mu]) * n[nu] for nu in range(4))
        ref = sl.expm(1j * T * 0.5 / n2 * (1j * 2.5 ** 2 / (n2 + 2.5 ** 2)))
        assert np.abs(U[mu, lex] - ref).max() < 1e-15


def test_argument_validation(special):
    with pytest.raises(ValueError):
        special.oneinstanton_sun_embedded(3, (4, 4, 4, 4), block=(1, 1))
    with pytest.raises(ValueError):
        special.oneinstanton_sun_embedded(3, (4, 4, 4, 4), block=(1, 4))
    with pytest.raises(ValueError):
        special.oneinstanton_sun_embedded(3, (4, 4, 4, 4), block=(2, 1))
    with pytest.raises(ValueError):
        special.oneinstanton_sun_embedded(3, (4, 4, 4, 4), block=(1, 2, 3))
    with pytest.raises(ValueError):
        special.validate_block(1, (1, 2))
    with pytest.raises(ValueError):
        special.su2_instanton_links((4, 4, 4, 4), radius=0)
    with pytest.raises(ValueError):
        special.su2_instanton_links((4, 4, 4, 4), sign=0)
    with pytest.raises(ValueError):
        special.su2_instanton_links((4, 4, 4, 4), center=(1, 2, 3))
    with pytest.raises(ValueError, match="coincide"):
        special.oneinstanton_sun_embedded(3, (5, 5, 5, 5))   # the default centre is the site (3, 3, 3, 3)
    with pytest.raises(ValueError):
        special.su2_instanton_links((4, 4, 4))


def test_package_exports_the_instanton(pkg):
    assert callable(pkg.Oneinstanton_SUN_embedded)
    with pytest.raises(ValueError):
        pkg.Oneinstanton_SUN_embedded(2, 4, 4, 4, 4)
    with pytest.raises(ValueError):
        pkg.Oneinstanton_SUN_embedded(3, 4, 4, 4, 4, NDW=-1)


@pytest.mark.gpu
def test_instanton_on_the_device(pkg, special, oracle):
    """Uploaded instanton: the device plaquette is the oracle's and follows the
    embedding identity; the download is exact; the Wilson action matches."""
    L = (4, 4, 4, 4)
    U = pkg.Oneinstanton_SUN_embedded(3, *L, block=(1, 3))
    host = special.oneinstanton_sun_embedded(3, L, block=(1, 3))
    assert np.array_equal(U.to_host(), host)
    P2 = _plaquette(special.su2_instanton_links(L), L, 2)
    got = pkg.measure_plaquette(U)
    assert abs(got - (2 * P2 + 1) / 3) <= 1e-13
    assert abs(got - oracle.plaquette(list(L), host) / (6 * 256 * 3)) <= 1e-13
    beta = 6.0
    action = pkg.GaugeAction(U)
    pkg.push_(action, beta / 2, "plaquette")
    v = pkg.md_potential(action, U)
    want = oracle.action(list(L), host, beta)
    assert abs(v - want) <= 1e-13 * abs(want)
