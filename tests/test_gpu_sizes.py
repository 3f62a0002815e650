"""GPU parity at the sizes of the workloads, on non-unitary inputs, and on a
thermalised SU(3) configuration written by the reference.

* 2-level stout (rho = 0.1) Wilson force at 16^4 from the Haar start seed 7,
  in the plain fp64 and double-float forms, against the oracle's stout force
  (the restated back_prop of src/smearing/Abstractsmearing.jl:316-411) to
  1e-11 per link (Frobenius): the per-link force check of the differentiation
  workload at its stated lattice.
* 32^4 Wilson plaquette (1e-13 relative) and force (1e-12 per link) against
  the oracle: the plain fp64 workload at scale.
* gf_reunitarize (normalize3!, src/AbstractGaugefields.jl:3378-3457) on
  matrices that are not unitary, against the oracle's restatement.
* gaussian_momenta_ with sigma != 1 (gf_mom_scale).
* The reference's thermalised 8^4 SU(3) configuration
  (samples/measurements/conf_08080808.ildg, generated at beta = 5.7, as its
  docs/src/legacyapi.md:219-240 loads it): plaquette, Wilson force, stout
  force and one QPQ trajectory against the oracle. The file is read in place
  from the path in GF_REFERENCE_CONF (the test skips without it); it is not
  part of this repository.
* dS/drho of each stout level on the device (gf_stout_param_derivatives)
  against the oracle's parameter_derivatives and against central differences
  of the device potential.
* The smallest lattices the layout takes (extents of 2, fewer sites than a
  block): plaquette, rectangle sum, Wilson, stout and rectangle forces and a
  stout trajectory against the oracle.
"""
import os

import numpy as np
import pytest

from test_gpu_parity import exact_exp_oracle, frob_links, frob_mom  # noqa: F401 (fixture)

pytestmark = pytest.mark.gpu

L16 = (16, 16, 16, 16)
L32 = (32, 32, 32, 32)


def _stout_driver(pkg, U, prec, beta=6.0, rho=(0.1, 0.1), steps=1, **kw):
    action = pkg.GaugeAction(U)
    pkg.push_(action, beta / 2, "plaquette")
    net = pkg.CovNeuralnet(U)
    for r in rho:
        pkg.push_(net, pkg.STOUT_Layer("plaquette", r))
    return pkg.md_driver(U, action, steps=steps, smearing=net, precision=prec, **kw)


@pytest.fixture(scope="module")
def stout16_reference(pkg, oracle):
    """Haar start seed 7 at 16^4 and the oracle's 2-level stout force on it."""
    U = pkg.gauge_configuration(L16, start="hot", seed=7)
    Uh = U.to_host()
    return Uh, oracle.stout_force(list(L16), Uh, [0.1, 0.1], 6.0)


def _rel_frob_mom(A, B):
    """max over links of |A - B| / max(1, |B|) (Frobenius norms of the 8 coefficients)."""
    d = np.sqrt(((A - B) ** 2).sum(-1))
    return (d / np.maximum(1.0, np.sqrt((B ** 2).sum(-1)))).max()


def test_stout_force_16x4_haar_seed7(pkg, stout16_reference):
    """The 2-level stout force at 16^4 in the plain fp64 and the double-float
    forms against the oracle, per link to 1e-11 relative to the link's force
    (|F| is 1-6 here). The two device forms, with different arithmetic, agree
    with each other to 1e-11 absolute (9e-12 measured), and deviate alike
    from the oracle (1.7e-11 absolute on the worst of the 262,144 links): the
    oracle follows the reference's closed-form exponential coefficients
    (calc_coefficients_Q), which lose digits where the eigenvalues of Q nearly
    coincide, while the device sums the coefficients' power series."""
    Uh, ref = stout16_reference
    got = {}
    for prec in ("fp64", "dfloat"):
        U = pkg.gauge_configuration(L16, start="cold")
        U.from_host(Uh)
        P = pkg.gauge_momenta(U)
        pkg.update_momenta_(P, U, 1.0, _stout_driver(pkg, U, prec))
        got[prec] = P.to_host()
        assert _rel_frob_mom(got[prec], ref) < 1e-11, prec
    assert frob_mom(got["dfloat"], got["fp64"]) < 1e-11


def test_wilson_plaquette_and_force_32x4(pkg, oracle):
    U = pkg.gauge_configuration(L32, start="hot", seed=1234)
    Uh = U.to_host()
    ref = oracle.plaquette(list(L32), Uh)
    got = pkg.calculate_Plaquette(U)
    assert abs(got - ref) <= 1e-13 * abs(ref)
    action = pkg.GaugeAction(U)
    pkg.push_(action, 3.0, "plaquette")
    F = pkg.gauge_momenta(U)
    pkg.md_force_(F, action, U)
    assert frob_mom(F.to_host(), oracle.force(list(L32), Uh, 6.0)) < 1e-12


def test_reunitarize_non_unitary_links(pkg, oracle):
    """Haar links with 5% complex Gaussian noise added, and plain complex
    Gaussian matrices: the GPU's Gram-Schmidt of rows 1-2 with row 3 the
    conjugate cross product equals the oracle's normalize3! to 1e-12 per
    link, and the result is unitary with det 1."""
    L = (4, 4, 4, 8)
    V = int(np.prod(L))
    U = pkg.gauge_configuration(L, start="hot", seed=3)
    rng = np.random.RandomState(42)
    noise = rng.randn(4, V, 3, 3) + 1j * rng.randn(4, V, 3, 3)
    A = U.to_host() + 0.05 * noise
    A[2:] = rng.randn(2, V, 3, 3) + 1j * rng.randn(2, V, 3, 3)
    A = np.ascontiguousarray(A)
    ref = A.copy()
    oracle.normalize(list(L), ref)
    U.from_host(A)
    pkg.normalize_U_(U)
    got = U.to_host()
    assert frob_links(got, A) > 0.1  # the input was far from unitary
    assert frob_links(got, ref) < 1e-12
    m = np.swapaxes(got, -1, -2)
    assert np.abs(m @ np.conj(np.swapaxes(m, -1, -2)) - np.eye(3)).max() < 1e-14
    assert np.abs(np.linalg.det(m) - 1).max() < 1e-14


def test_gaussian_momenta_sigma_scales_the_draws(pkg):
    """gaussian_momenta_ with sigma = 0.5 gives 0.5 x the sigma = 1 draws of
    the same (seed, sweep), elementwise, so P.P scales by 0.25."""
    U = pkg.gauge_configuration((8, 8, 8, 8), start="cold")
    P1 = pkg.gaussian_momenta(U, sigma=1.0, seed=77, sweep=4)
    P2 = pkg.gaussian_momenta(U, sigma=0.5, seed=77, sweep=4)
    a, b = P1.to_host(), P2.to_host()
    assert np.array_equal(b, 0.5 * a)
    k1, k2 = P1 * P1, P2 * P2
    assert abs(k2 - 0.25 * k1) <= 1e-14 * k1


def _reference_conf():
    path = os.environ.get("GF_REFERENCE_CONF")
    if not path or not os.path.exists(path):
        pytest.skip("GF_REFERENCE_CONF (the reference's conf_08080808.ildg) not given")
    from gaugefields_gb300 import ildg
    links, head = ildg.read(path, L=[8, 8, 8, 8], NC=3)
    assert head["precision"] == 64
    return np.ascontiguousarray(links)


def test_reference_thermalised_configuration(pkg, exact_exp_oracle):
    """The reference's thermalised 8^4 SU(3) configuration (beta = 5.7):
    plaquette and action 1e-13 relative, Wilson force 1e-12 and 2-level stout
    force 1e-11 per link, and one QPQ trajectory (beta = 5.7, tau = 1, 10
    steps, Gaussian momenta seed 1234) with Delta H to 1e-10 and links to 1e-12
    against the oracle."""
    O = exact_exp_oracle
    L = (8, 8, 8, 8)
    Uh = _reference_conf()
    U = pkg.gauge_configuration(L, start="cold")
    U.from_host(Uh)
    ref = O.plaquette(list(L), Uh)
    assert 0.55 < ref / (6 * 8 ** 4 * 3) < 0.56  # thermalised at beta = 5.7
    assert abs(pkg.calculate_Plaquette(U) - ref) <= 1e-13 * abs(ref)
    action = pkg.GaugeAction(U)
    pkg.push_(action, 2.85, "plaquette")
    assert abs(pkg.md_potential(action, U) - O.action(list(L), Uh, 5.7)) <= 1e-13 * abs(O.action(list(L), Uh, 5.7))
    F = pkg.gauge_momenta(U)
    pkg.md_force_(F, action, U)
    assert frob_mom(F.to_host(), O.force(list(L), Uh, 5.7)) < 1e-12
    Ps = pkg.gauge_momenta(U)
    pkg.update_momenta_(Ps, U, 1.0, _stout_driver(pkg, U, "fp64", beta=5.7))
    assert frob_mom(Ps.to_host(), O.stout_force(list(L), Uh, [0.1, 0.1], 5.7)) < 1e-11
    P = pkg.gaussian_momenta(U, seed=1234, sweep=0)
    Ph = P.to_host()
    drv = pkg.md_driver(U, action, steps=10, trajectory_length=1.0, reunitarize=False)
    res = pkg.md_trajectory_(U, P, drv)
    Uo = Uh.copy()
    h = O.md_trajectory(list(L), Uo, Ph, 5.7, 1.0, 10, "QPQ")
    assert abs(res.delta_hamiltonian - h[2]) <= 1e-10
    assert abs(res.delta_hamiltonian) < 5.0  # a thermalised start: Delta H is O(1)
    assert frob_links(U.to_host(), Uo) < 1e-12


@pytest.mark.parametrize("prec", ["mixed", "dfloat"])
def test_reference_thermalised_configuration_precision_forms(pkg, prec):
    """One 2-level stout trajectory (beta = 5.7, tau = 1, 20 QPQ steps) from
    the reference's thermalised configuration in each fast form against the
    plain fp64 form with the same momenta. The double-float form (the
    benchmark's headline) meets |Delta H_form - Delta H_fp64| <= 1e-4 with a
    wide margin (asserted: 1e-7). The mixed form (fp32 force) does not: on
    this configuration, which is thermalised for the unsmeared action, so
    Delta H is -27.9 on the smeared one, it moves Delta H by 5.2e-4; the
    assertion records that scale (<= 2e-3) as a regression bound only."""
    Uh = _reference_conf()
    L = (8, 8, 8, 8)
    dh = {}
    for p in ("fp64", prec):
        U = pkg.gauge_configuration(L, start="cold")
        U.from_host(Uh)
        P = pkg.gaussian_momenta(U, seed=1234, sweep=1)
        dh[p] = pkg.md_trajectory_(U, P, _stout_driver(pkg, U, p, beta=5.7, steps=20)).delta_hamiltonian
    tol = 2e-3 if prec == "mixed" else 1e-7
    assert abs(dh[prec] - dh["fp64"]) <= tol, dh


def _dsdrho_inputs(pkg, oracle, L, seed, rho, beta=6.0):
    """Haar links and dS/dUbar = dS/dU of the Wilson action on the smeared links
    (the cotangent of parameter_derivatives in a stout-HMC force)."""
    U = pkg.gauge_configuration(L, start="hot", seed=seed)
    Uh = U.to_host()
    Ub = oracle.stout_forward(list(L), Uh, rho)
    dbar = np.empty_like(Uh)
    for mu in range(4):
        dbar[mu] = oracle.dsdu(list(L), Ub, beta, mu)
    _, drho = oracle.stout_backward(list(L), Uh, rho, dbar)
    return U, Uh, np.ascontiguousarray(dbar), drho


@pytest.mark.parametrize("prec,rtol", [("fp64", 1e-11), ("dfloat", 1e-11), ("mixed", 1e-4)])
@pytest.mark.parametrize("L", [(4, 4, 4, 4), (8, 4, 4, 8)])
def test_stout_dsdrho_matches_oracle(pkg, oracle, prec, rtol, L):
    """dS/drho of each of two stout levels (rho = 0.1, 0.12) on the device
    (gf_stout_param_derivatives) against the oracle's restatement of
    parameter_derivatives (stout_fast.jl:371-386)."""
    from gaugefields_gb300 import _lib
    rho = [0.1, 0.12]
    U, Uh, dbar, ref = _dsdrho_inputs(pkg, oracle, L, 41, rho)
    net = pkg.CovNeuralnet(U)
    for r in rho:
        pkg.push_(net, pkg.STOUT_Layer("plaquette", r))
    D = pkg.Gaugefields4D(U.ctx, _lib.GF_MAT64)
    D.from_host(dbar)
    got = pkg.get_parameter_derivatives(D, net, U, precision=prec)
    for l in range(2):
        assert abs(got[l] - ref[l]) <= rtol * abs(ref[l]), (l, got, ref)


def test_stout_dsdrho_matches_finite_differences_of_the_device_potential(pkg, oracle):
    """dS/drho against central differences (h = 1e-6) of the device's smeared
    Wilson potential V: with dS/dUbar = dS/dU of beta/2 (plaq U plaq^dag), the
    derivative is that of Re evaluate_GaugeAction = -3 V."""
    from gaugefields_gb300 import _lib
    L = (4, 4, 4, 4)
    rho = [0.1, 0.12]
    U, Uh, dbar, _ = _dsdrho_inputs(pkg, oracle, L, 43, rho)
    net = pkg.CovNeuralnet(U)
    for r in rho:
        pkg.push_(net, pkg.STOUT_Layer("plaquette", r))
    D = pkg.Gaugefields4D(U.ctx, _lib.GF_MAT64)
    D.from_host(dbar)
    got = pkg.get_parameter_derivatives(D, net, U)
    zero = pkg.gauge_momenta(U)
    h = 1e-6
    for l in range(2):
        vals = []
        for sgn in (+1, -1):
            r = list(rho)
            r[l] += sgn * h
            action = pkg.GaugeAction(U)
            pkg.push_(action, 3.0, "plaquette")
            n = pkg.CovNeuralnet(U)
            for x in r:
                pkg.push_(n, pkg.STOUT_Layer("plaquette", x))
            vals.append(pkg.md_hamiltonian(U, zero, pkg.md_driver(U, action, steps=1, smearing=n)))
        fd = -3.0 * (vals[0] - vals[1]) / (2 * h)
        assert abs(got[l] - fd) <= 1e-6 * abs(fd), (l, got[l], fd)


@pytest.mark.parametrize("L", [(2, 4, 2, 6), (2, 2, 2, 2)])
def test_minimal_extents(pkg, oracle, exact_exp_oracle, L):
    """Lattices with extent 2 (x + mu and x - mu are the same site; x + 2 mu
    is x itself) and a partial block (96 or 16 sites): plaquette, rectangle
    sum, Wilson force, the 2-level stout force in the fp64 and double-float
    forms, the plaquette + rectangle force and one fp64 stout trajectory
    against the oracle."""
    U = pkg.gauge_configuration(L, start="hot", seed=61)
    Uh = U.to_host()
    ref = oracle.plaquette(list(L), Uh)
    assert abs(pkg.calculate_Plaquette(U) - ref) <= 1e-13 * abs(ref)
    rref = oracle.rectangle_sum(list(L), Uh)
    assert abs(pkg.rectangle_sum(U) - rref) <= 1e-13 * abs(rref)
    action = pkg.GaugeAction(U)
    pkg.push_(action, 2.85, "plaquette")
    F = pkg.gauge_momenta(U)
    pkg.md_force_(F, action, U)
    assert frob_mom(F.to_host(), oracle.force(list(L), Uh, 5.7)) < 1e-12
    sref = oracle.stout_force(list(L), Uh, [0.1, 0.1], 6.0)
    for prec in ("fp64", "dfloat"):
        P = pkg.gauge_momenta(U)
        pkg.update_momenta_(P, U, 1.0, _stout_driver(pkg, U, prec))
        assert frob_mom(P.to_host(), sref) < 1e-11 * max(1.0, np.abs(sref).max()), prec
    iwa = pkg.GaugeAction(U)
    pkg.push_(iwa, 4.2, "plaquette")
    pkg.push_(iwa, -0.38, "rectangular")
    for prec in ("fp64", "dfloat"):
        P = pkg.gauge_momenta(U)
        pkg.update_momenta_(P, U, 1.0, pkg.md_driver(U, iwa, steps=1, precision=prec))
        assert np.abs(P.to_host() - oracle.force_loops(list(L), Uh, 4.2, -0.38)).max() < 1e-11, prec
    P = pkg.gaussian_momenta(U, seed=62)
    Ph = P.to_host()
    res = pkg.md_trajectory_(U, P, _stout_driver(pkg, U, "fp64", steps=4, trajectory_length=0.4,
                                                 reunitarize=False))
    h = exact_exp_oracle.md_trajectory(list(L), Uh, Ph, 6.0, 0.4, 4, rho=[0.1, 0.1])
    assert abs(res.delta_hamiltonian - h[2]) <= 1e-10
    assert frob_links(U.to_host(), Uh) < 1e-12
