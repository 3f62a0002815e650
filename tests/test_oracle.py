"""Pins of the CPU oracle against the reference's own tests and invariants.

The reference (Gaugefields.jl) is Julia and cannot run here; these checks are
its known answers and invariant tests, restated:
  * test/init.jl:175-211        cold-start plaquette == 1 exactly
  * test/md_driver.jl:269-281   cold start: Delta H == 0, P*P == 0
  * test/md_driver.jl:347-367   reversibility tau then -tau < 2e-12
  * test/md_driver.jl:88-95     force additivity over split actions < 2e-12
  * test/gradientflow_test.jl:136 flowed plaquette 0.8786515255315753 at the
    test's tolerance eps = 1e-1 (runtests.jl:36), from the reference's hot
    start distribution (uniform entries, normalize_U!)
  * test/HMC_test_nowing.jl:459-470 acceptance > 0.5 at 4^4, beta = 5.7
plus the self-checks the survey of the reference lists (finite differences of
the action against the force, O(eps^2) scaling of Delta H, exponential against
scipy, gauge invariance).
"""
import numpy as np
import pytest
from scipy.linalg import expm

L4 = [4, 4, 4, 4]

LAM = np.zeros((8, 3, 3), complex)
LAM[0][0, 1] = LAM[0][1, 0] = 1
LAM[1][0, 1] = -1j
LAM[1][1, 0] = 1j
LAM[2][0, 0] = 1
LAM[2][1, 1] = -1
LAM[3][0, 2] = LAM[3][2, 0] = 1
LAM[4][0, 2] = -1j
LAM[4][2, 0] = 1j
LAM[5][1, 2] = LAM[5][2, 1] = 1
LAM[6][1, 2] = -1j
LAM[6][2, 1] = 1j
LAM[7] = np.diag([1, 1, -2]) / np.sqrt(3)


def test_cold_start_plaquette_is_exactly_one(oracle):
    for L in ([4, 4, 4, 4], [2, 4, 6, 8]):
        U = oracle.cold_start(L)
        assert oracle.plaquette(L, U) / (6 * oracle.vol(L) * 3) == 1.0


def test_cold_start_md_conserves_exactly(oracle):
    U = oracle.cold_start(L4)
    P = oracle.new_mom(L4)
    h = oracle.md_trajectory(L4, U, P, 5.7, 1.0, 10)
    assert h[2] == 0.0
    assert oracle.kinetic(L4, P) == 0.0
    assert oracle.plaquette(L4, U) / (6 * 256 * 3) == pytest.approx(1.0, abs=1e-15)


def test_haar_start_is_special_unitary(oracle):
    U = oracle.mats(oracle.hot_start(L4, 1234))
    M = U.reshape(-1, 3, 3)
    eye = np.eye(3)
    assert np.abs(M @ np.conj(np.swapaxes(M, -1, -2)) - eye).max() < 1e-14
    assert np.abs(np.linalg.det(M) - 1).max() < 1e-14


def test_haar_start_moments(oracle):
    # E|U_ij|^2 = 1/3 and E tr U = 0 for Haar SU(3)
    M = oracle.mats(oracle.hot_start([8, 8, 8, 8], 5)).reshape(-1, 3, 3)
    assert np.mean(np.abs(M) ** 2) == pytest.approx(1 / 3, abs=2e-3)
    tr = np.trace(M, axis1=1, axis2=2)
    assert abs(np.mean(tr)) < 0.02


def test_gaussian_momenta_moments(oracle):
    P = oracle.gauss_mom([8, 8, 8, 8], 1234, 3)
    assert abs(P.mean()) < 5e-3 and P.var() == pytest.approx(1.0, abs=5e-3)
    Q = oracle.gauss_mom([8, 8, 8, 8], 1234, 4)
    assert np.abs(np.corrcoef(P.ravel(), Q.ravel())[0, 1]) < 5e-3


def test_eigen_exponential_matches_expm(oracle):
    rng = np.random.RandomState(0)
    for _ in range(20):
        u = rng.randn(8)
        t = rng.uniform(-1, 1)
        Q = sum(u[a] * LAM[a] / 2 for a in range(8))
        assert np.abs(oracle.expt(t, u) - expm(1j * t * Q)).max() < 1e-13


def test_eigen_exponential_degenerate_branch(oracle):
    # a pure lambda_8 generator has two equal eigenvalues: the reference falls
    # back to its 4th-order Taylor series (exp_T4), which is not exact.
    before = oracle.taylor_fallbacks()
    u = np.zeros(8)
    u[7] = 0.2
    E = oracle.expt(1.0, u)
    assert oracle.taylor_fallbacks() == before + 1
    exact = expm(1j * 0.1 * LAM[7])
    assert 1e-8 < np.abs(E - exact).max() < 1e-5
    # csum == 0 shortcut returns the identity
    u = np.array([1.0, -1.0, 0, 0, 0, 0, 0, 0])
    assert np.array_equal(oracle.expt(0.5, u), np.eye(3))


def _bump(oracle, U, mu, x, a, h):
    M = oracle.mats(U.copy())
    M[mu, x] = expm(1j * h * LAM[a] / 2) @ M[mu, x]
    return oracle.from_mats(M)


@pytest.mark.parametrize("rho", [(), (0.1,), (0.1, 0.1)])
def test_force_is_minus_gradient_of_potential(oracle, rho):
    # central finite differences along su(3) directions (h = 1e-4: O(h^2) ~ 1e-9)
    U = oracle.hot_start(L4, 7)
    beta = 6.0
    F = oracle.stout_force(L4, U, list(rho), beta)
    rng = np.random.RandomState(11)
    h = 1e-4
    for _ in range(4):
        mu, x, a = rng.randint(4), rng.randint(256), rng.randint(8)
        vp = oracle.stout_action(L4, _bump(oracle, U, mu, x, a, h), list(rho), beta)
        vm = oracle.stout_action(L4, _bump(oracle, U, mu, x, a, -h), list(rho), beta)
        fd = (vp - vm) / (2 * h)
        assert fd == pytest.approx(-F[mu, x, a], rel=1e-6, abs=1e-7)


def test_force_additivity(oracle):
    U = oracle.hot_start(L4, 3)
    F1 = oracle.force(L4, U, 2.0)
    F2 = oracle.force(L4, U, 3.7)
    F = oracle.force(L4, U, 5.7)
    assert np.abs(F1 + F2 - F).max() < 2e-12


@pytest.mark.parametrize("integrator", ["QPQ", "PQP"])
def test_reversibility(oracle, integrator):
    U0 = oracle.hot_start(L4, 1234)
    P0 = oracle.gauss_mom(L4, 99)
    U, P = U0.copy(), P0.copy()
    oracle.md_trajectory(L4, U, P, 5.7, 1.0, 10, integrator)
    oracle.md_trajectory(L4, U, P, 5.7, -1.0, 10, integrator)
    assert np.abs(U - U0).max() < 2e-12
    assert np.abs(P - P0).max() < 2e-12


def test_omelyan_is_reversible_and_second_order(oracle):
    U0 = oracle.hot_start(L4, 1234)
    P0 = oracle.gauss_mom(L4, 99)
    U, P = U0.copy(), P0.copy()
    oracle.md_trajectory(L4, U, P, 5.7, 1.0, 8, "OMELYAN")
    oracle.md_trajectory(L4, U, P, 5.7, -1.0, 8, "OMELYAN")
    assert np.abs(U - U0).max() < 2e-12 and np.abs(P - P0).max() < 2e-12
    dh = []
    for n in (8, 16):
        U, P = U0.copy(), P0.copy()
        dh.append(abs(oracle.md_trajectory(L4, U, P, 5.7, 1.0, n, "OMELYAN")[2]))
    assert dh[0] / dh[1] == pytest.approx(4.0, rel=0.25)


def test_delta_h_scales_as_eps_squared(oracle):
    U0 = oracle.hot_start(L4, 1234)
    P0 = oracle.gauss_mom(L4, 99)
    dh = []
    for n in (10, 20):
        U, P = U0.copy(), P0.copy()
        dh.append(oracle.md_trajectory(L4, U, P, 5.7, 1.0, n)[2])
    assert dh[0] / dh[1] == pytest.approx(4.0, rel=0.1)


def test_stout_delta_h_scales_as_eps_squared(oracle):
    U0 = oracle.hot_start(L4, 7)
    P0 = oracle.gauss_mom(L4, 5)
    dh = []
    for n in (10, 20):
        U, P = U0.copy(), P0.copy()
        dh.append(oracle.md_trajectory(L4, U, P, 6.0, 1.0, n, rho=[0.1, 0.1])[2])
    assert dh[0] / dh[1] == pytest.approx(4.0, rel=0.1)


def test_plaquette_gauge_invariance(oracle):
    U = oracle.hot_start(L4, 21)
    G = oracle.mats(oracle.hot_start(L4, 22))[0]  # one SU(3) per site
    M = oracle.mats(U)
    Mt = np.empty_like(M)
    for mu in range(4):
        nb = np.array([oracle_shift(L4, x, mu) for x in range(256)])
        Mt[mu] = G @ M[mu] @ np.conj(np.swapaxes(G[nb], -1, -2))
    Ut = oracle.from_mats(Mt)
    assert oracle.plaquette(L4, Ut) == pytest.approx(oracle.plaquette(L4, U), rel=1e-13)
    assert oracle.stout_action(L4, Ut, [0.1, 0.1], 6.0) == pytest.approx(oracle.stout_action(L4, U, [0.1, 0.1], 6.0),
                                                                        rel=1e-12)


def test_polyakov_loop_invariants(oracle):
    """calculate_Polyakov_loop: 3 on a cold start (measure_polyakov_loop == 1,
    test/high_level_api.jl:49), gauge invariant, and multiplied by the centre
    element exp(2 pi i / 3) when every time link of one time slice is."""
    L = [4, 4, 4, 6]
    V = 4 * 4 * 4 * 6
    assert oracle.polyakov_loop(L, oracle.cold_start(L)) == 3
    U = oracle.hot_start(L, 23)
    p0 = oracle.polyakov_loop(L, U)
    G = oracle.mats(oracle.hot_start(L, 24))[0]
    M = oracle.mats(U)
    Mt = np.empty_like(M)
    for mu in range(4):
        nb = np.array([oracle_shift(L, x, mu) for x in range(V)])
        Mt[mu] = G @ M[mu] @ np.conj(np.swapaxes(G[nb], -1, -2))
    assert abs(oracle.polyakov_loop(L, oracle.from_mats(Mt)) - p0) < 1e-13
    z = np.exp(2j * np.pi / 3)
    Mz = M.copy()
    t2 = np.arange(V) // 64 == 2  # the time slice t = 2
    Mz[3, t2] *= z
    assert abs(oracle.polyakov_loop(L, oracle.from_mats(Mz)) - z * p0) < 1e-13


def oracle_shift(L, lex, mu):
    x = [lex % L[0], (lex // L[0]) % L[1], (lex // (L[0] * L[1])) % L[2], lex // (L[0] * L[1] * L[2])]
    x[mu] = (x[mu] + 1) % L[mu]
    return x[0] + L[0] * (x[1] + L[1] * (x[2] + L[2] * x[3]))


def test_flow_golden_value_at_reference_tolerance(oracle):
    # gradientflow_test.jl: 4^4 SU(3), hot start (uniform entries + normalize_U!),
    # 100 RK3 steps of eps = 0.01 -> plaquette 0.8786515255315753, tolerance 0.1
    U = oracle.uniform_hot_start(L4, 123)
    oracle.flow(L4, U, 0.01, 100)
    plaq = oracle.plaquette(L4, U) / (6 * 256 * 3)
    assert abs(plaq - 0.8786515255315753) / 0.8786515255315753 < 1e-1


def test_flow_increases_plaquette_monotonically(oracle):
    U = oracle.hot_start(L4, 9)
    last = oracle.plaquette(L4, U)
    for _ in range(5):
        oracle.flow(L4, U, 0.02, 2)
        p = oracle.plaquette(L4, U)
        assert p > last
        last = p


def test_hmc_acceptance_physics_smoke(oracle):
    # HMC_test_nowing.jl: 4^4, beta = 5.7, tau = 1 with 100 MD steps, 10
    # trajectories, acceptance > 0.5
    U = oracle.uniform_hot_start(L4, 123)
    rng = np.random.RandomState(1)
    acc = 0
    for traj in range(10):
        Uold = U.copy()
        P = oracle.gauss_mom(L4, 77, traj)
        h = oracle.md_trajectory(L4, U, P, 5.7, 1.0, 100)
        if rng.uniform() < np.exp(-h[2]):
            acc += 1
        else:
            U[...] = Uold
    assert acc / 10 > 0.5


def test_stout_backward_is_linear_in_the_cotangent(oracle):
    U = oracle.hot_start(L4, 31)
    rng = np.random.RandomState(2)
    d1 = rng.randn(*U.shape) + 1j * rng.randn(*U.shape)
    d2 = rng.randn(*U.shape) + 1j * rng.randn(*U.shape)
    a, _ = oracle.stout_backward(L4, U, [0.1, 0.1], np.ascontiguousarray(d1))
    b, _ = oracle.stout_backward(L4, U, [0.1, 0.1], np.ascontiguousarray(d2))
    c, _ = oracle.stout_backward(L4, U, [0.1, 0.1], np.ascontiguousarray(d1 + 2.5 * d2))
    assert np.abs(a + 2.5 * b - c).max() < 1e-11


def test_stout_dsdrho_matches_finite_difference(oracle):
    # parameter_derivatives: dS/drho of each layer (stout_fast.jl:371-386)
    U = oracle.hot_start(L4, 41)
    beta = 6.0
    rho = [0.1, 0.12]
    Ub = oracle.stout_forward(L4, U, rho)
    dbar = np.empty_like(U)
    for mu in range(4):
        D = oracle.dsdu(L4, Ub, beta, mu)
        dbar[mu] = D
    _, drho = oracle.stout_backward(L4, U, rho, dbar)
    h = 1e-6
    for l in range(2):
        rp = list(rho)
        rm = list(rho)
        rp[l] += h
        rm[l] -= h
        # evaluate = -3 * potential; derivative of Re(evaluate) w.r.t. rho
        fd = (-3 * oracle.stout_action(L4, U, rp, beta) + 3 * oracle.stout_action(L4, U, rm, beta)) / (2 * h)
        assert drho[l] == pytest.approx(fd, rel=1e-6)
