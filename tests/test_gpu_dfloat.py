"""GPU parity of the double-float form (precision "dfloat", GF_DFLOAT): the
Wilson and stout forces, the stout adjoint and the link updates run in
double-float arithmetic (fp32 hi + lo pairs, 48-bit significand) on fp64
links, with the Hamiltonian, Delta H and Metropolis in fp64.

The form has no counterpart in the reference; it is checked against the same
oracle as the plain fp64 form. Tolerances: forces 1e-11 (Frobenius per link,
the stout-force target), Delta H of a trajectory within 1e-8 relative of the
fp64 form on an unthermalised hot start (the MD amplifies per-operation
differences of ~1e-15 by its Lyapunov growth).
"""
import numpy as np
import pytest

from test_gpu_parity import L4, L8, exact_exp_oracle, frob_links, frob_mom  # noqa: F401 (fixture)

pytestmark = pytest.mark.gpu


def _driver(pkg, U, beta, prec, rho=(0.1, 0.1), steps=10, **kw):
    action = pkg.GaugeAction(U)
    pkg.push_(action, beta / 2, "plaquette")
    net = None
    if rho:
        net = pkg.CovNeuralnet(U)
        for r in rho:
            pkg.push_(net, pkg.STOUT_Layer("plaquette", r))
    return pkg.md_driver(U, action, steps=steps, smearing=net, precision=prec, **kw)


def test_dfloat_wilson_force_matches_oracle(pkg, oracle):
    U = pkg.gauge_configuration(L8, start="hot", seed=31)
    Uh = U.to_host()
    P = pkg.gauge_momenta(U)
    pkg.update_momenta_(P, U, 1.0, _driver(pkg, U, 5.7, "dfloat", rho=()))
    assert frob_mom(P.to_host(), oracle.force(list(L8), Uh, 5.7)) < 1e-12


@pytest.mark.parametrize("L", [L4, (8, 4, 4, 8)])
def test_dfloat_stout_force_matches_oracle(pkg, oracle, L):
    """Two stout levels rho = 0.1: forward, adjoint and thin-link force."""
    U = pkg.gauge_configuration(L, start="hot", seed=7)
    Uh = U.to_host()
    P = pkg.gauge_momenta(U)
    pkg.update_momenta_(P, U, 1.0, _driver(pkg, U, 6.0, "dfloat"))
    ref = oracle.stout_force(list(L), Uh, [0.1, 0.1], 6.0)
    assert frob_mom(P.to_host(), ref) < 1e-11


def test_dfloat_stout_force_recompute_matches_store(pkg):
    """Recomputing C in the adjoint gives the stored-C force to 1e-11 per link:
    the two paths form C in different kernels (the forward, and the local
    adjoint's recompute) with fixed-grid products (rms ~2^-43 of the operand
    norms), and are not bitwise equal as in the fp64 form."""
    out = []
    for recompute in (False, True):
        U = pkg.gauge_configuration(L4, start="hot", seed=13)
        P = pkg.gauge_momenta(U)
        pkg.update_momenta_(P, U, 1.0, _driver(pkg, U, 6.0, "dfloat", rho=(0.12, 0.08), recompute=recompute))
        out.append(P.to_host())
    assert frob_mom(out[0], out[1]) < 1e-11


def test_dfloat_stout_backward_matches_oracle(pkg, oracle):
    """gf_stout_backward on a double-float stack: dS/dU from a given dS/dUbar."""
    from gaugefields_gb300 import _lib
    from gaugefields_gb300.api import _StoutStack
    U = pkg.gauge_configuration(L4, start="hot", seed=17)
    Uh = U.to_host()
    rng = np.random.RandomState(5)
    d = rng.randn(*Uh.shape) + 1j * rng.randn(*Uh.shape)
    stack = _StoutStack(U.ctx, [0.1, 0.1], "dfloat")
    _lib.check(_lib.load().gf_stout_forward(U.ctx.h, stack.h, U.field.h, None), U.ctx.h)
    D = pkg.Gaugefields4D(U.ctx, _lib.GF_MAT64)
    D.from_host(d)
    out = pkg.Gaugefields4D(U.ctx, _lib.GF_MAT64)
    _lib.check(_lib.load().gf_stout_backward(U.ctx.h, stack.h, D.field.h, out.field.h), U.ctx.h)
    ref, _ = oracle.stout_backward(list(L4), Uh, [0.1, 0.1], d)
    assert frob_links(out.to_host(), ref) < 1e-11


def test_dfloat_trajectory_matches_oracle(pkg, exact_exp_oracle):
    """4^4 Haar start, one stout level, 5 QPQ steps: Delta H and the final
    links against the oracle at the plain form's tolerances."""
    U = pkg.gauge_configuration(L4, start="hot", seed=7)
    P = pkg.gaussian_momenta(U, seed=1)
    Uh, Ph = U.to_host(), P.to_host()
    drv = _driver(pkg, U, 6.0, "dfloat", rho=(0.1,), steps=5, trajectory_length=0.5, reunitarize=False)
    res = pkg.md_trajectory_(U, P, drv)
    h = exact_exp_oracle.md_trajectory(list(L4), Uh, Ph, 6.0, 0.5, 5, rho=[0.1])
    assert abs(res.delta_hamiltonian - h[2]) <= 1e-10
    assert frob_links(U.to_host(), Uh) < 1e-12


def test_dfloat_delta_h_tracks_fp64(pkg):
    """8^4 Haar start, two stout levels, 20 QPQ steps, same momenta."""
    res = {}
    for prec in ("fp64", "dfloat"):
        U = pkg.gauge_configuration(L8, start="hot", seed=7)
        P = pkg.gaussian_momenta(U, seed=1)
        res[prec] = pkg.md_trajectory_(U, P, _driver(pkg, U, 6.0, prec, steps=20))
    h0 = res["fp64"].initial_hamiltonian
    assert abs(res["dfloat"].initial_hamiltonian - h0) <= 1e-13 * abs(h0)
    d64 = res["fp64"].delta_hamiltonian
    assert abs(res["dfloat"].delta_hamiltonian - d64) <= 1e-8 * max(1.0, abs(d64))


@pytest.mark.parametrize("prec", ["fp64", "mixed", "dfloat"])
def test_custom_integrator_uses_the_driver_precision(pkg, prec):
    """A Python-side QPQ built from update_momenta_/update_gaugefields_ follows
    the native trajectory of the same precision (which merges adjacent half
    steps, so the two differ by rounding only)."""
    U = pkg.gauge_configuration(L4, start="hot", seed=8)
    P = pkg.gaussian_momenta(U, seed=8)
    U2 = U.similar()
    pkg.substitute_U_(U2, U)
    P2 = pkg.gauge_momenta(U)
    P2.from_host(P.to_host())

    def my_qpq(U, P, eps, driver):
        pkg.update_gaugefields_(U, P, eps / 2, driver)
        pkg.update_momenta_(P, U, eps, driver)
        pkg.update_gaugefields_(U, P, eps / 2, driver)

    r1 = pkg.md_trajectory_(U, P, _driver(pkg, U, 5.7, prec, rho=(0.1,), steps=5))
    r2 = pkg.md_trajectory_(U2, P2, _driver(pkg, U2, 5.7, prec, rho=(0.1,), steps=5, integrator=my_qpq))
    tol = 1e-4 if prec == "mixed" else 1e-10
    assert abs(r1.delta_hamiltonian - r2.delta_hamiltonian) < tol
    assert np.abs(U.to_host() - U2.to_host()).max() < (1e-5 if prec == "mixed" else 1e-11)


def test_md_step_entry_points_validate_arguments(pkg):
    """gf_md_mom_update / gf_md_link_update reject what update_momenta! and
    update_gaugefields! reject (ArgumentError), without touching the fields."""
    import ctypes
    from gaugefields_gb300 import _lib
    lib = _lib.load()
    U = pkg.gauge_configuration(L4, start="hot", seed=2)
    P = pkg.gaussian_momenta(U, seed=3)
    U0, P0 = U.to_host(), P.to_host()
    drv = _driver(pkg, U, 6.0, "dfloat", rho=(0.1,))
    prm = drv.params()
    nan = ctypes.c_double(float("nan"))
    assert lib.gf_md_mom_update(U.ctx.h, P.field.h, U.field.h, nan, ctypes.byref(prm)) == _lib.GF_EINVAL
    assert lib.gf_md_link_update(U.ctx.h, U.field.h, P.field.h, nan, ctypes.byref(prm)) == _lib.GF_EINVAL
    # kinds swapped
    assert lib.gf_md_mom_update(U.ctx.h, U.field.h, P.field.h, ctypes.c_double(0.1), ctypes.byref(prm)) == _lib.GF_EINVAL
    bad = drv.params()
    bad.precision = 7
    assert lib.gf_md_link_update(U.ctx.h, U.field.h, P.field.h, ctypes.c_double(0.1), ctypes.byref(bad)) == _lib.GF_EINVAL
    bad = drv.params()
    bad.steps = 0
    assert lib.gf_md_mom_update(U.ctx.h, P.field.h, U.field.h, ctypes.c_double(0.1), ctypes.byref(bad)) == _lib.GF_EINVAL
    assert np.array_equal(U.to_host(), U0) and np.array_equal(P.to_host(), P0)
    with pytest.raises(ValueError):
        pkg.update_momenta_(P, U, float("inf"), drv)


@pytest.mark.parametrize("nlev", [3, 4])
def test_hamiltonian_with_alternating_level_buffers(pkg, nlev):
    """The mixed form's Hamiltonian smears with a forward-only double-float
    stack whose levels beyond the second reuse two buffers in turn; with 3 and
    4 levels it equals the fp64 Hamiltonian to 5e-13 relative (double-float
    smearing with fixed-grid products, rms ~2^-43 relative per product, over 3-4
    levels; a reused buffer holding a wrong level would be off by ~1e-3)."""
    U = pkg.gauge_configuration(L4, start="hot", seed=19)
    P = pkg.gaussian_momenta(U, seed=20)
    rho = (0.1, 0.08, 0.12, 0.1)[:nlev]
    h = {prec: pkg.md_hamiltonian(U, P, _driver(pkg, U, 6.0, prec, rho=rho)) for prec in ("fp64", "mixed", "dfloat")}
    assert abs(h["mixed"] - h["fp64"]) <= 5e-13 * abs(h["fp64"])
    assert abs(h["dfloat"] - h["fp64"]) <= 5e-13 * abs(h["fp64"])


def test_partial_blocks_in_every_form(pkg, oracle, exact_exp_oracle):
    """A 6x4x4x6 lattice (576 sites, not a multiple of the 128-thread blocks):
    the stout force of every form and a double-float trajectory against the
    oracle, so that the idle threads of the last block of each kernel are
    exercised."""
    L = (6, 4, 4, 6)
    U = pkg.gauge_configuration(L, start="hot", seed=23)
    Uh = U.to_host()
    ref = oracle.stout_force(list(L), Uh, [0.1, 0.1], 6.0)
    for prec, tol in (("fp64", 1e-11), ("dfloat", 1e-11), ("mixed", 1e-4)):
        P = pkg.gauge_momenta(U)
        pkg.update_momenta_(P, U, 1.0, _driver(pkg, U, 6.0, prec))
        assert frob_mom(P.to_host(), ref) < tol * max(1.0, np.abs(ref).max()), prec
    P = pkg.gaussian_momenta(U, seed=24)
    Ph = P.to_host()
    res = pkg.md_trajectory_(U, P, _driver(pkg, U, 6.0, "dfloat", rho=(0.1,), steps=3, trajectory_length=0.3,
                                           reunitarize=False))
    h = exact_exp_oracle.md_trajectory(list(L), Uh, Ph, 6.0, 0.3, 3, rho=[0.1])
    assert abs(res.delta_hamiltonian - h[2]) <= 1e-10
    assert frob_links(U.to_host(), Uh) < 1e-12


def test_dfloat_flow_tracks_fp64(pkg, oracle):
    """The RK3 Wilson flow with the force and the exponentials in double-float
    (gf_flow_precision, GF_DFLOAT): 10 steps of eps = 0.02 from an 8^4 Haar
    start equal the fp64 flow's links to 1e-12 and the oracle's to 1e-11;
    the plaquette to 1e-13 relative."""
    U = pkg.gauge_configuration(L8, start="hot", seed=81)
    Uh = U.to_host()
    V = pkg.copy_configuration(U)
    pkg.flow_(U, pkg.Gradientflow(U, Nflow=10, eps=0.02))
    pkg.flow_(V, pkg.Gradientflow(V, Nflow=10, eps=0.02, precision="dfloat"))
    oracle.flow(list(L8), Uh, 0.02, 10)
    a, b = U.to_host(), V.to_host()
    du, do = np.abs(b - a).max(), np.abs(b - Uh).max()
    pa, pb = pkg.calculate_Plaquette(U), pkg.calculate_Plaquette(V)
    print("dfloat flow: |dU| fp64 %.2e oracle %.2e  plaquette rel %.2e" % (du, do, abs(pb - pa) / abs(pa)))
    assert du < 1e-12 and do < 1e-11 and abs(pb - pa) <= 1e-13 * abs(pa)
    with pytest.raises(ValueError):
        pkg.Gradientflow(U, precision="mixed")

