"""Rectangle loops in the gauge action (push!(action, c, rect U rect'),
make_loops_fromname("rectangular"); src/action/GaugeActions.jl,
src/autostaples/wilsonloops.jl:304-330), e.g. the Iwasaki action
beta (c0 plaq + c1 rect) with c1 = -0.331, c0 = 1 - 8 c1.

The oracle builds the staples of any loop set by the rule of Wilsonloop's
make_staple (each forward occurrence of U_mu contributes the rest of its
loop); the CPU tests pin that rule on the plaquettes against the oracle's own
Wilson force, and the rectangle force against finite differences of the
rectangle potential. The GPU tests compare the fused fp64 kernels of
gf_rect.cu with the oracle, and the double-float force (the GF_DFLOAT form)
with the oracle and with the plain form's trajectories."""
import numpy as np
import pytest
from scipy.linalg import expm

from test_md_timescales import BETA, L4, _HostLinks, _HostMomenta, _fake_library, _split_actions  # noqa: F401
from test_oracle import LAM

C1 = -0.331
C0 = 1 - 8 * C1
B_IWA = 2.3
CP, CR = 0.5 * B_IWA * C0, 0.5 * B_IWA * C1      # push! coefficients of plaq U plaq' and rect U rect'
L6 = (6, 4, 4, 6)                                 # 576 sites: a partial last block of 128


def _bump(oracle, U, mu, x, a, h):
    M = oracle.mats(U.copy())
    M[mu, x] = expm(1j * h * LAM[a] / 2) @ M[mu, x]
    return oracle.from_mats(M)


def test_loop_sets_and_staple_counts(oracle):
    assert [oracle.loop_staple_count(0, mu) for mu in range(4)] == [6] * 4
    assert [oracle.loop_staple_count(1, mu) for mu in range(4)] == [18] * 4
    U = oracle.hot_start(list(L4), 3)
    # the general rule on the plaquette set is the Wilson action and force
    assert np.abs(oracle.force_loops(list(L4), U, 2.85, 0.0) - oracle.force(list(L4), U, 5.7)).max() < 1e-14
    assert oracle.action_loops(list(L4), U, 2.85, 0.0) == pytest.approx(oracle.action(list(L4), U, 5.7), rel=1e-14)
    assert 0.5 * oracle.loop_trace(list(L4), U, 0) == pytest.approx(oracle.plaquette(list(L4), U), rel=1e-14)
    C = oracle.cold_start(list(L4))
    assert oracle.rectangle_sum(list(L4), C) == 36 * 256
    assert oracle.action_loops(list(L4), C, CP, CR) == pytest.approx(-(2 / 3) * (CP * 18 + CR * 36) * 256, rel=1e-15)


@pytest.mark.parametrize("coefs", [(CP, CR), (0.0, 1.7)])
def test_rectangle_force_is_minus_gradient_of_potential(oracle, coefs):
    U = oracle.hot_start(list(L4), 7)
    F = oracle.force_loops(list(L4), U, *coefs)
    rng = np.random.RandomState(5)
    h = 1e-4
    for _ in range(6):
        mu, x, a = rng.randint(4), rng.randint(256), rng.randint(8)
        vp = oracle.action_loops(list(L4), _bump(oracle, U, mu, x, a, h), *coefs)
        vm = oracle.action_loops(list(L4), _bump(oracle, U, mu, x, a, -h), *coefs)
        assert (vp - vm) / (2 * h) == pytest.approx(-F[mu, x, a], rel=1e-6, abs=1e-7)


def test_smeared_rectangle_force_is_minus_gradient_of_the_smeared_potential(oracle):
    """Two stout levels (rho = 0.1) under the plaquette + rectangle action:
    the loop-set dS/dUbar on the top level, back-propagated by the stout
    adjoint, is minus the gradient of the smeared action (central
    differences); with c_rect = 0 it is the smeared Wilson force."""
    U = oracle.hot_start(list(L4), 8)
    rho = (0.1, 0.1)
    F0 = oracle.stout_force_loops(list(L4), U, rho, 2.85, 0.0)
    assert np.abs(F0 - oracle.stout_force(list(L4), U, rho, 5.7)).max() < 1e-13
    assert oracle.stout_action_loops(list(L4), U, rho, 2.85, 0.0) == pytest.approx(
        oracle.stout_action(list(L4), U, rho, 5.7), rel=1e-14)
    F = oracle.stout_force_loops(list(L4), U, rho, CP, CR)
    rng = np.random.RandomState(6)
    h = 1e-4
    for _ in range(6):
        mu, x, a = rng.randint(4), rng.randint(256), rng.randint(8)
        vp = oracle.stout_action_loops(list(L4), _bump(oracle, U, mu, x, a, h), rho, CP, CR)
        vm = oracle.stout_action_loops(list(L4), _bump(oracle, U, mu, x, a, -h), rho, CP, CR)
        assert (vp - vm) / (2 * h) == pytest.approx(-F[mu, x, a], rel=1e-6, abs=1e-7)


def test_smeared_iwasaki_md_is_reversible(oracle):
    U0, P0 = oracle.hot_start(list(L4), 1235), oracle.gauss_mom(list(L4), 98)
    U, P = U0.copy(), P0.copy()
    h = oracle.md_trajectory(list(L4), U, P, B_IWA * C0, 0.3, 6, "QPQ", rho=(0.1,), c_rect=CR)
    oracle.md_trajectory(list(L4), U, P, B_IWA * C0, -0.3, 6, "QPQ", rho=(0.1,), c_rect=CR)
    assert np.abs(U - U0).max() < 2e-12 and np.abs(P - P0).max() < 2e-12
    assert h[0] == pytest.approx(oracle.stout_action_loops(list(L4), U0, (0.1,), CP, CR)
                                 + oracle.kinetic(list(L4), P0) / 2, rel=1e-14)


def _rect_table():
    """The double-float rectangle kernel's product table (c_rect_ops of
    gf_rect.cu), parsed from the source."""
    import os
    import re
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "gaugefields.jl_gb300",
                            "csrc", "gf_rect.cu")).read()
    block = src[src.index("__constant__ DfOpR c_rect_ops[28]"):]
    block = block[:block.index("};")]
    ops = [tuple(int(v) for v in m.group(1).split(","))
           for m in re.finditer(r"\{(-?\d+(?:,\s*-?\d+){11})\}", block)]
    assert len(ops) == 28
    return ops


def test_double_float_rectangle_table_builds_the_loop_staples(oracle):
    """The table of k_force_rect_df (28 products per plane: the two
    plaquette staples into S, the six rectangle staples into R), run on the
    host in complex128 with its own operand rules (link of direction mu or nu
    at x + mo mu + no nu, optionally daggered, or the running product t),
    gives cp S + cr R equal to the oracle's loop-set dS/dU to 1e-13: the
    table holds exactly the rectangles of make_rect and the plaquette staples."""
    L = list(L4)
    U = oracle.hot_start(L, 9)
    M = oracle.mats(U)
    ref = oracle.mats(oracle.dsdu_loops(L, U, CP, CR))
    ops = _rect_table()
    V = int(np.prod(L))

    def site(x, mu, a, nu, b):
        c = [x % L[0], (x // L[0]) % L[1], (x // (L[0] * L[1])) % L[2], x // (L[0] * L[1] * L[2])]
        c[mu] = (c[mu] + a) % L[mu]
        c[nu] = (c[nu] + b) % L[nu]
        return c[0] + L[0] * (c[1] + L[1] * (c[2] + L[2] * c[3]))

    worst = 0.0
    for mu in range(4):
        for x in range(0, V, 7):
            slots = [np.zeros((3, 3), complex) for _ in range(3)]
            for k in range(1, 4):
                nu = (mu + k) % 4

                def operand(src, d, mo, no, dag):
                    m = slots[0] if src == 1 else M[nu if d else mu, site(x, mu, mo, nu, no)]
                    return m.conj().T if dag else m

                for op in ops:
                    a = operand(*op[0:5])
                    b = operand(*op[5:10])
                    r = a @ b
                    slots[op[10]] = (slots[op[10]] + r) if op[11] else r
            T = CP * slots[1] + CR * slots[2]
            worst = max(worst, np.abs(T - ref[mu, x]).max())
    assert worst < 1e-13


def test_rectangle_sum_is_gauge_invariant(oracle):
    from test_oracle import oracle_shift
    U = oracle.hot_start(list(L4), 21)
    G = oracle.mats(oracle.hot_start(list(L4), 22))[0]
    M = oracle.mats(U)
    Mt = np.empty_like(M)
    for mu in range(4):
        nb = np.array([oracle_shift(list(L4), x, mu) for x in range(256)])
        Mt[mu] = G @ M[mu] @ np.conj(np.swapaxes(G[nb], -1, -2))
    assert oracle.rectangle_sum(list(L4), oracle.from_mats(Mt)) == pytest.approx(oracle.rectangle_sum(list(L4), U),
                                                                                 rel=1e-13)


@pytest.mark.parametrize("integrator", ["QPQ", "PQP"])
def test_iwasaki_md_is_reversible_and_second_order(oracle, integrator):
    U0, P0 = oracle.hot_start(list(L4), 1234), oracle.gauss_mom(list(L4), 99)
    U, P = U0.copy(), P0.copy()
    oracle.md_trajectory(list(L4), U, P, B_IWA * C0, 0.5, 10, integrator, c_rect=CR)
    oracle.md_trajectory(list(L4), U, P, B_IWA * C0, -0.5, 10, integrator, c_rect=CR)
    assert np.abs(U - U0).max() < 2e-12 and np.abs(P - P0).max() < 2e-12
    dh = []
    for n in (10, 20):
        U, P = U0.copy(), P0.copy()
        dh.append(oracle.md_trajectory(list(L4), U, P, B_IWA * C0, 0.5, n, integrator, c_rect=CR)[2])
    assert dh[0] / dh[1] == pytest.approx(4.0, rel=0.15)


def test_action_api_with_rectangles(pkg):
    a = pkg.GaugeAction(None)
    pkg.push_(a, CP, ("plaquette", "plaquette_dag"))
    pkg.push_(a, CR, "rectangular")
    assert a.beta == pytest.approx(2 * CP) and a.c_rect == pytest.approx(CR)
    with pytest.raises(ValueError):
        pkg.push_(a, 1.0, "chair")
    U = [None] * 4
    drv = pkg.md_driver(U, a, steps=4)
    p = drv.params()
    assert p.beta == pytest.approx(2 * CP) and p.c_rect == pytest.approx(CR)
    net = pkg.CovNeuralnet()
    pkg.push_(net, pkg.STOUT_Layer("plaquette", 0.1))
    for prec in ("mixed", "dfloat"):
        for sm in (None, net):
            p = pkg.md_driver(U, a, steps=4, precision=prec, smearing=sm).params()
            assert p.c_rect == pytest.approx(CR) and p.nstout == (0 if sm is None else 1)


def test_sexton_weingarten_with_a_rectangle_member(md, oracle):
    """Plaquette member on the fast scale, rectangle member on the slow one:
    the group kicks carry their own coefficients; reversible to 3e-12."""
    p, log = md
    api = p.api
    fast, slow = api.GaugeAction(None), api.GaugeAction(None)
    api.push_(fast, CP, "plaquette")
    api.push_(slow, CR, "rectangular")
    actions = api.MDActionSet(fast=fast, slow=slow)
    sw = api.SextonWeingarten(slow="slow", fast="fast", n_fast=2)
    Uh, Ph = oracle.hot_start(list(L4), 5), oracle.gauss_mom(list(L4), 6)
    U0, P0 = Uh.copy(), Ph.copy()
    U, P = _HostLinks(L4, Uh), _HostMomenta(L4, Ph)
    api.md_trajectory_(U, P, api.md_driver(U, actions, steps=2, trajectory_length=0.2, integrator=sw),
                       diagnostics=False)
    kicks = {(e[2], e[3]) for e in log if e[0] == "P"}
    assert kicks == {(2.0 * CP, 0.0), (0.0, CR)}
    api.md_trajectory_(U, P, api.md_driver(U, actions, steps=2, trajectory_length=-0.2, integrator=sw),
                       diagnostics=False)
    assert np.abs(U.U - U0).max() < 3e-12 and np.abs(P.P - P0).max() < 3e-12


@pytest.fixture
def md(monkeypatch, oracle):
    import __graft_entry__ as entry
    from types import SimpleNamespace
    pkg = entry.load_package()
    import gaugefields_gb300.api as api
    log = []
    monkeypatch.setattr(api, "call", _fake_library(oracle, log))
    return SimpleNamespace(pkg=pkg, api=api), log


# ---------------------------------------------------------------------------
# device
# ---------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("L", [(8, 8, 8, 8), L6])
def test_rectangle_sum_action_and_force_match_the_oracle(pkg, oracle, L):
    U = pkg.gauge_configuration(L, start="hot", seed=31)
    Uh = U.to_host()
    ref = oracle.rectangle_sum(list(L), Uh)
    assert abs(pkg.rectangle_sum(U) - ref) <= 1e-13 * abs(ref)
    a = pkg.GaugeAction(U)
    pkg.push_(a, CP, "plaquette")
    pkg.push_(a, CR, "rectangular")
    v = pkg.md_potential(a, U)
    vr = oracle.action_loops(list(L), Uh, CP, CR)
    assert abs(v - vr) <= 1e-13 * abs(vr)
    e = pkg.evaluate_GaugeAction(a, U)
    assert abs(e + 3 * vr) <= 1e-13 * abs(vr)
    F = pkg.gauge_momenta(U)
    pkg.md_force_(F, a, U)
    dF = np.abs(F.to_host() - oracle.force_loops(list(L), Uh, CP, CR)).max()
    print("rectangle %s: sum rel %.2e  action rel %.2e  |dF| %.2e"
          % (L, abs(pkg.rectangle_sum(U) - ref) / abs(ref), abs(v - vr) / abs(vr), dF))
    assert dF < 1e-12
    # cold start: every rectangle has trace 3
    C = pkg.gauge_configuration(L, start="cold")
    assert pkg.rectangle_sum(C) == 36 * int(np.prod(L))


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", ["QPQ", "PQP"])
def test_iwasaki_trajectory_matches_the_oracle(pkg, oracle, integrator):
    """8^4 Haar start, Iwasaki beta = 2.3, tau = 0.5, 10 steps: Delta H to
    1e-10, links and momenta to 1e-12 against the oracle with a
    full-double-precision exponential."""
    U = pkg.gauge_configuration((8, 8, 8, 8), start="hot", seed=41)
    P = pkg.gaussian_momenta(U, seed=42)
    Uh, Ph = U.to_host(), P.to_host()
    a = pkg.GaugeAction(U)
    pkg.push_(a, CP, "plaquette")
    pkg.push_(a, CR, "rectangular")
    integ = pkg.QPQ() if integrator == "QPQ" else pkg.PQP()
    drv = pkg.md_driver(U, a, steps=10, trajectory_length=0.5, integrator=integ, reunitarize=False)
    res = pkg.md_trajectory_(U, P, drv)
    oracle.set_exp_method("taylor")
    try:
        h = oracle.md_trajectory([8, 8, 8, 8], Uh, Ph, 2 * CP, 0.5, 10, integrator, c_rect=CR)
    finally:
        oracle.set_exp_method("eigen")
    du, dp = np.abs(U.to_host() - Uh).max(), np.abs(P.to_host() - Ph).max()
    print("iwasaki %s: dH %.6e oracle %.6e  |dU| %.2e |dP| %.2e" % (integrator, res.delta_hamiltonian, h[2], du, dp))
    assert abs(res.initial_hamiltonian - h[0]) <= 1e-13 * abs(h[0])
    assert abs(res.delta_hamiltonian - h[2]) <= 1e-10
    assert du < 1e-12 and dp < 1e-12


def _dfloat_force(pkg, U, a, eps):
    """P = eps F(U) through gf_md_mom_update in the double-float form."""
    from gaugefields_gb300 import _lib
    import ctypes
    P = pkg.gauge_momenta(U)
    p = pkg.md_driver(U, a, steps=2, precision="dfloat").params()
    _lib.call("gf_md_mom_update", U.ctx.h, P.field.h, U.field.h, ctypes.c_double(eps), ctypes.byref(p), ctx=U.ctx.h)
    return P.to_host()


@pytest.mark.gpu
@pytest.mark.parametrize("L", [(8, 8, 8, 8), L6])
def test_dfloat_rectangle_force_matches_the_oracle(pkg, oracle, L):
    """The double-float plaquette + rectangle force (k_force_rect_df): 84
    fixed-grid products per link, each carrying rms ~2^-43 (1.2e-13) of its
    operands' norms through chains of four products and 24 staples weighted
    by c_plaq = 4.2, c_rect = -0.38; the force (|F| ~ 10 at beta = 2.3 on a
    Haar start) agrees with the fp64 oracle to 1e-12 of max |F| (measured
    3.6e-13). A momentum step with eps = -0.5 adds -0.5 F to the zero momenta
    (keep = 1 path)."""
    U = pkg.gauge_configuration(L, start="hot", seed=33)
    Uh = U.to_host()
    a = pkg.GaugeAction(U)
    pkg.push_(a, CP, "plaquette")
    pkg.push_(a, CR, "rectangular")
    ref = oracle.force_loops(list(L), Uh, CP, CR)
    F = _dfloat_force(pkg, U, a, 1.0)
    dF = np.abs(F - ref).max()
    Fh = _dfloat_force(pkg, U, a, -0.5)
    dFh = np.abs(Fh + 0.5 * ref).max()
    print("dfloat rectangle %s: |F| %.3f  |dF| %.2e  half step %.2e" % (L, np.abs(ref).max(), dF, dFh))
    fmax = np.abs(ref).max()
    assert dF < 1e-12 * fmax and dFh < 0.5e-12 * fmax


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", ["QPQ", "PQP"])
def test_dfloat_iwasaki_trajectory_tracks_the_plain_form(pkg, integrator):
    """8^4 Haar start, Iwasaki beta = 2.3, tau = 0.5, 10 steps: the
    double-float form (rectangle force and link updates in double-float)
    against the plain fp64 form from the same start: Delta H to 1e-9 (the
    form's bound is 1e-4), links and momenta to 1e-11."""
    U = pkg.gauge_configuration((8, 8, 8, 8), start="hot", seed=43)
    P = pkg.gaussian_momenta(U, seed=44)
    Uh, Ph = U.to_host(), P.to_host()
    res = {}
    for prec in ("fp64", "dfloat"):
        U.from_host(Uh)
        P.from_host(Ph)
        a = pkg.GaugeAction(U)
        pkg.push_(a, CP, "plaquette")
        pkg.push_(a, CR, "rectangular")
        integ = pkg.QPQ() if integrator == "QPQ" else pkg.PQP()
        drv = pkg.md_driver(U, a, steps=10, trajectory_length=0.5, integrator=integ, precision=prec)
        r = pkg.md_trajectory_(U, P, drv)
        res[prec] = (r.delta_hamiltonian, U.to_host(), P.to_host())
    ddh = abs(res["dfloat"][0] - res["fp64"][0])
    du = np.abs(res["dfloat"][1] - res["fp64"][1]).max()
    dp = np.abs(res["dfloat"][2] - res["fp64"][2]).max()
    print("dfloat iwasaki %s: dH %.6e fp64 %.6e  |ddH| %.2e |dU| %.2e |dP| %.2e"
          % (integrator, res["dfloat"][0], res["fp64"][0], ddh, du, dp))
    assert ddh < 1e-9 and du < 1e-11 and dp < 1e-11


def _iwasaki(pkg, U):
    a = pkg.GaugeAction(U)
    pkg.push_(a, CP, "plaquette")
    pkg.push_(a, CR, "rectangular")
    return a


@pytest.mark.gpu
def test_mixed_rectangle_force_is_close(pkg, oracle):
    """The mixed form's plaquette + rectangle force: fp32 staples on the
    12-real fp32 links, against the fp64 oracle to 1e-5 of max |F|."""
    U = pkg.gauge_configuration(L6, start="hot", seed=35)
    Uh = U.to_host()
    P = pkg.gauge_momenta(U)
    pkg.update_momenta_(P, U, 1.0, pkg.md_driver(U, _iwasaki(pkg, U), steps=1, precision="mixed"))
    ref = oracle.force_loops(list(L6), Uh, CP, CR)
    rel = np.abs(P.to_host() - ref).max() / np.abs(ref).max()
    print("mixed rectangle force: rel %.2e" % rel)
    assert rel < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("dfloat", 1e-11), ("mixed", 1e-5)])
def test_smeared_rectangle_force_matches_the_oracle(pkg, oracle, prec, tol):
    """Two stout levels (rho = 0.1) under the Iwasaki action at 8^4: the top
    level's loop-set dS/dUbar (k_dsdu_rect, or k_force_rect_df writing it
    double-float-native), back-propagated by the stout adjoint of the form,
    against the oracle; tolerance relative to max |F| (fp64 1e-12,
    double-float 1e-11, mixed 1e-5)."""
    L = (8, 8, 8, 8)
    U = pkg.gauge_configuration(L, start="hot", seed=36)
    Uh = U.to_host()
    net = pkg.CovNeuralnet(U)
    pkg.push_(net, pkg.STOUT_Layer("plaquette", 0.1))
    pkg.push_(net, pkg.STOUT_Layer("plaquette", 0.1))
    P = pkg.gauge_momenta(U)
    pkg.update_momenta_(P, U, 1.0, pkg.md_driver(U, _iwasaki(pkg, U), steps=1, smearing=net, precision=prec))
    ref = oracle.stout_force_loops(list(L), Uh, (0.1, 0.1), CP, CR)
    rel = np.abs(P.to_host() - ref).max() / np.abs(ref).max()
    print("smeared rectangle force %s: |F| %.3f rel %.2e" % (prec, np.abs(ref).max(), rel))
    assert rel < tol


@pytest.mark.gpu
def test_smeared_iwasaki_trajectory_matches_the_oracle(pkg, oracle):
    """4^4 Haar start, one stout level under the Iwasaki action, tau = 0.3,
    6 QPQ steps in the plain form: H0 to 1e-13 relative, Delta H to 1e-10,
    links to 1e-12 against the oracle with a full-double-precision
    exponential."""
    U = pkg.gauge_configuration(L4, start="hot", seed=45)
    P = pkg.gaussian_momenta(U, seed=46)
    Uh, Ph = U.to_host(), P.to_host()
    net = pkg.CovNeuralnet(U)
    pkg.push_(net, pkg.STOUT_Layer("plaquette", 0.1))
    drv = pkg.md_driver(U, _iwasaki(pkg, U), steps=6, trajectory_length=0.3, smearing=net, reunitarize=False)
    res = pkg.md_trajectory_(U, P, drv)
    oracle.set_exp_method("taylor")
    try:
        h = oracle.md_trajectory(list(L4), Uh, Ph, 2 * CP, 0.3, 6, "QPQ", rho=(0.1,), c_rect=CR)
    finally:
        oracle.set_exp_method("eigen")
    du = np.abs(U.to_host() - Uh).max()
    print("smeared iwasaki: dH %.6e oracle %.6e |dU| %.2e" % (res.delta_hamiltonian, h[2], du))
    assert abs(res.initial_hamiltonian - h[0]) <= 1e-13 * abs(h[0])
    assert abs(res.delta_hamiltonian - h[2]) <= 1e-10
    assert du < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("dfloat", 1e-8), ("mixed", 2e-2)])
def test_smeared_iwasaki_forms_track_the_plain_form(pkg, prec, tol):
    """8^4 Haar start, two stout levels under the Iwasaki action, tau = 0.5,
    10 steps: Delta H of the double-float form within 1e-8 of the plain
    form's; the mixed form's (fp32 force and adjoint) within 2e-2 at this
    volume."""
    U = pkg.gauge_configuration((8, 8, 8, 8), start="hot", seed=47)
    P = pkg.gaussian_momenta(U, seed=48)
    Uh, Ph = U.to_host(), P.to_host()
    dh = {}
    for form in ("fp64", prec):
        U.from_host(Uh)
        P.from_host(Ph)
        net = pkg.CovNeuralnet(U)
        pkg.push_(net, pkg.STOUT_Layer("plaquette", 0.1))
        pkg.push_(net, pkg.STOUT_Layer("plaquette", 0.1))
        drv = pkg.md_driver(U, _iwasaki(pkg, U), steps=10, trajectory_length=0.5, smearing=net, precision=form)
        dh[form] = pkg.md_trajectory_(U, P, drv).delta_hamiltonian
    print("smeared iwasaki %s: dH %.6e fp64 %.6e diff %.2e" % (prec, dh[prec], dh["fp64"], abs(dh[prec] - dh["fp64"])))
    assert abs(dh[prec] - dh["fp64"]) < tol


# ---------------------------------------------------------------------------
# general flow (Gradientflow_general, src/smearing/gradientflow.jl:240-336)
# ---------------------------------------------------------------------------
def test_general_flow_with_plaquettes_is_the_wilson_flow(oracle):
    """F_update! with the plaquette set at coefficient 1 is add_force!(plaqonly):
    the two flows agree to rounding (exact exponential)."""
    oracle.set_exp_method("taylor")
    try:
        U = oracle.uniform_hot_start(list(L4), 123)
        V = U.copy()
        oracle.flow(list(L4), U, 0.01, 10)
        oracle.flow_loops(list(L4), V, 0.01, 10, 1.0, 0.0)
    finally:
        oracle.set_exp_method("eigen")
    assert np.abs(U - V).max() < 1e-14


def test_general_flow_lowers_the_iwasaki_action(oracle):
    U = oracle.hot_start(list(L4), 5)
    s = [oracle.action_loops(list(L4), U, C0, C1)]
    for _ in range(4):
        oracle.flow_loops(list(L4), U, 0.01, 5, C0, C1)
        s.append(oracle.action_loops(list(L4), U, C0, C1))
    assert all(b < a for a, b in zip(s, s[1:]))


def test_general_flow_api(pkg, monkeypatch):
    import gaugefields_gb300.api as api
    g = pkg.gradient_flow(None, ["plaquette", "rectangular"], [C0, C1], steps=7, step_size=0.02)
    assert isinstance(g, pkg.Gradientflow_general)
    assert (g.c_plaq, g.c_rect, g.Nflow, g.eps) == (C0, C1, 7, 0.02)
    assert isinstance(pkg.gradient_flow(None, steps=3), pkg.Gradientflow)
    with pytest.raises(ValueError):
        pkg.gradient_flow(None, ["plaquette"], None)
    with pytest.raises(ValueError):
        pkg.Gradientflow_general(None, ["plaquette", "rectangular"], [1.0])
    with pytest.raises(ValueError):
        pkg.Gradientflow_general(None, ["chair"], [1.0])
    with pytest.raises(ValueError):
        pkg.Gradientflow_general(None, ["plaquette"], [1.0 + 0.5j])
    seen = []
    monkeypatch.setattr(api, "call", lambda name, *args, ctx=None: seen.append((name, args)))
    from types import SimpleNamespace
    U = SimpleNamespace(ctx=SimpleNamespace(h="ctx"), field=SimpleNamespace(h="U"))
    pkg.flow_(U, g)
    name, args = seen[0]
    assert name == "gf_flow_loops" and args[:2] == ("ctx", "U") and args[2].value == 0.02 and args[3] == 7
    assert (args[4].value, args[5].value) == (C0, C1)


@pytest.mark.gpu
def test_general_flow_matches_the_oracle(pkg, oracle):
    """4^4 Haar start, Iwasaki loops (c0, c1), 10 steps of 0.01: links to
    1e-12 against the oracle with the exact exponential; the (1, 0) flow is
    the Wilson flow of gf_flow to 1e-12."""
    U = pkg.gauge_configuration(L4, start="hot", seed=9)
    Uh = U.to_host()
    pkg.flow_(U, pkg.gradient_flow(U, ["plaquette", "rectangular"], [C0, C1], steps=10, step_size=0.01))
    oracle.set_exp_method("taylor")
    try:
        oracle.flow_loops(list(L4), Uh, 0.01, 10, C0, C1)
    finally:
        oracle.set_exp_method("eigen")
    d = np.abs(U.to_host() - Uh).max()
    A = pkg.gauge_configuration(L4, start="hot", seed=9)
    B = pkg.gauge_configuration(L4, start="hot", seed=9)
    pkg.flow_(A, pkg.Gradientflow(A, Nflow=10, eps=0.01))
    pkg.flow_(B, pkg.Gradientflow_general(B, "plaquette", 1.0, Nflow=10, eps=0.01))
    dw = np.abs(A.to_host() - B.to_host()).max()
    print("general flow: |dU| vs oracle %.2e, vs Wilson flow %.2e" % (d, dw))
    assert d < 1e-12 and dw < 1e-12
