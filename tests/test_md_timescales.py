"""Action sets, force groups and the Sexton-Weingarten integrator
(MDActionSet, MDForceGroup, SextonWeingarten; src/molecular_dynamics.jl:45-93,
:296-402, :553-686), after the reference's own test set "Multiple MD actions
and time scales" (test/md_driver.jl:68-260).

The CPU tests drive the package's MD layer against a fake of the C-ABI whose
MD entry points (gf_md_mom_update, gf_md_link_update, gf_force,
gf_hamiltonian) are answered by the oracle on host arrays: the schedule, the group couplings
and the parameters that reach the library are the package's own, the
arithmetic is the oracle's. The GPU test runs the same trajectory on the
device and compares it with the fake's."""
from types import SimpleNamespace

import numpy as np
import pytest

import __graft_entry__ as entry

L4 = (4, 4, 4, 4)
BETA = 5.7


class _HostLinks:
    """Stands for a device link field: the fake library reads .U."""

    def __init__(self, L, U):
        self.L = L
        self.U = U
        self.ctx = SimpleNamespace(h=None, L=L)
        self.field = SimpleNamespace(h=self)

    def __len__(self):
        return 4

    def similar(self):
        return _HostLinks(self.L, np.zeros_like(self.U))


class _HostMomenta:
    def __init__(self, L, P):
        self.L = L
        self.P = P
        self.ctx = SimpleNamespace(h=None, L=L)
        self.field = SimpleNamespace(h=self)

    def __len__(self):
        return 4


def _fake_library(oracle, log):
    """call(name, *args, ctx) answering the MD entry points with the oracle."""

    def rho_of(p):
        return [p.rho[i] for i in range(p.nstout)]

    def call(name, *args, ctx=None):
        if name == "gf_md_mom_update":
            _, P, U, eps, prm = args
            p = prm._obj
            if p.c_rect != 0.0:
                F = oracle.stout_force_loops(list(P.L), U.U, rho_of(p), 0.5 * p.beta, p.c_rect)
            else:
                F = oracle.stout_force(list(P.L), U.U, rho_of(p), p.beta)
            P.P += eps.value * F
            log.append(("P", eps.value, p.beta, p.c_rect))
        elif name == "gf_md_link_update":
            _, U, P, eps, prm = args
            oracle.link_update(list(U.L), U.U, P.P, eps.value)
            log.append(("Q", eps.value))
        elif name == "gf_force":
            _, U, beta, F = args
            F.P[...] = oracle.force(list(U.L), U.U, beta.value)
            log.append(("F", beta.value))
        elif name == "gf_field_copy":
            _, dst, src = args
            dst.U[...] = src.U
        elif name == "gf_gaussian_momenta":
            _, P, seed, sweep = args
            P.P[...] = oracle.gauss_mom(list(P.L), seed.value, sweep.value)
        elif name == "gf_hamiltonian":
            _, U, P, prm, out = args
            p = prm._obj
            out._obj.value = oracle.hamiltonian(list(U.L), U.U, P.P, p.beta, rho_of(p), c_rect=p.c_rect)
        else:
            raise AssertionError("the fake library has no %s" % name)

    return call


@pytest.fixture
def md(pkg_host, oracle, monkeypatch):
    log = []
    monkeypatch.setattr(pkg_host.api, "call", _fake_library(oracle, log))
    return pkg_host, log


@pytest.fixture(scope="module")
def pkg_host():
    """The package's host layer (no library needed for these tests)."""
    pkg = entry.load_package()
    import gaugefields_gb300.api as api
    return SimpleNamespace(pkg=pkg, api=api)


def _split_actions(api, couplings):
    terms = {}
    for name, beta in couplings.items():
        a = api.GaugeAction(None)
        api.push_(a, beta / 2, "plaquette")
        terms[name] = a
    return api.MDActionSet(**terms)


def _start(oracle, seed=11, mseed=5):
    return oracle.hot_start(list(L4), seed), oracle.gauss_mom(list(L4), mseed)


def test_action_set_validation(pkg_host):
    api = pkg_host.api
    with pytest.raises(ValueError):
        api.MDActionSet()
    with pytest.raises(ValueError):
        api.MDActionSet(a=api.GaugeAction(None))            # a member without loops
    with pytest.raises(ValueError):
        api.MDForceGroup()
    with pytest.raises(ValueError):
        api.MDForceGroup("a", "a")
    assert api.MDForceGroup(("a", "b")).names == ("a", "b")
    with pytest.raises(ValueError):
        api.SextonWeingarten(slow="a", fast="b", n_fast=0)
    with pytest.raises(ValueError):
        api.SextonWeingarten(slow="a", fast="b", n_fast=1, ordering=api.OmelyanPQP())
    actions = _split_actions(api, {"first": 0.25 * BETA, "second": 0.75 * BETA})
    U = [None] * 4
    ok = api.md_driver(U, actions, steps=1, integrator=api.SextonWeingarten(slow="second", fast="first", n_fast=1))
    assert ok.params().beta == pytest.approx(BETA) and ok.params("first").beta == pytest.approx(0.25 * BETA)
    for bad in (dict(slow="second", fast="second"), dict(slow="second", fast="third"), dict(slow="second", fast=())):
        with pytest.raises(ValueError):
            api.md_driver(U, actions, steps=1, integrator=api.SextonWeingarten(n_fast=1, **bad))
    three = _split_actions(api, {"a": 1.0, "b": 2.0, "c": 3.0})
    with pytest.raises(ValueError, match="does not schedule"):
        api.md_driver(U, three, steps=1, integrator=api.SextonWeingarten(slow="a", fast="b", n_fast=2))
    grouped = api.md_driver(U, three, steps=1, integrator=api.SextonWeingarten(slow=("b", "c"), fast="a", n_fast=2))
    assert grouped.params(api.MDForceGroup("b", "c")).beta == pytest.approx(5.0)
    single = api.GaugeAction(None)
    api.push_(single, BETA / 2, "plaquette")
    with pytest.raises(ValueError, match="requires an MDActionSet"):
        api.md_driver(U, single, steps=1, integrator=api.SextonWeingarten(slow="a", fast="b", n_fast=1))
    with pytest.raises(ValueError):
        api.md_driver(U, single, steps=1).params("a")     # a group needs an action set


@pytest.mark.parametrize("ordering", ["QPQ", "PQP"])
def test_sexton_weingarten_schedule(md, oracle, ordering):
    """The reference's call counts (test/md_driver.jl:204-231): n_fast = 3,
    one step: QPQ ordering 1 slow and 6 fast kicks, PQP 2 slow and 3 fast;
    each group's kicks and the link steps add up to the step size."""
    p, log = md
    api = p.api
    actions = _split_actions(api, {"slow": 0.75 * BETA, "fast": 0.25 * BETA})
    order = api.QPQ() if ordering == "QPQ" else api.PQP()
    sw = api.SextonWeingarten(slow="slow", fast="fast", n_fast=3, ordering=order)
    Uh, Ph = _start(oracle)
    U, P = _HostLinks(L4, Uh), _HostMomenta(L4, Ph)
    drv = api.md_driver(U, actions, steps=1, trajectory_length=0.1, integrator=sw)
    api.md_trajectory_(U, P, drv, diagnostics=False)
    slow = [e for e in log if e[0] == "P" and e[2] == pytest.approx(0.75 * BETA)]
    fast = [e for e in log if e[0] == "P" and e[2] == pytest.approx(0.25 * BETA)]
    links = [e for e in log if e[0] == "Q"]
    assert (len(slow), len(fast)) == ((1, 6) if ordering == "QPQ" else (2, 3))
    assert len(slow) + len(fast) + len(links) == len(log)
    for group in (slow, fast, links):
        assert sum(e[1] for e in group) == pytest.approx(0.1, rel=1e-14)
    if ordering == "QPQ":
        assert [e[0] for e in log[:3]] == ["Q", "P", "Q"] and log[0][1] == pytest.approx(0.1 / 12)


@pytest.mark.parametrize("ordering", ["QPQ", "PQP"])
def test_sexton_weingarten_is_reversible(md, oracle, ordering):
    """test/md_driver.jl:233-256: tau then -tau returns links and momenta to
    within 3e-12."""
    p, _ = md
    api = p.api
    actions = _split_actions(api, {"slow": 0.75 * BETA, "fast": 0.25 * BETA})
    order = api.QPQ() if ordering == "QPQ" else api.PQP()
    sw = api.SextonWeingarten(slow="slow", fast="fast", n_fast=3, ordering=order)
    Uh, Ph = _start(oracle)
    U0, P0 = Uh.copy(), Ph.copy()
    U, P = _HostLinks(L4, Uh), _HostMomenta(L4, Ph)
    api.md_trajectory_(U, P, api.md_driver(U, actions, steps=2, trajectory_length=0.1, integrator=sw),
                       diagnostics=False)
    assert np.abs(U.U - U0).max() > 1e-3
    api.md_trajectory_(U, P, api.md_driver(U, actions, steps=2, trajectory_length=-0.1, integrator=sw),
                       diagnostics=False)
    assert np.abs(U.U - U0).max() < 3e-12 and np.abs(P.P - P0).max() < 3e-12


def test_group_kicks_add_up_to_the_full_kick(md, oracle):
    """test/md_driver.jl:98-121: kicking with each group in turn equals one
    kick with the whole set (2e-12)."""
    p, _ = md
    api = p.api
    actions = _split_actions(api, {"first": 0.25 * BETA, "second": 0.75 * BETA})
    Uh, Ph = _start(oracle)
    U = _HostLinks(L4, Uh)
    drv = api.md_driver(U, actions, steps=1)
    whole, grouped = _HostMomenta(L4, Ph.copy()), _HostMomenta(L4, Ph.copy())
    api.update_momenta_(whole, U, 0.02, drv)
    api.update_momenta_(grouped, U, 0.02, drv, api.MDForceGroup("first"))
    api.update_momenta_(grouped, U, 0.02, drv, api.MDForceGroup(("second",)))
    assert np.abs(whole.P - grouped.P).max() < 2e-12
    # md_force! of the set equals the sum of its groups' forces (test/md_driver.jl:88-95)
    total, first, second = (_HostMomenta(L4, np.zeros_like(Ph)) for _ in range(3))
    api.md_force_(total, actions, U)
    api.md_force_(first, actions, U, group="first")
    api.md_force_(second, actions, U, group=("second",))
    assert np.abs(total.P - first.P - second.P).max() < 2e-12
    with pytest.raises(ValueError):
        api.md_force_(total, actions, U, group="third")


def test_sexton_weingarten_error_is_second_order(md, oracle):
    """Delta H of a Sexton-Weingarten trajectory falls ~4x when the step
    halves, with a smeared action as well."""
    p, _ = md
    api = p.api
    actions = _split_actions(api, {"slow": 0.6 * BETA, "fast": 0.4 * BETA})
    sw = api.SextonWeingarten(slow="slow", fast="fast", n_fast=2)
    net = api.CovNeuralnet()
    api.push_(net, api.STOUT_Layer("plaquette", 0.1))
    dh = []
    for steps in (4, 8):
        Uh, Ph = _start(oracle, seed=3, mseed=9)
        U, P = _HostLinks(L4, Uh), _HostMomenta(L4, Ph)
        drv = api.md_driver(U, actions, steps=steps, trajectory_length=0.5, integrator=sw, smearing=net)
        dh.append(abs(api.md_trajectory_(U, P, drv).delta_hamiltonian))
    assert 2.8 < dh[0] / dh[1] < 5.5, dh


@pytest.mark.gpu
def test_sexton_weingarten_on_the_device_matches_the_oracle(pkg, pkg_host, oracle, monkeypatch):
    """The same SW trajectory (split Wilson action, n_fast = 2, both
    orderings) on the device and through the oracle: links and momenta to
    1e-10, Delta H to 1e-10."""
    api = pkg_host.api
    actions = _split_actions(api, {"slow": 0.75 * BETA, "fast": 0.25 * BETA})
    for order in (api.QPQ(), api.PQP()):
        sw = api.SextonWeingarten(slow="slow", fast="fast", n_fast=2, ordering=order)
        Uh, Ph = _start(oracle, seed=21, mseed=22)
        U = pkg.gauge_configuration(L4, start="cold").from_host(Uh)
        P = pkg.gauge_momenta(U)
        P.from_host(Ph)
        dev = api.md_trajectory_(U, P, api.md_driver(U, actions, steps=4, trajectory_length=0.5, integrator=sw))
        Ud, Pd = U.to_host(), P.to_host()
        with monkeypatch.context() as m:
            m.setattr(api, "call", _fake_library(oracle, []))
            Uo, Po = _HostLinks(L4, Uh.copy()), _HostMomenta(L4, Ph.copy())
            ref = api.md_trajectory_(Uo, Po, api.md_driver(Uo, actions, steps=4, trajectory_length=0.5,
                                                           integrator=sw))
        assert np.abs(Ud - Uo.U).max() < 1e-10 and np.abs(Pd - Po.P).max() < 1e-10
        assert abs(dev.delta_hamiltonian - ref.delta_hamiltonian) < 1e-10


def test_hmc_update_with_sexton_weingarten(md, oracle):
    """hmc_update_ for a non-builtin integrator: momentum refresh from (seed,
    sweep), the trajectory, Metropolis (accept when dH <= 0 or unif <
    exp(-dH)); a rejection restores the links exactly."""
    p, _ = md
    api = p.api
    actions = _split_actions(api, {"slow": 0.75 * BETA, "fast": 0.25 * BETA})
    sw = api.SextonWeingarten(slow="slow", fast="fast", n_fast=2)
    U0 = oracle.hot_start(list(L4), 8)
    U, P = _HostLinks(L4, U0.copy()), _HostMomenta(L4, np.zeros((4, 256, 8)))
    drv = api.md_driver(U, actions, steps=3, trajectory_length=0.3, integrator=sw)
    res = api.hmc_update_(U, P, drv, seed=17, sweep=2, unif=0.0)
    assert res.accepted and np.abs(U.U - U0).max() > 1e-3
    # the same trajectory composed by hand
    V, Q = _HostLinks(L4, U0.copy()), _HostMomenta(L4, oracle.gauss_mom(list(L4), 17, 2))
    ref = api.md_trajectory_(V, Q, drv)
    assert res.delta_hamiltonian == ref.delta_hamiltonian and np.array_equal(U.U, V.U)
    # a coarse trajectory (dH >> 1) is rejected at unif close to 1 and restores U
    coarse = api.md_driver(U, actions, steps=1, trajectory_length=2.0, integrator=sw)
    before = U.U.copy()
    res = api.hmc_update_(U, P, coarse, seed=18, sweep=0, unif=1.0 - 1e-15)
    assert res.delta_hamiltonian > 1.0 and not res.accepted and np.array_equal(U.U, before)
    with pytest.raises(ValueError):
        api.hmc_update_(U, P, coarse, seed=18, sweep=0, unif=1.0)
