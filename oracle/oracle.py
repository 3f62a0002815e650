"""ctypes binding of the oracle (gf_oracle.c) -- TEST INFRASTRUCTURE ONLY.

The oracle is the CPU restatement of Gaugefields.jl's SU(3) hot path (see the
header of gf_oracle.c for the reference files it follows). Only the tests,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline/reference leg import
this module, as the checker or as the timed CPU baseline.

Array conventions (the reference's host layouts, numpy C order):
  links   : complex128, shape (4, V, 3, 3) indexed [mu, lex, j, i] -- i.e. the
            column-major (3,3,NX,NY,NZ,NT) array of each direction, stacked.
            ``mats()`` / ``from_mats()`` convert to/from [mu, lex, i, j].
  momenta : float64, shape (4, V, 8) indexed [mu, lex, a].
  lex = x + NX*(y + NY*(z + NZ*t)).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "gf_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")

_lib = None


def build(force=False):
    """Compile liboracle.so from gf_oracle.c with gcc + OpenMP (seconds)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-std=gnu11", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", LIB, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        _declare(_lib)
    return _lib


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_U64 = ctypes.c_uint64


def _declare(l):
    sig = {
        "or_num_threads": ([], _I),
        "or_set_threads": ([_I], None),
        "or_taylor_fallbacks": ([], ctypes.c_long),
        "or_set_exp_method": ([_I], None),
        "or_set_omelyan_lambda": ([_D], None),
        "or_staple": ([_P, _P, _I, _P], None),
        "or_plaquette": ([_P, _P], _D),
        "or_dsdu": ([_P, _P, _D, _I, _P], None),
        "or_action": ([_P, _P, _D], _D),
        "or_force": ([_P, _P, _D, _P], None),
        "or_expt": ([_D, _P, _P], None),
        "or_link_update": ([_P, _P, _P, _D], None),
        "or_kinetic": ([_P, _P], _D),
        "or_normalize": ([_P, _P], None),
        "or_stout_forward": ([_P, _P, _I, _P, _P], None),
        "or_stout_backward": ([_P, _P, _I, _P, _P, _P, _P], None),
        "or_stout_force": ([_P, _P, _I, _P, _D, _P], None),
        "or_stout_action": ([_P, _P, _I, _P, _D], _D),
        "or_hamiltonian": ([_P, _P, _P, _D, _I, _P], _D),
        "or_md_trajectory": ([_P, _P, _P, _D, _D, _I, _I, _I, _P, _P], None),
        "or_md_steps": ([_P, _P, _P, _D, _D, _I, _I, _P], None),
        "or_flow_force": ([_P, _P, _P, _D], None),
        "or_flow": ([_P, _P, _D, _I], None),
        "or_hot_start": ([_P, _P, _U64], None),
        "or_uniform_hot_start": ([_P, _P, _U64], None),
        "or_gauss_mom": ([_P, _P, _U64, _U64], None),
        "or_loop_trace": ([_P, _P, _I], _D),
        "or_action_loops": ([_P, _P, _D, _D], _D),
        "or_force_loops": ([_P, _P, _D, _D, _P], None),
        "or_polyakov_loop": ([_P, _P, _P], None),
        "or_dsdu_loops": ([_P, _P, _D, _D, _P], None),
        "or_stout_force_loops": ([_P, _P, _I, _P, _D, _D, _P], None),
        "or_stout_action_loops": ([_P, _P, _I, _P, _D, _D], _D),
        "or_loop_staple_count": ([_I, _I], _I),
        "or_set_rect": ([_D], None),
        "or_flow_loops": ([_P, _P, _D, _I, _D, _D], None),
    }
    for name, (args, res) in sig.items():
        f = getattr(l, name)
        f.argtypes = args
        f.restype = res


def _L(L):
    a = np.ascontiguousarray(np.asarray(L, dtype=np.int32))
    assert a.shape == (4,)
    return a


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def vol(L):
    return int(np.prod(L))


def new_links(L):
    return np.zeros((4, vol(L), 3, 3), dtype=np.complex128)


def new_mom(L):
    return np.zeros((4, vol(L), 8), dtype=np.float64)


def mats(U):
    """[mu, lex, j, i] (reference memory order) -> [mu, lex, i, j]."""
    return np.swapaxes(U, -1, -2)


def from_mats(M):
    return np.ascontiguousarray(np.swapaxes(M, -1, -2))


def _chk(a, dtype, shape=None):
    assert a.dtype == dtype and a.flags.c_contiguous, (a.dtype, a.flags)
    if shape is not None:
        assert a.shape == shape, (a.shape, shape)


def set_threads(n):
    lib().or_set_threads(int(n))


def num_threads():
    return lib().or_num_threads()


def set_exp_method(name):
    """'eigen' (the reference's exptU!, default) or 'taylor' (full double
    precision); the choice applies to link updates, flow steps and stout."""
    lib().or_set_exp_method({"eigen": 0, "taylor": 1}[name])


def taylor_fallbacks():
    return lib().or_taylor_fallbacks()


def cold_start(L):
    U = new_links(L)
    for k in range(3):
        U[:, :, k, k] = 1.0
    return U


def hot_start(L, seed):
    U = new_links(L)
    lib().or_hot_start(_ptr(_L(L)), _ptr(U), _U64(seed))
    return U


def uniform_hot_start(L, seed):
    U = new_links(L)
    lib().or_uniform_hot_start(_ptr(_L(L)), _ptr(U), _U64(seed))
    return U


def gauss_mom(L, seed, sweep=0):
    P = new_mom(L)
    lib().or_gauss_mom(_ptr(_L(L)), _ptr(P), _U64(seed), _U64(sweep))
    return P


def plaquette(L, U):
    _chk(U, np.complex128)
    return lib().or_plaquette(_ptr(_L(L)), _ptr(U))


def polyakov_loop(L, U):
    """calculate_Polyakov_loop: mean over the first time slice of the traced
    product of the time links (complex)."""
    _chk(U, np.complex128)
    out = np.zeros(2)
    lib().or_polyakov_loop(_ptr(_L(L)), _ptr(U), _ptr(out))
    return complex(out[0], out[1])


def staple(L, U, mu):
    V = np.zeros((vol(L), 3, 3), dtype=np.complex128)
    lib().or_staple(_ptr(_L(L)), _ptr(U), int(mu), _ptr(V))
    return V


def dsdu(L, U, beta, mu):
    D = np.zeros((vol(L), 3, 3), dtype=np.complex128)
    lib().or_dsdu(_ptr(_L(L)), _ptr(U), float(beta), int(mu), _ptr(D))
    return D


def action(L, U, beta):
    _chk(U, np.complex128)
    return lib().or_action(_ptr(_L(L)), _ptr(U), float(beta))


def force(L, U, beta):
    F = new_mom(L)
    lib().or_force(_ptr(_L(L)), _ptr(U), float(beta), _ptr(F))
    return F


def expt(t, u):
    u = np.ascontiguousarray(np.asarray(u, dtype=np.float64))
    out = np.zeros(9, dtype=np.complex128)
    lib().or_expt(float(t), _ptr(u), _ptr(out))
    return out.reshape(3, 3).T.copy()  # column-major -> [i, j]


def link_update(L, U, P, eps):
    _chk(U, np.complex128)
    _chk(P, np.float64)
    lib().or_link_update(_ptr(_L(L)), _ptr(U), _ptr(P), float(eps))


def kinetic(L, P):
    _chk(P, np.float64)
    return lib().or_kinetic(_ptr(_L(L)), _ptr(P))


def normalize(L, U):
    lib().or_normalize(_ptr(_L(L)), _ptr(U))


def _rho(rho):
    return np.ascontiguousarray(np.asarray(list(rho) + [0.0] * 8, dtype=np.float64)[:8])


def stout_forward(L, U, rho):
    out = new_links(L)
    r = _rho(rho)
    lib().or_stout_forward(_ptr(_L(L)), _ptr(U), len(rho), _ptr(r), _ptr(out))
    return out


def stout_backward(L, U, rho, dSdUbar):
    out = new_links(L)
    r = _rho(rho)
    drho = np.zeros(8)
    _chk(dSdUbar, np.complex128)
    lib().or_stout_backward(_ptr(_L(L)), _ptr(U), len(rho), _ptr(r), _ptr(dSdUbar), _ptr(out), _ptr(drho))
    return out, drho[: len(rho)]


def stout_force(L, U, rho, beta):
    F = new_mom(L)
    r = _rho(rho)
    lib().or_stout_force(_ptr(_L(L)), _ptr(U), len(rho), _ptr(r), float(beta), _ptr(F))
    return F


def stout_action(L, U, rho, beta):
    r = _rho(rho)
    return lib().or_stout_action(_ptr(_L(L)), _ptr(U), len(rho), _ptr(r), float(beta))


def hamiltonian(L, U, P, beta, rho=(), c_rect=0.0):
    r = _rho(rho)
    lib().or_set_rect(float(c_rect))
    try:
        return lib().or_hamiltonian(_ptr(_L(L)), _ptr(U), _ptr(P), float(beta), len(rho), _ptr(r))
    finally:
        lib().or_set_rect(0.0)


def loop_trace(L, U, kind):
    """Re sum_x sum tr over the plaquette (kind 0) or rectangle (kind 1) loops
    and their conjugates: twice the sum of Re tr over the geometric loops."""
    _chk(U, np.complex128)
    return lib().or_loop_trace(_ptr(_L(L)), _ptr(U), int(kind))


def rectangle_sum(L, U):
    """sum_x sum_{mu<nu} Re tr (R^{1x2}_{mu nu}(x) + R^{2x1}_{mu nu}(x))."""
    return 0.5 * loop_trace(L, U, 1)


def action_loops(L, U, c_plaq, c_rect):
    _chk(U, np.complex128)
    return lib().or_action_loops(_ptr(_L(L)), _ptr(U), float(c_plaq), float(c_rect))


def force_loops(L, U, c_plaq, c_rect):
    _chk(U, np.complex128)
    F = new_mom(L)
    lib().or_force_loops(_ptr(_L(L)), _ptr(U), float(c_plaq), float(c_rect), _ptr(F))
    return F


def dsdu_loops(L, U, c_plaq, c_rect):
    """dS/dU_mu(x) = c_plaq (plaquette staples) + c_rect (rectangle staples)
    of every link, links layout."""
    _chk(U, np.complex128)
    D = new_links(L)
    lib().or_dsdu_loops(_ptr(_L(L)), _ptr(U), float(c_plaq), float(c_rect), _ptr(D))
    return D


def stout_force_loops(L, U, rho, c_plaq, c_rect):
    """Force of the plaquette + rectangle action on the stout-smeared links,
    back-propagated to the thin links."""
    _chk(U, np.complex128)
    F = new_mom(L)
    r = _rho(rho)
    lib().or_stout_force_loops(_ptr(_L(L)), _ptr(U), len(rho), _ptr(r), float(c_plaq), float(c_rect), _ptr(F))
    return F


def stout_action_loops(L, U, rho, c_plaq, c_rect):
    _chk(U, np.complex128)
    r = _rho(rho)
    return lib().or_stout_action_loops(_ptr(_L(L)), _ptr(U), len(rho), _ptr(r), float(c_plaq), float(c_rect))


def flow_loops(L, U, eps, nsteps, c_plaq, c_rect):
    """Gradientflow_general with the plaquette and rectangle loops, in place."""
    _chk(U, np.complex128)
    lib().or_flow_loops(_ptr(_L(L)), _ptr(U), float(eps), int(nsteps), float(c_plaq), float(c_rect))


def loop_staple_count(kind, mu):
    return lib().or_loop_staple_count(int(kind), int(mu))


def md_trajectory(L, U, P, beta, tau, steps, integrator="QPQ", rho=(), lam=0.1931833275037836, c_rect=0.0):
    """In place on U, P. Returns (H0, H1, dH). integrator: QPQ, PQP or OMELYAN.
    c_rect: coefficient of the rectangle loops (of the smeared links when rho
    is given)."""
    _chk(U, np.complex128)
    _chk(P, np.float64)
    out = np.zeros(3)
    r = _rho(rho)
    integ = {"QPQ": 0, "PQP": 1, "OMELYAN": 2}[integrator]
    lib().or_set_omelyan_lambda(float(lam))
    lib().or_set_rect(float(c_rect))
    try:
        lib().or_md_trajectory(_ptr(_L(L)), _ptr(U), _ptr(P), float(beta), float(tau), int(steps), integ, len(rho),
                               _ptr(r), _ptr(out))
    finally:
        lib().or_set_rect(0.0)
    return tuple(out)


def md_steps(L, U, P, beta, eps, nsteps, rho=()):
    r = _rho(rho)
    lib().or_md_steps(_ptr(_L(L)), _ptr(U), _ptr(P), float(beta), float(eps), int(nsteps), len(rho), _ptr(r))


def flow_force(L, U, factor=1.0):
    F = new_mom(L)
    lib().or_flow_force(_ptr(_L(L)), _ptr(U), _ptr(F), float(factor))
    return F


def flow(L, U, eps, nsteps):
    _chk(U, np.complex128)
    lib().or_flow(_ptr(_L(L)), _ptr(U), float(eps), int(nsteps))
