"""The product tables of the double-float stout kernels (gf_stout.cu), run on
the host in complex128 with the kernels' operand rules: an operand is field
F0, F1 or F2 in direction d0 or d1 at one of the kernel's five sites
(optionally daggered) or a per-thread slot; a product goes to a slot,
optionally added to it. The GPU tests check the kernels against the oracle;
these pin the tables' encoding on the CPU.

* c_stout_ops 0-3 (per axis nu, sites x, x+mu, x+nu, x+mu-nu, x-nu): the
  staple sum S_mu of the stout forward, against the oracle's dS/dU of the
  Wilson action (beta = 2: the plain staple sum, calc_dSdUmu!).
* c_local_ops 0-11 and 12-23 (the local adjoint's recomputed C and its top
  level's Dbar staples, same sites): the same staple sum of F0 and of F1.
* c_gather_ops (per axis kappa, F0 = U, F1 = Z, d0 = nu, d1 = kappa, sites x,
  x+nu, x+kappa, x-kappa, x-kappa+nu): the six staple-position terms of the
  adjoint's pull-back through C,
    (a) U_k(x+n) U_n(x+k)^+ Z_k(x)     (b) U_k(x-k+n)^+ U_n(x-k)^+ Z_k(x-k)^+
    (c) Z_k(x+n)^+ U_n(x+k)^+ U_k(x)^+ (d) Z_k(x+n-k) U_n(x-k)^+ U_k(x-k)
    (e) U_k(x-k+n)^+ Z_n(x-k) U_k(x-k) (f) U_k(x+n) Z_n(x+k) U_k(x)^+
  on random matrices.
"""
import numpy as np

from test_library import _df_tables
from test_oracle import L4

V4 = 256


def _site(L, x, moves):
    c = [x % L[0], (x // L[0]) % L[1], (x // (L[0] * L[1])) % L[2], x // (L[0] * L[1] * L[2])]
    for axis, d in moves:
        c[axis] = (c[axis] + d) % L[axis]
    return c[0] + L[0] * (c[1] + L[1] * (c[2] + L[2] * c[3]))


def _run(ops, fields, sites, d0, d1, slots):
    """Execute table rows on the host: fields[f][dir][site] -> 3x3 matrix."""
    for r in ops:
        a_src, a_dir, a_site, a_dag, b_src, b_dir, b_site, b_dag, out, acc = r

        def operand(src, d, site, dag):
            if src >= 3:
                m = slots[src - 3]
            else:
                m = fields[src][d1 if d else d0, sites[site]]
            return m.conj().T if dag else m

        prod = operand(a_src, a_dir, a_site, a_dag) @ operand(b_src, b_dir, b_site, b_dag)
        slots[out] = slots[out] + prod if acc else prod
    return slots


def _staple_sites(L, x, mu, nu):
    return [x, _site(L, x, [(mu, 1)]), _site(L, x, [(nu, 1)]), _site(L, x, [(mu, 1), (nu, -1)]),
            _site(L, x, [(nu, -1)])]


def test_forward_and_local_tables_build_the_staple_sum(oracle):
    _, tables = _df_tables()
    L = list(L4)
    U = oracle.hot_start(L, 17)
    M = oracle.mats(U)
    fwd = tables["c_stout_ops"][0:4]
    loc = tables["c_local_ops"]
    worst = 0.0
    for mu in range(4):
        ref = np.swapaxes(oracle.dsdu(L, U, 2.0, mu), -1, -2)
        for x in range(0, V4, 5):
            s_fwd = [np.zeros((3, 3), complex) for _ in range(2)]
            s_loc = [np.zeros((3, 3), complex) for _ in range(6)]
            for k in range(3):
                nu = (mu + 1 + k) % 4
                sites = _staple_sites(L, x, mu, nu)
                _run(fwd, [M], sites, mu, nu, s_fwd)
                # local adjoint: ops 0-11 on F0 into slot 5, ops 12-23 on F1 into slot 4 (four rows per axis)
                _run(loc[4 * k:4 * k + 4], [M, M, M], sites, mu, nu, s_loc)
                _run(loc[12 + 4 * k:12 + 4 * k + 4], [M, M, M], sites, mu, nu, s_loc)
            worst = max(worst, np.abs(s_fwd[1] - ref[x]).max(), np.abs(s_loc[5] - ref[x]).max(),
                        np.abs(s_loc[4] - ref[x]).max())
    assert worst < 1e-13


def test_gather_table_builds_the_six_terms():
    _, tables = _df_tables()
    ops = tables["c_gather_ops"]
    L = list(L4)
    rng = np.random.RandomState(3)
    U = rng.normal(size=(4, V4, 3, 3)) + 1j * rng.normal(size=(4, V4, 3, 3))
    Z = rng.normal(size=(4, V4, 3, 3)) + 1j * rng.normal(size=(4, V4, 3, 3))
    d = lambda m: m.conj().T  # noqa: E731
    worst = 0.0
    for n in range(4):
        for x in range(0, V4, 3):
            slots = [np.zeros((3, 3), complex) for _ in range(2)]
            ref = np.zeros((3, 3), complex)
            for j in range(1, 4):
                k = (n + j) % 4
                xn, xk, xmk = _site(L, x, [(n, 1)]), _site(L, x, [(k, 1)]), _site(L, x, [(k, -1)])
                xmkn = _site(L, x, [(k, -1), (n, 1)])
                _run(ops, [U, Z, Z], [x, xn, xk, xmk, xmkn], n, k, slots)
                ref += U[k, xn] @ d(U[n, xk]) @ Z[k, x]                   # (a)
                ref += d(U[k, xmkn]) @ d(U[n, xmk]) @ d(Z[k, xmk])        # (b)
                ref += d(Z[k, xn]) @ d(U[n, xk]) @ d(U[k, x])             # (c)
                ref += Z[k, xmkn] @ d(U[n, xmk]) @ U[k, xmk]              # (d)
                ref += d(U[k, xmkn]) @ Z[n, xmk] @ U[k, xmk]              # (e)
                ref += U[k, xn] @ Z[n, xk] @ d(U[k, x])                   # (f)
            worst = max(worst, np.abs(slots[1] - ref).max() / np.abs(ref).max())
    assert worst < 1e-13
