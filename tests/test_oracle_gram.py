"""The overlap and metric of subspaces A and C factor through the (nelec +- 1)-electron space.

The reference builds, for A (solve_A_subspace.F90) and C (solve_C_subspace.F90),
    S_A = -<E_zy E_tx E_uv> + delta_tx <E_zy E_uv>,   S_C = <E_zy E_xt E_uv>
and B = S-like terms with the active Fock operator.  With g_tuv = a_t^+ E_uv|0> (A) or
a_t E_uv|0> (C) these are exactly S = G^H G and B = G^H D G, D the active Fock operator
(diagonal over determinants).  The GPU path diagonalises K = G G^H instead of S; this test
pins the identity on the oracle's own density formulas."""
import numpy as np
import pytest

from conftest import oracle_system


def _colex(na, ne):
    if ne < 0 or ne > na:
        return []
    if ne == 0:
        return [0]
    out, cur = [], (1 << ne) - 1
    while cur < (1 << na):
        out.append(cur)
        t = (cur | (cur - 1)) + 1
        cur = t | ((((t & -t) // (cur & -cur)) >> 1) - 1)
    return out


def _above(i, p, na):
    return bin(i & (((1 << na) - 1) ^ ((1 << (p + 1)) - 1))).count("1")


def _state(cfg):
    from oracle import caspt2_oracle as O
    from dirac_caspt2_gb300 import api, synth
    s = oracle_system(api.SystemInput.from_synth(synth.make_system(cfg)))
    ni, na = s.ninact, s.nact
    ints = O.Integrals(s)
    g_occ = ints.occ_block()
    dets = O.enumerate_dets(s)
    _, v = O.heev_upper(O.casmat(s, dets, g_occ))
    c0 = v[:, s.selectroot - 1]
    fs = O.FullSpace(s, dets)
    f = O.fock_casci(s, ints, g_occ, O.RDM(fs, c0, order=1).D1)
    U, eps = O.fock_diag(s, f)
    c = O.ci_rotate(s, dets, U[ni:ni + na, ni:ni + na], c0)
    rd = O.RDM(fs, c, eps_act=eps[ni:ni + na], order=3)
    return s, fs, c, rd, eps


@pytest.mark.parametrize("real", [False, True])
def test_gram_factor_of_A_and_C(real):
    from dirac_caspt2_gb300 import synth
    s, fs, c, rd, eps = _state(synth.SynthConfig(2, 6, 4, 4, realonly=real, seed=9))
    ni, na, ne = s.ninact, s.nact, s.nelec
    psi = fs.embed(c)
    Y = {(u, v): fs.apply(u, v, psi) for u in range(na) for v in range(na)}
    cols = [(t, u, v) for t in range(na) for u in range(na) for v in range(na)]
    x = np.array([q[0] for q in cols])
    y = np.array([q[1] for q in cols])
    z = np.array([q[2] for q in cols])
    t, u, v = x, y, z
    gi = lambda q: ni + q
    for kind, ne2 in (("A", ne + 1), ("C", ne - 1)):
        space = _colex(na, ne2)
        index = {d: k for k, d in enumerate(space)}
        G = np.zeros((len(space), len(cols)), complex)
        for j, (tt, uu, vv) in enumerate(cols):
            yv = Y[(uu, vv)]
            for n, I in enumerate(fs.full):
                if yv[n] == 0:
                    continue
                occ = (I >> tt) & 1
                if (kind == "A" and occ) or (kind == "C" and not occ):
                    continue
                J = I | (1 << tt) if kind == "A" else I & ~(1 << tt)
                G[index[J], j] += (-1) ** _above(I, tt, na) * yv[n]
        D = np.array([sum(eps[gi(w)] for w in range(na) if (K >> w) & 1) for K in space])
        if kind == "A":
            Sm = (-rd.D3[z[:, None], y[:, None], t[None, :], x[:, None], u[None, :], v[None, :]]
                  + (t[None, :] == x[:, None]) * rd.D2[z[:, None], y[:, None], u[None, :], v[None, :]])
            e = eps[gi(u)] + eps[gi(t)] - eps[gi(v)]
            Bm = (-rd.T3[z[:, None], y[:, None], t[None, :], x[:, None], u[None, :], v[None, :]]
                  + (t[None, :] == x[:, None]) * rd.T2[z[:, None], y[:, None], u[None, :], v[None, :]]
                  + Sm * e[None, :])
        else:
            Sm = rd.D3[z[:, None], y[:, None], x[:, None], t[None, :], u[None, :], v[None, :]]
            e = eps[gi(y)] - eps[gi(z)] - eps[gi(x)]
            Bm = rd.T3[z[:, None], y[:, None], x[:, None], t[None, :], u[None, :], v[None, :]] + Sm * e[None, :]
        up = np.triu_indices(len(cols))   # the triangle ZHEEV(uplo='U') reads
        assert np.abs((Sm - G.conj().T @ G)[up]).max() < 1e-13
        assert np.abs((Bm - G.conj().T @ (D[:, None] * G))[up]).max() < 1e-12
