"""Reference derivatives for the VJP tests: analytic gradients of the
closed-form equities and central finite differences of the oracle.

Closed forms (reference src/cpu/icm.c:145-170):
  V1_i = 1 + sum_{j != i} S_i / (S_i + S_j)            payout[m] = n - m, k = n
  V2_i = sum_{j < l; j, l != i} S_i / (S_i + S_j + S_l)  payout[m] = C(n-1-m, 2)
and for payout (k - j + 1)^2 with k = n:  E = 2 V2 + 3 V1 - 2.
"""
import numpy as np


def v1_loss_grad(S, cot):
    """d/dS of sum_i cot_i V1_i."""
    S = np.asarray(S, dtype=np.float64)
    T = S[:, None] + S[None, :]
    M = 1.0 / (T * T)
    np.fill_diagonal(M, 0.0)
    # d V1_i / d S_i = sum_{j != i} S_j / T_ij^2 ; d V1_i / d S_j = -S_i / T_ij^2
    return cot * (M @ S) - (cot * S) @ M


def v1_loss_grad_blocked(S, cot, block=1024):
    """v1_loss_grad in row blocks (memory O(block n) for large n)."""
    S = np.asarray(S, dtype=np.float64)
    cot = np.asarray(cot, dtype=np.float64)
    out = np.zeros_like(S)
    for i0 in range(0, len(S), block):
        Si = S[i0:i0 + block]
        T = Si[:, None] + S[None, :]
        M = 1.0 / (T * T)
        idx = np.arange(i0, i0 + len(Si))
        M[np.arange(len(Si)), idx] = 0.0
        out[i0:i0 + block] += cot[i0:i0 + block] * (M @ S)
        out -= (cot[i0:i0 + block] * Si) @ M
    return out


def v2_loss_grad(S, cot):
    """d/dS of sum_i cot_i V2_i (O(n^3); small n only)."""
    S = np.asarray(S, dtype=np.float64)
    n = len(S)
    T = S[:, None, None] + S[None, :, None] + S[None, None, :]
    idx = np.arange(n)
    valid = ((idx[:, None, None] != idx[None, :, None]) & (idx[:, None, None] != idx[None, None, :])
             & (idx[None, :, None] < idx[None, None, :]))
    inv2 = np.where(valid, 1.0 / (T * T), 0.0)
    # own term: d/dS_i S_i / T = (S_j + S_l) / T^2
    own = np.einsum("ijl,ijl->i", inv2, (S[None, :, None] + S[None, None, :]) * np.ones_like(T))
    # cross term: d/dS_j S_i / T = -S_i / T^2 for j in the pair {j, l}
    w = cot * S                                # weight of row i
    cross = -(np.einsum("i,ijl->j", w, inv2) + np.einsum("i,ijl->l", w, inv2))
    return cot * own + cross


def quadratic_loss_grad(S, cot):
    """d/dS of sum_i cot_i (2 V2_i + 3 V1_i - 2), the (k - j + 1)^2 payout at k = n."""
    return 2.0 * v2_loss_grad(S, cot) + 3.0 * v1_loss_grad(S, cot)


def fd_directional(f, S, u, rel_step=1e-6):
    """Central difference of f along S -> S * (1 + h u) (relative step)."""
    S = np.asarray(S, dtype=np.float64)
    up = f(S * (1.0 + rel_step * u))
    dn = f(S * (1.0 - rel_step * u))
    return (up - dn) / (2.0 * rel_step)
