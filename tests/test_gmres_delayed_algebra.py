"""The delayed CGS2 recurrences of the device GMRES (the reorthogonalisation
of a vector deferred to the next step's pass of dot products), restated in
numpy and checked against classical Gram-Schmidt applied twice: the same
Hessenberg matrix and basis up to rounding.  These are the formulas the
staged passes 4-6 evaluate (the last CTA's scalar work and the per-element
updates), in FP64 on the CPU."""
import numpy as np


def _arnoldi_cgs2(M, r0, m):
    n = r0.size
    Q = np.zeros((n, m + 1))
    H = np.zeros((m + 1, m))
    Q[:, 0] = r0 / np.linalg.norm(r0)
    for k in range(m):
        w = M @ Q[:, k]
        h = Q[:, :k + 1].T @ w
        w = w - Q[:, :k + 1] @ h
        h2 = Q[:, :k + 1].T @ w
        w = w - Q[:, :k + 1] @ h2
        H[:k + 1, k] = h + h2
        H[k + 1, k] = np.linalg.norm(w)
        Q[:, k + 1] = w / H[k + 1, k]
    return Q, H


def _arnoldi_delayed(M, r0, m):
    """Column k holds u_k (once orthogonalised, unnormalised) until step
    k + 1; Hr holds the Hessenberg columns before the rotations, column k
    tentative until step k + 1 adds its reorthogonalisation coefficients."""
    n = r0.size
    V = np.zeros((n, m + 1))
    Hr = np.zeros((m + 1, m + 1))
    V[:, 0] = r0 / np.linalg.norm(r0)
    for k in range(m):
        u = V[:, k].copy()
        w = M @ u                                   # the SpMV on u_k
        Q = V[:, :k]
        t, gamma = Q.T @ w, u @ w                   # pass 4, first half
        s, alpha = Q.T @ u, u @ u                   # pass 4, second half
        if k == 0:
            r = 1.0
        else:
            r = np.sqrt(alpha - s @ s)              # Pythagorean norm of u_k - Q s
            Hr[:k, k - 1] += s                      # column k - 1 is final
            Hr[k, k - 1] = r
        tau = (gamma - s @ t) / r                   # q_k . w
        for i in range(k + 1):                      # tentative column k
            hs = sum(Hr[i, j] * s[j] for j in range(max(i - 1, 0), k))
            Hr[i, k] = ((t[i] if i < k else tau) - hs) / r
        q = (u - Q @ s) / r if k > 0 else u         # pass 5
        V[:, k] = q
        V[:, k + 1] = (w - Q @ t - tau * q) / r
    u = V[:, m]                                     # pass 6: the cycle's last column
    s, alpha = V[:, :m].T @ u, u @ u
    Hr[:m, m - 1] += s
    Hr[m, m - 1] = np.sqrt(alpha - s @ s)
    return V[:, :m], Hr[:, :m]


def test_delayed_cgs2_matches_cgs2():
    rng = np.random.default_rng(3)
    n, m = 300, 20
    M = np.eye(n) * 3.0 + rng.standard_normal((n, n)) * 0.08   # nonsymmetric
    r0 = rng.standard_normal(n)
    Q, H = _arnoldi_cgs2(M, r0, m)
    Qd, Hd = _arnoldi_delayed(M, r0, m)
    assert np.abs(Hd - H).max() <= 1e-12 * np.abs(H).max()
    assert np.abs(Qd - Q[:, :m]).max() <= 1e-12
    # the Arnoldi relation M Q_m = Q_{m+1} H with the delayed quantities
    Qm1 = np.column_stack([Qd, Q[:, m]])
    assert np.abs(M @ Qd - Qm1 @ Hd).max() <= 1e-11
