"""CPU model of the two-stage reduction of csrc/k_sbr.cu (numpy, FP64): the panel QR with
its compact-WY two-sided update (stage 1) and the bulge chase on lower band storage with
2*b+1 offsets in the wavefront order of k_sb_chase (stage 2), checked against eigvalsh; and
the schedule's claims: the tasks of one time step touch disjoint index ranges at a lag of
four steps (not at two or three), and warp c % 8 is free for sweep c when n <= 32*b + 1."""
import numpy as np
import pytest


def house(x):
    alpha = x[0]
    xn2 = float(x[1:] @ x[1:])
    v = np.zeros_like(x)
    v[0] = 1.0
    if xn2 == 0.0:
        return v, 0.0, alpha
    beta = -np.copysign(np.sqrt(alpha * alpha + xn2), alpha)
    v[1:] = x[1:] / (alpha - beta)
    return v, (beta - alpha) / beta, beta


def stage1(A, b):
    n = A.shape[0]
    S = A.copy()
    k = 0
    while n - k - b >= 1:
        m = n - k - b
        P = S[k + b:, k:k + b].copy()
        V = np.zeros((m, b))
        T = np.zeros((b, b))
        for j in range(min(b, m)):
            v, t, beta = house(P[j:, j])
            P[j:, j + 1:] -= t * np.outer(v, v @ P[j:, j + 1:])
            P[j, j], P[j + 1:, j] = beta, 0.0
            V[j:, j] = v
            T[:j, j] = -t * (T[:j, :j] @ (V[:, :j].T @ V[:, j]))
            T[j, j] = t
        S[k + b:, k:k + b] = P
        S[k:k + b, k + b:] = P.T
        Y = S[k + b:, k + b:] @ V @ T
        W = Y - 0.5 * V @ (T.T @ (V.T @ Y))
        S[k + b:, k + b:] -= V @ W.T + W @ V.T
        k += b
    return S


def nsteps(n, b, c):
    return (n - 1 - c + b - 1) // b


def task_span(n, b, c, k):
    rk = c + 1 + k * b
    L = min(b, n - rk)
    lo = c if k == 0 else rk - b
    return lo, min(n, rk + L + min(b, max(0, n - rk - L)))


def stage2(S, b, lag=4):
    n = S.shape[0]
    Bd = np.zeros((n, 2 * b + 1))
    for c in range(n):
        for o in range(min(b, n - 1 - c) + 1):
            Bd[c, o] = S[c + o, c]

    def get(r, c):
        r, c = max(r, c), min(r, c)
        return Bd[c, r - c] if r - c <= 2 * b else 0.0

    def put(r, c, x):
        r, c = max(r, c), min(r, c)
        assert r - c <= 2 * b or abs(x) < 1e-9
        if r - c <= 2 * b:
            Bd[c, r - c] = x

    nsw = n - 2
    tmax = lag * (nsw - 1) + nsteps(n, b, 0)
    for tt in range(tmax):
        for c in range(nsw):
            k = tt - lag * c
            if k < 0 or k >= nsteps(n, b, c):
                continue
            rk = c + 1 + k * b
            L = min(b, n - rk)
            col = c if k == 0 else rk - b
            x = np.array([get(rk + i, col) for i in range(L)])
            v, t, beta = house(x)
            cols = range(col, rk)
            Bk = np.array([[get(rk + i, cc) for cc in cols] for i in range(L)])
            Bk -= t * np.outer(v, v @ Bk)
            Bk[:, 0] = 0.0
            Bk[0, 0] = beta
            for i in range(L):
                for jj, cc in enumerate(cols):
                    put(rk + i, cc, Bk[i, jj])
            D = np.array([[get(rk + i, rk + j) for j in range(L)] for i in range(L)])
            p = t * (D @ v)
            z = p - 0.5 * t * (v @ p) * v
            D -= np.outer(v, z) + np.outer(z, v)
            for i in range(L):
                for j in range(i + 1):
                    put(rk + i, rk + j, D[i, j])
            r2 = rk + L
            L2 = min(b, n - r2)
            if L2 > 0:
                B2 = np.array([[get(r2 + i, rk + j) for j in range(L)] for i in range(L2)])
                B2 -= t * np.outer(B2 @ v, v)
                for i in range(L2):
                    for j in range(L):
                        put(r2 + i, rk + j, B2[i, j])
    return Bd


@pytest.mark.parametrize("n,b", [(3, 4), (40, 4), (67, 8), (130, 16)])
def test_two_stage_model_keeps_the_eigenvalues(n, b):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n))
    A = a + a.T
    S = stage1(A, b)
    assert np.abs(np.tril(S, -b - 1)).max(initial=0.0) == 0.0        # a band of width b
    Bd = stage2(S, b)
    assert np.abs(Bd[:, 2:]).max() < 1e-12                            # tridiagonal, the fill chased out
    T = np.diag(Bd[:, 0]) + np.diag(Bd[:-1, 1], -1) + np.diag(Bd[:-1, 1], 1)
    np.testing.assert_allclose(np.linalg.eigvalsh(T), np.linalg.eigvalsh(A), atol=1e-10 * np.abs(A).max())


def _disjoint(n, b, lag):
    nsw = n - 2
    tmax = lag * (nsw - 1) + nsteps(n, b, 0)
    widest = 0
    for tt in range(tmax):
        spans = sorted(task_span(n, b, c, tt - lag * c) for c in range(nsw)
                       if 0 <= tt - lag * c < nsteps(n, b, c))
        if any(s1[0] < s0[1] for s0, s1 in zip(spans, spans[1:])):
            return False, widest
        widest = max(widest, len(spans))
    return True, widest


def test_chase_schedule_lag_four_at_order_1024():
    assert not _disjoint(1024, 32, 2)[0]
    assert not _disjoint(1024, 32, 3)[0]
    ok, widest = _disjoint(1024, 32, 4)
    assert ok and widest <= 8                      # at most eight tasks: one per warp of k_sb_chase
    # warp c % 8 runs sweep c from step 4c; sweep c - 8 has ended by then
    for n in (1024, 1025):
        assert max(nsteps(n, 32, c) for c in range(n - 2)) <= 4 * 8
