"""CPU model of the algebra in csrc/k_backtransform.cu's split-form preparation (numpy,
FP64): T of a block of Householder reflectors from its diagonal sub-blocks and the
compact-WY combination T_AB = -T_A G_AB T_B (k_bt_tmat), and a pair of blocks applied as one,
T = [[T_1, -T_1 X^T T_2], [0, T_2]] and Y = [Y_1; Y_2 - C Y_1] with X = V_2^T V_1 and
C = T_2^T X (k_bt_cross and the pair correction), against the reflectors multiplied out."""
import numpy as np


def reflectors(n, k0, nb, kd, rng):
    """nb reflectors of a block starting at column k0, reflector j with its unit at row
    k0 + j + kd and zeros above (LAPACK sytrd storage for kd = 1)."""
    V = np.zeros((n, nb))
    for j in range(nb):
        r = k0 + j + kd
        V[r, j] = 1.0
        V[r + 1:, j] = rng.standard_normal(n - r - 1) * 0.3
    tau = 2.0 / np.sum(V * V, axis=0)
    return V, tau


def slarft(G, tau):
    nb = len(tau)
    T = np.zeros((nb, nb))
    for j in range(nb):
        T[:j, j] = -tau[j] * (T[:j, :j] @ G[:j, j])
        T[j, j] = tau[j]
    return T


def blocked_t(G, tau, w):
    """k_bt_tmat's order: diagonal blocks of w columns by the recursion, then pairs of blocks
    combined, doubling the width until the whole block is covered."""
    nb = len(tau)
    T = np.zeros((nb, nb))
    for a in range(0, nb, w):
        T[a:a + w, a:a + w] = slarft(G[a:a + w, a:a + w], tau[a:a + w])
    while w < nb:
        for a in range(0, nb, 2 * w):
            b = a + w
            T[a:b, b:b + w] = -T[a:b, a:b] @ (G[a:b, b:b + w] @ T[b:b + w, b:b + w])
        w *= 2
    return T


def product(V, tau):
    Q = np.eye(V.shape[0])
    for j in range(V.shape[1]):
        Q = Q @ (np.eye(V.shape[0]) - tau[j] * np.outer(V[:, j], V[:, j]))
    return Q


def test_blocked_t_equals_the_column_recursion():
    rng = np.random.default_rng(0)
    V, tau = reflectors(70, 0, 16, 1, rng)
    G = V.T @ V
    T = slarft(G, tau)
    np.testing.assert_allclose(blocked_t(G, tau, 4), T, atol=1e-12 * np.abs(T).max())
    np.testing.assert_allclose(np.eye(70) - V @ T @ V.T, product(V, tau), atol=1e-12)


def test_pair_of_blocks_applied_as_one():
    rng = np.random.default_rng(1)
    n, nb = 90, 12
    V1, t1 = reflectors(n, 0, nb, 1, rng)
    V2, t2 = reflectors(n, nb, nb, 1, rng)
    T1, T2 = slarft(V1.T @ V1, t1), slarft(V2.T @ V2, t2)
    X = V2.T @ V1                          # the cross Gram, over V_2's rows (V_2 is zero above)
    C = T2.T @ X                            # k_bt_cross
    Y1, Y2 = T1.T @ V1.T, T2.T @ V2.T       # the blocks' own Y_b = T_b^T V_b^T
    Y = np.vstack([Y1, Y2 - C @ Y1])        # the pair correction
    V = np.hstack([V1, V2])
    T = np.block([[T1, -T1 @ X.T @ T2], [np.zeros((nb, nb)), T2]])
    np.testing.assert_allclose(Y, T.T @ V.T, atol=1e-12)
    np.testing.assert_allclose(np.eye(n) - V @ T @ V.T, product(V, np.concatenate([t1, t2])), atol=1e-12)
    # the update in the transposed view: Z^T <- Z^T (I - V T^T V^T) = Z^T - (Z^T V) Y
    Z = rng.standard_normal((n, n))
    np.testing.assert_allclose(Z.T - (Z.T @ V) @ Y, (product(V, np.concatenate([t1, t2])) @ Z).T, atol=1e-11)
