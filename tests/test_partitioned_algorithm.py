"""The partitioned banded solve of the device solver (csrc/band_torn.cuh,
csrc/band_bcr.cuh), restated in numpy and checked against a dense solve: a
banded matrix cut into interiors and separators of s dofs, the spikes
Y = A_I⁻¹E, the block-tridiagonal Schur complement on the separators, its
block cyclic reduction with the device's level and role rule (level l,
stride h = 2ˡ: block k is eliminated when k/h is odd, kept when even), the
root solve and the back-substitutions.  Separator counts 1..40 (powers of two
and not), block sizes 1..5."""
import numpy as np
import pytest


def bcr_role(k, N, l):
    h = 1 << l
    if k % h != 0 or k >= N:
        return 0
    return 1 if (k // h) & 1 else 2


def bcr_solve(D, L, U, r):
    """x with L_k x_{k-1} + D_k x_k + U_k x_{k+1} = r_k (L_0 = U_{N-1} = 0), by the
    device's block cyclic reduction."""
    N = len(D)
    D, L, U, r = [d.copy() for d in D], [x.copy() for x in L], [x.copy() for x in U], [x.copy() for x in r]
    nlev = 0
    while (1 << nlev) < N:
        nlev += 1
    WL, WU, z = [None] * N, [None] * N, [None] * N
    for l in range(nlev):
        h = 1 << l
        for k in range(N):
            if bcr_role(k, N, l) == 1:
                WL[k] = np.linalg.solve(D[k], L[k])
                WU[k] = np.linalg.solve(D[k], U[k]) if k + h < N else np.zeros_like(D[k])
                z[k] = np.linalg.solve(D[k], r[k])
        nD, nL, nU = list(D), list(L), list(U)
        for e in range(N):
            if bcr_role(e, N, l) != 2:
                continue
            up, dn = e + h < N, e >= h
            if up:
                r[e] = r[e] - U[e] @ z[e + h]
                nD[e] = nD[e] - U[e] @ WL[e + h]
                nU[e] = -U[e] @ WU[e + h]
            else:
                nU[e] = np.zeros_like(U[e])
            if dn:
                r[e] = r[e] - L[e] @ z[e - h]
                nD[e] = nD[e] - L[e] @ WU[e - h]
                nL[e] = -L[e] @ WL[e - h]
            else:
                nL[e] = np.zeros_like(L[e])
        D, L, U = nD, nL, nU
    x = [None] * N
    x[0] = np.linalg.solve(D[0], r[0])
    for l in range(nlev - 1, -1, -1):
        h = 1 << l
        for k in range(N):
            if bcr_role(k, N, l) == 1:
                v = z[k] - WL[k] @ x[k - h]
                if k + h < N:
                    v = v - WU[k] @ x[k + h]
                x[k] = v
    return x


def _banded(n, kl, ku, rng):
    A = np.zeros((n, n))
    for i in range(n):
        for j in range(max(0, i - kl), min(n, i + ku + 1)):
            A[i, j] = rng.normal()
        A[i, i] += 4.0 * (kl + ku + 1)  # diagonally dominant: no pivoting needed for the check
    return A


@pytest.mark.parametrize("N", list(range(1, 18)) + [31, 32, 33, 40])
@pytest.mark.parametrize("s", [1, 3, 5])
def test_block_cyclic_reduction_solves_the_block_tridiagonal_system(N, s):
    rng = np.random.default_rng(100 * N + s)
    D = [rng.normal(size=(s, s)) + 6.0 * s * np.eye(s) for _ in range(N)]
    L = [rng.normal(size=(s, s)) if k > 0 else np.zeros((s, s)) for k in range(N)]
    U = [rng.normal(size=(s, s)) if k < N - 1 else np.zeros((s, s)) for k in range(N)]
    r = [rng.normal(size=s) for _ in range(N)]
    A = np.zeros((N * s, N * s))
    for k in range(N):
        A[k * s:(k + 1) * s, k * s:(k + 1) * s] = D[k]
        if k > 0:
            A[k * s:(k + 1) * s, (k - 1) * s:k * s] = L[k]
        if k < N - 1:
            A[k * s:(k + 1) * s, (k + 1) * s:(k + 2) * s] = U[k]
    x = np.concatenate(bcr_solve(D, L, U, r))
    xr = np.linalg.solve(A, np.concatenate(r))
    assert np.max(np.abs(x - xr)) <= 1e-12 * np.max(np.abs(xr))


@pytest.mark.parametrize("P,kl,ku", [(2, 2, 2), (5, 3, 2), (13, 4, 4), (9, 1, 3)])
def test_partitioned_banded_solve_equals_the_dense_solve(P, kl, ku):
    """Interiors I_0 S_1 I_1 ... S_{P-1} I_{P-1} with separators of s = max(kl, ku)
    dofs: ỹ_a = A_a⁻¹ b_a, r_k = b_S_k - F^R_{k-1} ỹ_{k-1} - F^L_k ỹ_k,
    T x_S = r (T block tridiagonal, by cyclic reduction), x_a = ỹ_a - Y^L_a x_S_a - Y^R_a x_S_a+1."""
    rng = np.random.default_rng(P * 31 + kl)
    s = max(kl, ku)
    m = [int(v) for v in rng.integers(2 * s, 4 * s + 3, P)]  # interior sizes (>= 2s)
    n = sum(m) + (P - 1) * s
    A = _banded(n, kl, ku, rng)
    b = rng.normal(size=n)
    # positions
    I, S, p = [], [], 0
    for a in range(P):
        I.append(np.arange(p, p + m[a]))
        p += m[a]
        if a < P - 1:
            S.append(np.arange(p, p + s))
            p += s
    assert p == n
    # no entry couples two interiors
    for a in range(P):
        for c in range(P):
            if a != c:
                assert not np.any(A[np.ix_(I[a], I[c])])
    Aa = [A[np.ix_(I[a], I[a])] for a in range(P)]
    yt = [np.linalg.solve(Aa[a], b[I[a]]) for a in range(P)]
    YL = [np.linalg.solve(Aa[a], A[np.ix_(I[a], S[a - 1])]) if a > 0 else None for a in range(P)]
    YR = [np.linalg.solve(Aa[a], A[np.ix_(I[a], S[a])]) if a < P - 1 else None for a in range(P)]
    N = P - 1
    if N == 0:
        x = yt[0]
    else:
        D, L, U, r = [], [], [], []
        for k in range(N):  # separator k sits between interiors k and k+1
            FR = A[np.ix_(S[k], I[k])]      # F^R of interior k
            FL = A[np.ix_(S[k], I[k + 1])]  # F^L of interior k+1
            D.append(A[np.ix_(S[k], S[k])] - FR @ YR[k] - FL @ YL[k + 1])
            L.append(-FR @ YL[k] if k > 0 else np.zeros((s, s)))
            U.append(-FL @ YR[k + 1] if k < N - 1 else np.zeros((s, s)))
            r.append(b[S[k]] - FR @ yt[k] - FL @ yt[k + 1])
        xs = bcr_solve(D, L, U, r)
        x = np.zeros(n)
        for a in range(P):
            v = yt[a].copy()
            if a > 0:
                v -= YL[a] @ xs[a - 1]
            if a < P - 1:
                v -= YR[a] @ xs[a]
            x[I[a]] = v
        for k in range(N):
            x[S[k]] = xs[k]
    xr = np.linalg.solve(A, b)
    assert np.max(np.abs(x - xr)) <= 1e-11 * np.max(np.abs(xr))
