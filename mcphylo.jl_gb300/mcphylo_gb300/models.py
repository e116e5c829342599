"""Substitution models and discrete-Gamma rates: the FP64 host-side preparation
of the likelihood path.

Each model returns the eigensystem (U, D, Uinv, mu) of its rate matrix Q, as in
src/Likelihood/SubstitutionModels.jl:13-113; the engine builds
P(t) = U diag(exp(mu t D r)) Uinv on the device from it.  Eigenvector sign and
order do not affect P(t).
"""
from __future__ import annotations

import numpy as np

MCP_TIME_MIN = 1.0e-11   # SubstitutionModels.jl:1
MCP_TIME_MAX = 100.0     # SubstitutionModels.jl:2


def _eigensystem(Q: np.ndarray):
    D, U = np.linalg.eig(Q)
    idx = np.lexsort((D.imag, D.real))          # ascending, like LAPACK via eigen()
    D, U = D[idx], U[:, idx]
    if np.all(D.imag == 0) and np.all(U.imag == 0):
        D, U = D.real.copy(), U.real.copy()
    return U, D, np.linalg.inv(U)


def setmatrix(vec_vals) -> np.ndarray:
    """Symmetric matrix from its upper triangle, column by column
    (SubstitutionModels.jl:106-113): for K=4 the order is
    (1,2), (1,3), (2,3), (1,4), (2,4), (3,4)."""
    v = np.asarray(vec_vals, dtype=np.float64).ravel()
    s = int(round((np.sqrt(8 * len(v) + 1) + 1) / 2))
    if s * (s - 1) // 2 != len(v):
        raise ValueError("setmatrix: length of vector is not triangular")
    Q = np.zeros((s, s))
    iu = [(i, j) for j in range(s) for i in range(j)]
    for k, (i, j) in enumerate(iu):
        Q[i, j] = v[k]
    return Q + Q.T


def Restriction(base_freq, substitution_rates=None):
    """Two-state restriction-site model (SubstitutionModels.jl:13-24)."""
    bf = np.asarray(base_freq, dtype=np.float64)
    if bf.shape != (2,):
        raise AssertionError("Restriction: base_freq must have length 2")
    U = np.array([[bf[1], bf[1]], [bf[1] - 1.0, bf[1]]])
    D = np.array([-1.0, 0.0])
    return U, D, np.linalg.inv(U), 1.0 / (2.0 * bf[0] * bf[1])


def JC(base_freq, substitution_rates=None):
    """Jukes-Cantor (SubstitutionModels.jl:36-50); mu = K/(K-1)."""
    K = len(base_freq)
    Q = np.full((K, K), 1.0 / K)
    np.fill_diagonal(Q, -(K - 1) / K)
    U, D, Uinv = _eigensystem(Q)
    return U, D, Uinv, 1.0 / ((K - 1) / K)


def GTR(base_freq, substitution_rates):
    """General time-reversible (SubstitutionModels.jl:62-74):
    Q_ij = x_ij pi_j, Q_ii = -sum_j Q_ij, mu = 1 / sum of the row sums."""
    bf = np.asarray(base_freq, dtype=np.float64)
    Q = setmatrix(substitution_rates) * bf[np.newaxis, :]
    dia = Q.sum(axis=1)
    Q[np.diag_indices_from(Q)] = -dia
    U, D, Uinv = _eigensystem(Q)
    return U, D, Uinv, 1.0 / dia.sum()


def HKY(base_freq, kappa):
    """HKY85 as the GTR special case with transitions A<->G, C<->T scaled by
    kappa (state order A, C, G, T; setmatrix order gives [1, k, 1, 1, k, 1])."""
    k = float(np.asarray(kappa).ravel()[0])
    return GTR(base_freq, [1.0, k, 1.0, 1.0, k, 1.0])


def freeK(base_freq, substitution_rates):
    """Free K-state model (SubstitutionModels.jl:83-102): Q[j, i] takes the rates
    column by column, skipping the diagonal."""
    r = np.asarray(substitution_rates, dtype=np.float64).ravel()
    K = int(np.ceil(np.sqrt(len(r))))
    Q = np.zeros((K, K))
    mask = ~np.eye(K, dtype=bool)
    Q.T[mask] = r[:K * K - K]            # Q.T[i, j] = Q[j, i], row-major over (i, j)
    dia = Q.sum(axis=1)
    Q[np.diag_indices_from(Q)] = -dia
    U, D, Uinv = _eigensystem(Q)
    with np.errstate(divide="ignore"):          # a 1-state model has no rate (mu = Inf)
        mu = 1.0 / dia.sum()
    return U, D, Uinv, mu


def freeK_equilibrium(substitution_rates) -> np.ndarray:
    """Stationary distribution the reference's freeK PhyloDist constructor uses
    (Phylodist.jl:95-99): first row of U diag(0,..,0,1) Uinv."""
    U, D, Uinv, _ = freeK(None, substitution_rates)
    D = np.zeros(len(D))
    D[-1] = 1.0
    return np.real((U @ np.diag(D) @ Uinv)[0, :])


def calculate_transition(model, rate, mu, time, U, Uinv, D, pi_):
    """Single-branch P(t) with the reference's clipping (SubstitutionModels.jl:119-244).

    JC and Restriction clip: rate*time < MCP_TIME_MIN gives the identity,
    > MCP_TIME_MAX gives the uniform matrix (JC) or every column equal to
    reverse(pi_) (Restriction).  Complex eigensystems return |P|.  PhyloDist's
    likelihood path does not call this (it never clips)."""
    U = np.asarray(U)
    Uinv = np.asarray(Uinv)
    D = np.asarray(D)
    K = U.shape[0]
    if model is JC or model is Restriction:
        t = rate * time
        if t < MCP_TIME_MIN:
            return np.eye(K)
        if t > MCP_TIME_MAX:
            if model is JC:
                return np.full((K, K), 1.0 / len(pi_))
            return np.repeat(np.asarray(pi_, dtype=np.float64)[::-1][:, None], K, axis=1)
        t *= mu
    else:
        t = rate * mu * time
    P = U @ np.diag(np.exp(D * t)) @ Uinv
    if np.iscomplexobj(U) or np.iscomplexobj(Uinv) or np.iscomplexobj(D):
        return np.abs(P)
    return P


# ------------------------------------------------------------------ Gamma rates
def mean_boundaries(alpha, beta, k):
    """Category boundaries (Rates.jl:42-49); the last entry is unused."""
    from scipy.stats import chi2
    nu = (2.0 * alpha) / (2.0 * beta)
    b = np.zeros(k)
    b[:k - 1] = chi2.ppf(np.arange(1, k) / k, nu) / (2.0 * beta)
    return b


def median_boundaries(alpha, beta, k):
    """Category medians (Rates.jl:51-58)."""
    from scipy.stats import chi2
    nu = (2.0 * alpha) / (2.0 * beta)
    return chi2.ppf((2.0 * np.arange(1, k + 1) - 1.0) / (2.0 * k), nu)


def discrete_gamma_rates(alpha, beta, k, method="mean"):
    """Discrete-Gamma category rates as the reference computes them
    (Rates.jl:11-38, Yang 1994).  Note the reference's quantiles use a
    chi-square with (2 alpha)/(2 beta) degrees of freedom; this is kept."""
    from scipy.special import gammainc
    factor = alpha / beta * k
    if method == "median":
        m = median_boundaries(alpha, beta, k)
        return m * (factor / m.sum())
    b = mean_boundaries(alpha, beta, k)
    cdf = np.empty(k)
    cdf[:k - 1] = gammainc(alpha + 1.0, b[:k - 1] * beta)
    cdf[k - 1] = 1.0
    out = np.empty(k)
    out[0] = cdf[0] * factor
    out[1:] = (cdf[1:] - cdf[:-1]) * factor
    return out
