"""Ground-state energy of the periodic spin-1/2 Heisenberg ring by the Bethe
ansatz — an exact method independent of the oracle and of libsed, used to pin
the chain workloads' eigenvalues.

Method (Bethe 1931; logarithmic form of the Bethe equations as in Karbach &
Mueller, Computers in Physics 11, 36 (1997)): for H = J sum_i S_i . S_{i+1}
on N sites with M = N/2 flipped spins, the ground state has rapidities
lambda_1..lambda_M solving

    2 N arctan(2 lambda_j) = 2 pi I_j + sum_{k != j} 2 arctan(lambda_j - lambda_k),

with I_j = -(M-1)/2, ..., (M-1)/2, and energy

    E = J N / 4 - J sum_j 2 / (1 + 4 lambda_j^2).

The equations are solved by Newton's method from the free-magnon guess
lambda_j = tan(pi I_j / N) / 2. The workloads use the 2-site matrix of
sigma . sigma = 4 S . S, so their energies are 4 E.
"""
import numpy as np


def heisenberg_ring_e0(n: int, tol: float = 1e-15, max_iter: int = 100) -> float:
    """Ground-state energy of the n-site ring in sigma.sigma units (n even)."""
    if n % 2:
        raise ValueError("the ring needs an even number of sites")
    m = n // 2
    I = np.arange(m) - (m - 1) / 2.0
    lam = np.tan(np.pi * I / n) / 2.0
    for _ in range(max_iter):
        d = lam[:, None] - lam[None, :]
        F = 2 * n * np.arctan(2 * lam) - 2 * np.pi * I - 2 * np.arctan(d).sum(axis=1)
        K = 2.0 / (1.0 + d * d)
        np.fill_diagonal(K, 0.0)
        Jm = K.copy()
        np.fill_diagonal(Jm, 4 * n / (1 + 4 * lam * lam) - K.sum(axis=1))
        step = np.linalg.solve(Jm, F)
        lam = lam - step
        if np.max(np.abs(step)) <= tol * max(1.0, np.max(np.abs(lam))):
            break
    else:
        raise RuntimeError("Bethe equations did not converge")
    e_ss = n / 4.0 - np.sum(2.0 / (1.0 + 4 * lam * lam))
    return 4.0 * e_ss
