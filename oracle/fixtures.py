"""Seeded inputs of the reference tests and of the benchmark configurations.

TEST INFRASTRUCTURE ONLY (used by tests/, the smoke check and bench.py's
input generation for the oracle legs).

drand48_fixture restates the decomposition-independent fixture of the
reference tests: element (row, col) of an m-row matrix is the first
drand48() draw after srand48(99900 + (row + col*m)*61)
(test/QR/test_hh_recon.cxx:52,70-85; test/QR/test_qr_2d.cxx:87-103 subtracts
0.5).  srand48/drand48 are the POSIX 48-bit LCG: X0 = (seed_lo32 << 16) |
0x330E, X1 = (0x5DEECE66D * X0 + 0xB) mod 2^48, value = X1 / 2^48.
"""
import numpy as np

_A48 = np.uint64(0x5DEECE66D)
_C48 = np.uint64(0xB)
_M48 = np.uint64((1 << 48) - 1)


def drand48_first(seeds):
    """First drand48() value after srand48(seed), vectorised over int64 seeds."""
    s = np.asarray(seeds, dtype=np.int64).astype(np.uint64) & np.uint64(0xFFFFFFFF)
    x0 = (s << np.uint64(16)) | np.uint64(0x330E)
    x1 = (_A48 * x0 + _C48) & _M48
    return x1.astype(np.float64) / float(1 << 48)


def drand48_fixture(m, n, offset=0.0, seed_offset=99900):
    """m x n matrix of the reference tests' srand48 fixture, minus `offset`."""
    row = np.arange(m, dtype=np.int64)[:, None]
    col = np.arange(n, dtype=np.int64)[None, :]
    seeds = seed_offset + (row + col * m) * 61
    return drand48_first(seeds) - offset


def gaussian(m, n, seed):
    """m x n N(0,1) matrix: element (i, j) is draw i*n+j of PCG64(seed)."""
    rng = np.random.default_rng(seed)
    return rng.standard_normal((m, n))


def haar(n, rng, ncols=None):
    """Haar-distributed orthonormal columns: Q*diag(sign(diag R)) of a Gaussian QR (Mezzadri 2007)."""
    G = rng.standard_normal((n, ncols or n))
    Q, R = np.linalg.qr(G)
    return Q * np.sign(np.diag(R))[None, :]


def batched_problems(count, seed=3, m_lo=256, m_hi=262144, widths=(8, 16, 32, 64, 128)):
    """Uneven least-squares problem set: per-problem PCG64 streams from
    SeedSequence(seed).spawn(count); m_i = round(exp(U(ln m_lo, ln m_hi))),
    n_i uniform over `widths` (m_i >= n_i enforced), A_i and b_i ~ N(0, 1).
    Returns a list of (m, n, generator) so callers can draw A_i, b_i lazily."""
    out = []
    for ss in np.random.SeedSequence(seed).spawn(count):
        rng = np.random.default_rng(ss)
        m = int(round(np.exp(rng.uniform(np.log(m_lo), np.log(m_hi)))))
        n = int(rng.choice(widths))
        out.append((max(m, n), n, rng))
    return out


def svd_matrix(m, n, seed, sigma_min):
    """A = U diag(sigma) V^T, U (m x n) and V (n x n) Haar from PCG64(seed), U drawn first,
    sigma log-spaced from 1 to sigma_min."""
    rng = np.random.default_rng(seed)
    U = haar(m, rng, n)
    V = haar(n, rng)
    s = np.logspace(0, np.log10(sigma_min), n)
    return (U * s[None, :]) @ V.T
