"""Seeded synthetic inputs for the benchmark configurations (numpy PCG64, so
identical on every host).  No public dataset is involved; these stand in for
the workloads the project measures.

plain_kde_16d    4096 train / 1024 query, N(0, I_16), one generator seed 0
                 (train drawn first).
gmm8_16d         8-component Gaussian mixture: weights ~ Dirichlet(1_8),
                 means ~ N(0, 4 I), covariances A A^T / 16 + 0.1 I with A
                 having N(0, 1) entries (parameters seed 0).
student_t_16d    multivariate Student-t (nu = 5), per-axis scale 10^U(-1, 1),
                 offset +100 (distance-cancellation stress).
lowrank_16d      z diag(k^-1/2), k = 1..16, z ~ N(0, I).
gmm3_1d          1-D mixture: means (-2, 0, 3), std (0.5, 1, 0.3),
                 weights (0.3, 0.5, 0.2); grid queries on [-5, 6].
gm_diag_16d      the error-suite smoke configuration: 4-component diagonal
                 mixture, means N(0, I) * 2, unit per-axis std, equal weights,
                 8192 train / 4096 test, standardised by the train statistics.
"""
from __future__ import annotations

import numpy as np

D = 16


def plain_kde_16d(n_train: int = 4096, n_query: int = 1024, seed: int = 0):
    rng = np.random.default_rng(seed)
    train = rng.standard_normal((n_train, D)).astype(np.float32)
    query = rng.standard_normal((n_query, D)).astype(np.float32)
    return train, query


class GMM16:
    """8-component full-covariance mixture in 16-D."""

    def __init__(self, seed: int = 0, k: int = 8):
        rng = np.random.default_rng(seed)
        self.weights = rng.dirichlet(np.ones(k))
        self.means = rng.normal(0.0, 2.0, size=(k, D))
        a = rng.standard_normal((k, D, D))
        self.cov = a @ a.transpose(0, 2, 1) / 16.0 + 0.1 * np.eye(D)
        self.chol = np.linalg.cholesky(self.cov)

    def sample(self, n: int, seed: int) -> np.ndarray:
        rng = np.random.default_rng(seed)
        comp = rng.choice(len(self.weights), size=n, p=self.weights)
        z = rng.standard_normal((n, D))
        x = self.means[comp] + np.einsum("nij,nj->ni", self.chol[comp], z)
        return x.astype(np.float32)

    def log_density(self, x: np.ndarray) -> np.ndarray:
        """True mixture log-density (FP64)."""
        x = np.asarray(x, dtype=np.float64)
        out = []
        for w, mu, L in zip(self.weights, self.means, self.chol):
            y = np.linalg.solve(L, (x - mu).T).T
            logdet = 2.0 * np.log(np.diag(L)).sum()
            out.append(np.log(w) - 0.5 * (y * y).sum(1) - 0.5 * logdet - 0.5 * D * np.log(2 * np.pi))
        out = np.stack(out, 1)
        m = out.max(1)
        return m + np.log(np.exp(out - m[:, None]).sum(1))


def gmm8_16d(n_train: int = 65536, n_query: int = 65536):
    g = GMM16(seed=0)
    return g.sample(n_train, seed=1), g.sample(n_query, seed=2)


def student_t_16d(n: int, seed: int, scale_seed: int = 3, nu: float = 5.0) -> np.ndarray:
    scale = 10.0 ** np.random.default_rng(scale_seed).uniform(-1.0, 1.0, size=D)
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((n, D))
    chi = rng.chisquare(nu, size=(n, 1))
    return (z / np.sqrt(chi / nu) * scale + 100.0).astype(np.float32)


def lowrank_16d(n: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((n, D))
    return (z * (np.arange(1, D + 1) ** -0.5)).astype(np.float32)


def gmm3_1d(n: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    comp = rng.choice(3, size=n, p=[0.3, 0.5, 0.2])
    mu = np.array([-2.0, 0.0, 3.0])[comp]
    sd = np.array([0.5, 1.0, 0.3])[comp]
    return (mu + sd * rng.standard_normal(n)).astype(np.float32)


def grid_1d(m: int, lo: float = -5.0, hi: float = 6.0) -> np.ndarray:
    return np.linspace(lo, hi, m).astype(np.float32)


def gm_diag_16d(n_train: int = 8192, n_test: int = 4096, seed: int = 0, n_components: int = 4,
                component_std: float = 1.0, mean_scale: float = 2.0):
    """Train and test points of the reference's error-suite smoke run
    (configs/error_suite_16d/smoke.yaml; recipe of
    experiments/error_suite_16d/datasets.py:34-42 and :55-78, sampling of
    truth.py:57-63): component means ~ N(0, I) * mean_scale drawn with `seed`,
    equal weights, per-axis std `component_std`; the train set is sampled
    with `seed` and the test set with `seed + 1` (component index, then the
    Gaussian offsets); both are standardised by the train mean and unbiased
    per-axis std.  Returns float32 (train, test)."""
    rng = np.random.default_rng(seed)
    means = rng.normal(size=(n_components, D)) * mean_scale
    weights = np.full(n_components, 1.0 / n_components)

    def draw(count: int, s: int) -> np.ndarray:
        g = np.random.default_rng(s)
        comp = g.choice(n_components, size=count, p=weights)
        return g.normal(size=(count, D)) * component_std + means[comp]

    train, test = draw(n_train, seed), draw(n_test, seed + 1)
    mu, sd = train.mean(axis=0), train.std(axis=0, ddof=1)
    sd = np.where(sd <= 0, 1.0, sd)
    return ((train - mu) / sd).astype(np.float32), ((test - mu) / sd).astype(np.float32)


def shard(count: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous [start, stop) slice of `count` rows owned by `rank`."""
    base, extra = divmod(count, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)
