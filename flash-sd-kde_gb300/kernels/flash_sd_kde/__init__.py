"""Flash SD-KDE kernels (GB300): same exports as the reference's
kernels/flash_sd_kde/__init__.py:16-25."""

from .empirical import (
    emp_score_16d_flash_sd_kde,
    empirical_sd_kde_triton,
    empirical_sd_kde_triton_nd,
)
from .kde import (
    gaussian_kde_score_triton,
    gaussian_kde_triton,
    gaussian_kde_triton_nd,
    gaussian_kde_triton_nd_numpy,
    gaussian_kde_triton_numpy,
)

__all__ = [
    "emp_score_16d_flash_sd_kde",
    "empirical_sd_kde_triton",
    "empirical_sd_kde_triton_nd",
    "gaussian_kde_score_triton",
    "gaussian_kde_triton",
    "gaussian_kde_triton_nd",
    "gaussian_kde_triton_nd_numpy",
    "gaussian_kde_triton_numpy",
]
