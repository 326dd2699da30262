"""Flash-SD-KDE drop-in API on GB300 (same exports as the reference's
flash_sd_kde/__init__.py:9-15)."""
from flash_sd_kde.kde import (
    emp_sd_kde_fit_transform,
    kde_eval,
    kde_eval_linearized,
    kde_eval_linearized_nonfused,
)
from flash_sd_kde.estimator import FlashSDKDE

__all__ = [
    "FlashSDKDE",
    "emp_sd_kde_fit_transform",
    "kde_eval",
    "kde_eval_linearized",
    "kde_eval_linearized_nonfused",
]
