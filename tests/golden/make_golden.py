"""Generate tests/golden/*.npz by running the reference project's own CPU code.

Run where a checkout of the reference project is available, passing its root
directory (required):
    python tests/golden/make_golden.py <reference-checkout>

It imports the reference's flash_sd_kde.reference (FP32 numpy path) and its
FP64 log-space oracle (experiments/error_suite_16d/reference.py, with a stub
for its `gitbud` path helper), evaluates the seeded cases of the reference's
tests (tests/small/test_kde_eval_small.py, tests/large/test_consistency_large.py)
plus the plain-KDE workload (4096 train / 1024 query, N(0, I_16), seed 0,
Silverman bandwidth), and stores inputs and outputs.  The fixtures are what
the oracle restatement (oracle/) is pinned against; nothing at test time
reads the reference checkout.
"""
from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent


def _import_reference(root: str):
    sys.path.insert(0, root)
    gb = types.ModuleType("gitbud")
    gbg = types.ModuleType("gitbud.gitbud")
    gbg.inject_repo_into_sys_path = lambda *a, **k: None
    gb.gitbud = gbg
    sys.modules["gitbud"] = gb
    sys.modules["gitbud.gitbud"] = gbg
    import flash_sd_kde.reference as ref  # noqa: E402
    from experiments.error_suite_16d import reference as ref64  # noqa: E402
    return ref, ref64


def main(root: str) -> None:
    ref, ref64 = _import_reference(root)
    import torch

    def save(name, **arrays):
        np.savez_compressed(OUT / f"{name}.npz", **arrays)
        print("wrote", name, {k: np.shape(v) for k, v in arrays.items()})

    # tests/small/test_kde_eval_small.py:33-44
    rng = np.random.default_rng(0)
    tr = rng.normal(size=256).astype(np.float32)
    qu = rng.normal(size=128).astype(np.float32)
    save("kde1d_seed0", train=tr, queries=qu, h=0.7, density=ref.kde_eval_1d_numpy(qu, tr, 0.7))
    # :47-58
    rng = np.random.default_rng(1)
    tr = rng.normal(size=(256, 16)).astype(np.float32)
    qu = rng.normal(size=(64, 16)).astype(np.float32)
    save("kde16_seed1", train=tr, queries=qu, h=1.2, density=ref.kde_eval_nd_numpy(qu, tr, 1.2))
    # :61-72
    rng = np.random.default_rng(5)
    tr = rng.normal(size=(192, 16)).astype(np.float32)
    qu = rng.normal(size=(48, 16)).astype(np.float32)
    save("kde16_lin_seed5", train=tr, queries=qu, h=1.05, density=ref.kde_eval_nd_linearized_numpy(qu, tr, 1.05))
    # :75-92
    rng = np.random.default_rng(6)
    tr = rng.normal(size=128).astype(np.float32)
    qu = rng.normal(size=64).astype(np.float32)
    save("kde1d_lin_seed6", train=tr, queries=qu, h=0.85, density=ref.kde_eval_1d_linearized_numpy(qu, tr, 0.85))
    # :95-113
    rng = np.random.default_rng(7)
    tr = rng.normal(size=(128, 16)).astype(np.float32)
    qu = rng.normal(size=(32, 16)).astype(np.float32)
    save("kde16_lin_seed7", train=tr, queries=qu, h=1.15, density=ref.kde_eval_nd_linearized_numpy(qu, tr, 1.15))
    # :116-134, :137-172, :175-192 and tests/large/test_consistency_large.py:21-56
    for seed, n, h in ((2, 128, 0.9), (3, 256, 1.1), (4, 128, 1.0), (10, 1024, 1.0)):
        rng = np.random.default_rng(seed)
        tr = rng.normal(size=(n, 16)).astype(np.float32)
        pdf, w, score = ref.empirical_score_nd_numpy(tr, h)
        deb = ref.empirical_sd_kde_transform_nd_numpy(tr, h)
        save(f"score16_seed{seed}", train=tr, h=h, pdf_sum=pdf, weighted=w, score=score, debiased=deb)
    # tests/large/test_consistency_large.py:59-73
    rng = np.random.default_rng(11)
    tr = rng.normal(size=(512, 16)).astype(np.float32)
    qu = rng.normal(size=(1024, 16)).astype(np.float32)
    save("kde16_seed11", train=tr, queries=qu, h=1.1, density=ref.kde_eval_nd_numpy(qu, tr, 1.1))
    # plain 16-D KDE workload: 4096 train then 1024 query from default_rng(0)
    rng = np.random.default_rng(0)
    tr = rng.standard_normal((4096, 16)).astype(np.float32)
    qu = rng.standard_normal((1024, 16)).astype(np.float32)
    h = ref.silverman_bandwidth_nd(tr)
    dens = ref.kde_eval_nd_numpy(qu, tr, h)
    logp64 = ref64.reference_log_density(torch.from_numpy(tr), torch.from_numpy(qu), bandwidth=h,
                                         chunk_cfg={"query_chunk_size": 256, "sample_chunk_size": 4096},
                                         dtype=torch.float64).numpy()
    save("kde16_plain_4096x1024", train=tr, queries=qu, h=h, density=dens, log_density_fp64=logp64,
         silverman_fp64=ref64.silverman_diag_bandwidth(torch.from_numpy(tr)))
    # 1-D score and one-step 1-D debias (reference.py:83-141); bandwidths
    rng = np.random.default_rng(12)
    x1 = rng.normal(size=2000).astype(np.float32)
    q1 = np.linspace(-3, 3, 257).astype(np.float32)
    h1 = ref.silverman_bandwidth(x1)
    np.random.seed(0)
    mix = ref.sample_from_mixture(3000, ref.mixture_params_list[0]).astype(np.float32)
    deb1, hdeb = ref.one_step_debiased_data_emp_kde(mix)
    save("kde1d_score_seed12", train=x1, queries=q1, h=h1, score=ref.kde_score_eval(q1, x1, h1),
         pdf=ref.kde_pdf_eval(q1, x1, h1), mixture=mix, debiased_1d=deb1, h_sdkde=hdeb)
    # bandwidth rules on skewed / heavy-tailed data
    rng = np.random.default_rng(13)
    xs = (rng.standard_t(5, size=(3001, 16)) * 10 ** rng.uniform(-1, 1, size=16) + 100).astype(np.float32)
    save("silverman_seed13", data=xs, h_nd=ref.silverman_bandwidth_nd(xs), h_1d=ref.silverman_bandwidth(xs[:, 3]))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference-checkout>")
    main(sys.argv[1])
