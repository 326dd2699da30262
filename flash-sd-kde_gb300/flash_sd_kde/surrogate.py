"""Learned surrogate of the exact 16-D KDE log-density (no counterpart in the
reference; it serves bulk queries of a fitted Flash-SD-KDE model).

    sur = SurrogateKDE(members=4).fit(debiased_data, h)
    logp, served = sur.score_samples(queries, return_served=True)

* Training pairs: queries = data points + N(0, (noise_scale h)^2 I), targets =
  the exact normalised log-density from the tensor-core KDE kernel.
* Model: an ensemble of MLPs 16 -> 256 -> 256 -> 256 -> 1 (SiLU, bf16
  weights and activations, FP32 accumulation) on whitened inputs, fitted to
  the residual of log p after a Gaussian base a + b r^2 (r the whitened
  radius) that carries the tails; trained with the library's own forward,
  backward and AdamW kernels (fsk_mlp_fwd / _bwd / _adam).
* Serving: tensor-core inference of every member (fsk_mlp_infer), then the
  gate: a query is served by the surrogate when the members agree
  (max - min <= spread_tol, in log units) and its whitened radius is inside
  the training distribution (r^2 <= the radius_quantile of the training
  queries); every other query falls back to the exact KDE kernel, which is
  also what measures the surrogate's error.
* Checkpoints: save(path) writes the fitted state (support data and
  bandwidth, whitening, base, FP32 master weights, AdamW moments, step count,
  schedule length, the shuffling generator's state); SurrogateKDE.load(path)
  rebuilds a model that serves the same values, and resume(epochs) continues
  its training (the generated training pairs are rebuilt from the seed).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch

from fsk import ops
from globals import ND_FEATURES

MLP_H = 256


def _init_member(rng: np.random.Generator) -> np.ndarray:
    """Weights uniform in +-sqrt(6/fan_in) (+-1/sqrt(256) for the output
    vector), zero biases; the parameter layout of include/fsk.h."""
    parts = []
    for shape, bound in (((MLP_H, ND_FEATURES), math.sqrt(6.0 / ND_FEATURES)), ((MLP_H,), 0.0),
                         ((MLP_H, MLP_H), math.sqrt(6.0 / MLP_H)), ((MLP_H,), 0.0),
                         ((MLP_H, MLP_H), math.sqrt(6.0 / MLP_H)), ((MLP_H,), 0.0),
                         ((MLP_H,), 1.0 / math.sqrt(MLP_H)), ((1,), 0.0)):
        parts.append(rng.uniform(-bound, bound, size=shape).ravel() if bound > 0 else np.zeros(int(np.prod(shape))))
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == ops.MLP_PARAMS
    return p


@dataclass
class SurrogateKDE:
    members: int = 4
    epochs: int = 8
    batch_size: int = 8192
    lr: float = 2e-3
    lr_final: float = 2e-5
    weight_decay: float = 0.0
    spread_tol: float = 0.03
    radius_quantile: float = 0.999
    noise_scale: float = 1.0
    seed: int = 0
    device: str | torch.device = "cuda"
    history: list = field(default_factory=list)

    # ---- exact targets ---------------------------------------------------------
    def _exact_logp(self, queries: torch.Tensor, chunk: int = 1 << 20) -> torch.Tensor:
        n = self.data_.shape[0]
        h = self.bandwidth_
        norm = 1.0 / ((2.0 * math.pi) ** (ND_FEATURES / 2.0) * h ** ND_FEATURES * n)
        out = torch.empty(queries.shape[0], dtype=torch.float32, device=queries.device)
        for s in range(0, queries.shape[0], chunk):
            # exact log-density also where the FP32 sum underflows (far queries)
            ops.kde16_sum(queries[s:s + chunk], self.data_, h, out_scale=norm, log_exact=True,
                          out=out[s:s + chunk])
        return out

    def _radius2(self, x: torch.Tensor) -> torch.Tensor:
        return (((x - self.in_mean_) * self.in_inv_std_) ** 2).sum(1)

    # ---- fit -------------------------------------------------------------------
    def _training_pairs(self, n_pairs, queries, log_density):
        """Training queries and their exact log-densities; generated pairs come
        from the seeded generator, which then shuffles the epochs."""
        dev = ops._device(self.device)
        g = torch.Generator(device=dev)
        g.manual_seed(self.seed)
        if queries is None:
            idx = torch.randint(self.data_.shape[0], (n_pairs,), generator=g, device=dev)
            noise = torch.randn((n_pairs, ND_FEATURES), generator=g, device=dev)
            q = self.data_[idx] + noise * (self.noise_scale * self.bandwidth_)
        else:
            q = ops.as_matrix(queries, dev, ND_FEATURES)
        logp = self._exact_logp(q) if log_density is None else ops.as_vector(log_density, dev)
        ops.device_status(dev)
        keep = torch.isfinite(logp)      # a query whose FP32 kernel sum underflows teaches nothing
        if not bool(keep.all()):
            q, logp = q[keep].contiguous(), logp[keep].contiguous()
        if q.shape[0] == 0:
            raise ValueError("no training query has a finite log-density.")
        return q, logp, g

    def fit(self, data, bandwidth: float, *, n_pairs: int = 4_000_000, queries=None, log_density=None,
            verbose: bool = False) -> "SurrogateKDE":
        if bandwidth <= 0:
            raise ValueError("bandwidth must be positive.")
        dev = ops._device(self.device)
        self.data_ = ops.as_matrix(data, dev, ND_FEATURES)
        if self.data_.shape[0] == 0:
            raise ValueError("data must be non-empty.")
        self.bandwidth_ = float(bandwidth)
        self.n_pairs_ = int(n_pairs) if queries is None else None
        q, logp, g = self._training_pairs(n_pairs, queries, log_density)
        # whitening and the Gaussian base a + b r^2 (least squares)
        self.in_mean_ = q.mean(0).contiguous()
        self.in_inv_std_ = (1.0 / q.std(0).clamp_min(1e-12)).contiguous()
        r2 = self._radius2(q)
        r2d, lpd = r2.double(), logp.double()
        rm, lm = r2d.mean(), lpd.mean()
        var = ((r2d - rm) ** 2).mean()
        b = ((r2d - rm) * (lpd - lm)).mean() / var if float(var) > 0 else torch.zeros((), dtype=torch.float64)
        self.base_a_, self.base_b_ = float(lm - b * rm), float(b)
        resid = logp - (self.base_a_ + self.base_b_ * r2)
        self.out_shift_ = float(resid.mean())
        self.out_scale_ = float(resid.std().clamp_min(1e-12))
        target = ((resid - self.out_shift_) / self.out_scale_).contiguous()
        self.r2_max_ = float(torch.quantile(r2[: min(r2.numel(), 1 << 24)].float(), self.radius_quantile))
        # parameters, optimiser state
        rng = np.random.default_rng(self.seed)
        self.params_ = torch.from_numpy(np.concatenate([_init_member(rng) for _ in range(self.members)])).to(dev)
        self.adam_m_ = torch.zeros_like(self.params_)
        self.adam_v_ = torch.zeros_like(self.params_)
        self.step_ = 0
        self.total_steps_ = max(1, self.epochs * (q.shape[0] // min(self.batch_size, q.shape[0])))
        self._train(q, target, g, self.epochs, verbose)
        return self

    def _train(self, q, target, g, epochs: int, verbose: bool) -> None:
        """`epochs` epochs of AdamW from the current state; the cosine learning
        rate runs over total_steps_ (continued, not restarted, by resume)."""
        dev = ops._device(self.device)
        params, m, v = self.params_, self.adam_m_, self.adam_v_
        grads = torch.empty_like(params)
        B = min(self.batch_size, q.shape[0])
        ws = ops.mlp_train_workspace(self.members, B, dev)
        y = torch.empty((self.members, B), dtype=torch.float32, device=dev)
        dy = torch.empty_like(y)
        loss = torch.zeros(1, dtype=torch.float64, device=dev)
        steps_per_epoch = q.shape[0] // B
        total = self.total_steps_
        for epoch in range(epochs):
            perm = torch.randperm(q.shape[0], generator=g, device=dev)
            loss.zero_()
            for s in range(steps_per_epoch):
                sel = perm[s * B:(s + 1) * B]
                xb = q[sel].contiguous()
                tb = target[sel].contiguous()
                ops.mlp_fwd(params, self.members, xb, self.in_mean_, self.in_inv_std_, ws, y)
                ops.mlp_mse(y, tb, dy, loss)
                ops.mlp_bwd(params, self.members, B, dy, ws, grads)
                self.step_ += 1
                t = min(self.step_, total)
                lr = self.lr_final + 0.5 * (self.lr - self.lr_final) * (1.0 + math.cos(math.pi * t / total))
                ops.mlp_adam(params, grads, m, v, self.step_, lr, weight_decay=self.weight_decay)
            ep_loss = float(loss.item()) / max(1, steps_per_epoch) / self.members
            self.history.append(ep_loss)
            if verbose:
                print(f"epoch {len(self.history) - 1}: mse (normalised) {ep_loss:.3e}", flush=True)
        ops.device_status(dev)
        self.gen_state_ = g.get_state()
        self.packed_ = ops.mlp_pack(params, self.members, self.in_mean_, self.in_inv_std_, self.out_scale_,
                                    self.out_shift_)

    # ---- checkpoints -------------------------------------------------------------
    _CONFIG = ("members", "epochs", "batch_size", "lr", "lr_final", "weight_decay", "spread_tol",
               "radius_quantile", "noise_scale", "seed")
    _TENSORS = ("data_", "in_mean_", "in_inv_std_", "params_", "adam_m_", "adam_v_")
    _SCALARS = ("bandwidth_", "base_a_", "base_b_", "out_shift_", "out_scale_", "r2_max_", "step_",
                "total_steps_", "n_pairs_")

    def state_dict(self) -> dict:
        """Everything needed to serve and to continue training (CPU tensors)."""
        if not hasattr(self, "params_"):
            raise RuntimeError("the surrogate is not fitted.")
        return {"format": "fsk-surrogate-1",
                "config": {k: getattr(self, k) for k in self._CONFIG},
                "tensors": {k: getattr(self, k).detach().cpu() for k in self._TENSORS},
                "scalars": {k: getattr(self, k) for k in self._SCALARS},
                "history": list(self.history),
                "gen_state": self.gen_state_.cpu()}

    def save(self, path) -> None:
        torch.save(self.state_dict(), path)

    @classmethod
    def load(cls, path, device="cuda") -> "SurrogateKDE":
        st = torch.load(path, map_location="cpu", weights_only=True)
        if not isinstance(st, dict) or st.get("format") != "fsk-surrogate-1":
            raise ValueError("not a surrogate checkpoint.")
        sur = cls(device=device, history=list(st["history"]), **st["config"])
        dev = ops._device(device)
        for k, t in st["tensors"].items():
            setattr(sur, k, t.to(dev).contiguous())
        for k, v in st["scalars"].items():
            setattr(sur, k, v)
        sur.gen_state_ = st["gen_state"]
        sur.packed_ = ops.mlp_pack(sur.params_, sur.members, sur.in_mean_, sur.in_inv_std_, sur.out_scale_,
                                   sur.out_shift_)
        return sur

    def resume(self, epochs: int, *, queries=None, log_density=None, verbose: bool = False) -> "SurrogateKDE":
        """Continue training for `epochs` more epochs from the current (or
        loaded) weights and AdamW state.  Generated training pairs are rebuilt
        from the seed; a model fitted on given queries needs them again."""
        if not hasattr(self, "params_"):
            raise RuntimeError("the surrogate is not fitted.")
        if self.n_pairs_ is None and queries is None:
            raise ValueError("this surrogate was fitted on given queries: pass them (and log_density) again.")
        q, logp, g = self._training_pairs(self.n_pairs_, queries, log_density)
        g.set_state(self.gen_state_)
        r2 = self._radius2(q)
        resid = logp - (self.base_a_ + self.base_b_ * r2)
        target = ((resid - self.out_shift_) / self.out_scale_).contiguous()
        self._train(q, target, g, epochs, verbose)
        return self

    # ---- serving -----------------------------------------------------------------
    def predict(self, queries) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
        """(log-density estimate, member spread, served mask) from the surrogate alone."""
        dev = ops._device(self.device)
        x = ops.as_matrix(queries, dev, ND_FEATURES)
        y = ops.mlp_infer(self.packed_, self.members, x)
        return ops.mlp_combine(y, x, self.in_mean_, self.in_inv_std_, self.base_a_, self.base_b_, self.spread_tol,
                               self.r2_max_)

    def score_samples(self, queries, *, return_served: bool = False):
        """log-density of every query: surrogate where the gate serves it, the
        exact KDE elsewhere."""
        dev = ops._device(self.device)
        x = ops.as_matrix(queries, dev, ND_FEATURES)
        logp, _, served = self.predict(x)
        miss = torch.nonzero(served == 0).squeeze(1)
        if miss.numel():
            logp[miss] = self._exact_logp(x[miss].contiguous())
        if return_served:
            return logp, served.bool()
        return logp
