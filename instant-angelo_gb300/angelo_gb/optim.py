"""AdamW of the reference's optimizer config (systems/utils.py:314-325:
torch.optim.AdamW(lr, betas, eps), default weight decay 0.01, per-group lr)
with the update as one libangelo_gb streaming pass per large parameter
(angelo_adamw_step) and one launch for all small ones (angelo_adamw_step_multi).  Same parameter groups, hyper-parameters and state
names (step, exp_avg, exp_avg_sq) as torch.optim.AdamW, so state dicts load
either way.  Parameters must be float32 CUDA tensors; there is no other
path."""
from __future__ import annotations

import ctypes

import torch

from ._lib import call
from .ops import _p, _s


class AdamW(torch.optim.Optimizer):
    def __init__(self, params, lr=1e-3, betas=(0.9, 0.999), eps=1e-8, weight_decay=1e-2):
        if lr < 0 or eps < 0 or not (0.0 <= betas[0] < 1.0 and 0.0 <= betas[1] < 1.0):
            raise ValueError(f"invalid AdamW hyper-parameters lr={lr} betas={betas} eps={eps}")
        super().__init__(params, dict(lr=lr, betas=tuple(betas), eps=eps,
                                      weight_decay=weight_decay))

    # tensors below this size share one multi-tensor launch per step
    SMALL = 1 << 16

    @torch.no_grad()
    def step(self, closure=None):
        loss = None
        if closure is not None:
            with torch.enable_grad():
                loss = closure()
        small = []
        for group in self.param_groups:
            b1, b2 = group["betas"]
            for p in group["params"]:
                if p.grad is None:
                    continue
                if p.dtype != torch.float32 or not p.is_cuda or p.grad.is_sparse:
                    raise TypeError("AdamW: parameters must be dense float32 CUDA tensors")
                if not p.is_contiguous():
                    raise ValueError("AdamW: parameters must be contiguous")
                st = self.state[p]
                if not st:
                    st["step"] = torch.zeros((), dtype=torch.float32)
                    st["exp_avg"] = torch.zeros_like(p, memory_format=torch.contiguous_format)
                    st["exp_avg_sq"] = torch.zeros_like(p, memory_format=torch.contiguous_format)
                st["step"] += 1
                t = float(st["step"])
                g = p.grad if p.grad.is_contiguous() else p.grad.contiguous()
                hp = (float(group["lr"]), float(b1), float(b2), float(group["eps"]),
                      float(group["weight_decay"]), 1.0 - b1 ** t, 1.0 - b2 ** t)
                if p.numel() < self.SMALL:
                    small.append((p, g, st, hp))
                    continue
                call("angelo_adamw_step", _p(p), _p(g), _p(st["exp_avg"]), _p(st["exp_avg_sq"]),
                     p.numel(), *hp, _s(p.device),
                     launches=1 if p.numel() % 4 == 0 else 2, units=dict(n=p.numel()))
        by_dev = {}
        for item in small:
            by_dev.setdefault(item[0].device, []).append(item)
        for dev, items in by_dev.items():
            n = len(items)
            ptrs = lambda ts: (ctypes.c_void_p * n)(*[x.data_ptr() for x in ts])
            f32 = lambda j: (ctypes.c_float * n)(*[it[3][j] for it in items])
            call("angelo_adamw_step_multi", n, ptrs([it[0] for it in items]),
                 ptrs([it[1] for it in items]), ptrs([it[2]["exp_avg"] for it in items]),
                 ptrs([it[2]["exp_avg_sq"] for it in items]),
                 (ctypes.c_int64 * n)(*[it[0].numel() for it in items]), *[f32(j) for j in range(7)],
                 _s(dev), launches=(n + 31) // 32, units=dict(n=sum(it[0].numel() for it in items)))
        return loss
