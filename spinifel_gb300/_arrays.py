"""Array plumbing between the reference-facing API (numpy in, numpy out, as
the reference's CPU path and pybind11 module do) and torch CUDA tensors."""
from __future__ import annotations

import numpy as np
import torch


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("spinifel_gb300 needs a CUDA device (there is no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def to_dev(a, dtype=torch.float32) -> torch.Tensor:
    if isinstance(a, torch.Tensor):
        return a.to(device=device(), dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=device())


def is_torch(a) -> bool:
    return isinstance(a, torch.Tensor)


def like_input(t: torch.Tensor, ref):
    """Return t as the same array family as ref (torch stays on device)."""
    if is_torch(ref):
        return t
    return t.detach().cpu().numpy()
