"""Helpers shared by the tests: device round trips of uint64 arrays."""
from __future__ import annotations

import numpy as np


def to_dev(a: np.ndarray, device="cuda"):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).to(device)


def to_host(t) -> np.ndarray:
    return t.cpu().numpy().view(np.uint64)
