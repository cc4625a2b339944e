"""Helpers for the GPU tests: numpy <-> torch device buffers, bit for bit."""

import numpy as np
import torch

_VIEW = {np.dtype(np.uint32): (np.int32, torch.int32), np.dtype(np.uint64): (np.int64, torch.int64),
         np.dtype(np.int32): (np.int32, torch.int32), np.dtype(np.int64): (np.int64, torch.int64),
         np.dtype(np.uint8): (np.uint8, torch.uint8)}


def dev(a: np.ndarray) -> torch.Tensor:
    """Copy a numpy integer array to the GPU, reinterpreting unsigned types as signed of the same width."""
    a = np.ascontiguousarray(a)
    npv, _ = _VIEW[a.dtype]
    return torch.from_numpy(a.view(npv).copy()).cuda()


def host(t: torch.Tensor, dtype) -> np.ndarray:
    """Copy a device tensor back and reinterpret as dtype (same width)."""
    return t.cpu().numpy().view(dtype)


def per_key_success(keys: np.ndarray, flags: np.ndarray) -> dict:
    """Number of successful operations per distinct key."""
    u, inv = np.unique(keys, return_inverse=True)
    s = np.bincount(inv, weights=flags.astype(np.int64), minlength=len(u)).astype(np.int64)
    return dict(zip(u.tolist(), s.tolist()))
