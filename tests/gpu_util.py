"""Helpers shared by the GPU tests: column-major device copies of numpy arrays."""

import numpy as np

TORCH_DTYPES = None


def torch_dtype(dt):
    import torch

    return {np.dtype(np.float16): torch.float16, np.dtype(np.float32): torch.float32,
            np.dtype(np.float64): torch.float64}[np.dtype(dt)]


def to_dev(X, dtype, dev, ld=None):
    """Column-major device copy of X (shape (r, c), strides (1, ld))."""
    import torch

    X = np.asarray(X)
    r, c = X.shape
    ld = ld or max(r, 1)
    buf = torch.zeros((max(c, 1), ld), dtype=torch_dtype(dtype), device=dev)
    if r and c:
        buf[:c, :r] = torch.from_numpy(np.ascontiguousarray(X.T.astype(dtype)))
    return buf.T[:r, :c]


def to_host(Xd):
    return Xd.detach().cpu().numpy().astype(np.float64)
