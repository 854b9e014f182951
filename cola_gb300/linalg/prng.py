"""The reference's keyed random numbers for the torch backend (cola/backends/torch_fns.py:154, 222-241).

``PRNGKey(x)`` and ``next_key(key)`` are SHA-256 hashes reduced mod 2**32-1; ``randn`` seeds a
generator with the key and draws standard normals.  Probes and start vectors are drawn on the
host CPU generator (what the reference does for CPU tensors) and then moved to the device, so a
GPU run sees exactly the vectors a CPU reference run sees.
"""
from __future__ import annotations

import hashlib

import torch


def sha_hash(n: int) -> int:
    n_bytes = n.to_bytes((n.bit_length() + 7) // 8, "big")
    h = int.from_bytes(hashlib.sha256(n_bytes).digest(), "big")
    return int(h % (2**32 - 1))


def PRNGKey(x: int) -> int:
    return sha_hash(x)


def next_key(key: int) -> int:
    return sha_hash(key)


def randn(*shape, dtype=torch.float32, device=None, key=None) -> torch.Tensor:
    if key is None:
        key = PRNGKey(0)
    g = torch.Generator(device="cpu")
    g.manual_seed(int(key))
    z = torch.randn(*shape, dtype=dtype, generator=g)
    return z.to(device) if device is not None else z
