"""Shared helpers for the test suite (golden fixtures, input recipes)."""
from __future__ import annotations

import json
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
SEED = 12345


def load_manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def cases(op, include_skipped=False):
    m = load_manifest()
    out = []
    for c in m["ops"][op]:
        if "skipped" in c and not include_skipped:
            continue
        out.append(c)
    return out


def read_bin(op, fname):
    return np.fromfile(os.path.join(GOLDEN, op, fname), dtype=np.float32)


def as_complex(flat):
    return flat.view(np.complex64)


def regenerate(op, cfg):
    """Inputs built with the same recipe as the reference's gen_data.py.

    Used for cases whose fixture files are too large to commit: the values
    need not match the reference bit for bit, only follow its distribution
    and layout, because the expected output is then computed by the FP64
    oracle from these very inputs.
    """
    import torch

    torch.manual_seed(SEED)
    b = cfg.get("batch", 1)
    if op == "fft1_d":
        x = torch.randn(b, cfg["n"], dtype=torch.complex64)
        return x.numpy().reshape(-1)
    if op == "rfft1_d":
        return torch.randn(b * cfg["n"]).float().numpy()
    if op == "irfft1_d":
        nb = cfg["n"] // 2 + 1
        if cfg.get("nyquist_only"):
            x = torch.zeros(b, nb, dtype=torch.complex64)
            x[:, -1] = 1.0
        else:
            x = torch.randn(b, nb, dtype=torch.complex64)
        return x.numpy().reshape(-1)
    x = torch.randn(b, cfg["fft_x"], cfg["fft_y"], dtype=torch.complex64)
    return x.numpy().reshape(-1)
