"""Spatial FBP filters (deeprecon/deeprecon/torch/projector/filter.py:8-30).

``ramp`` is the band-limited Ram-Lak kernel sampled on the detector grid
(zero at even offsets n, -1/(pi^2 d^2 n^2) at odd offsets, 1/(4 d^2) at 0);
``sheeplogan`` is the Shepp-Logan kernel -2/(pi^2 d^2 (4 n^2 - 1)).  Both
have 2*num_det - 1 taps centred at index num_det - 1.  The arithmetic uses
the same torch type promotion as the reference (an int64 offset grid times a
Python float, evaluated in the default float dtype) so the taps are
bit-identical.
"""
from __future__ import annotations

import torch

FILTERS = ("ramp", "sheeplogan")


def _offsets(num_det: int) -> torch.Tensor:
    return torch.arange(num_det * 2 - 1) - num_det + 1


def ramp(num_det, det_size, dtype=None) -> torch.Tensor:
    n = _offsets(num_det)
    c = torch.pi * torch.pi * det_size * det_size
    odd = (n.abs() % 2) == 1
    taps = torch.zeros(num_det * 2 - 1, dtype=dtype)
    taps[odd] = (-1 / (c * (n[odd] ** 2))).to(taps.dtype)
    taps[num_det - 1] = 1 / (4 * det_size * det_size)
    return taps


def sheeplogan(num_det, det_size, dtype=None) -> torch.Tensor:
    n = _offsets(num_det)
    return (-2 / (torch.pi * torch.pi * det_size * det_size * (4 * n * n - 1))).to(dtype)


def filter_generate(num_det, det_size, filter_type="ramp", dtype=None) -> torch.Tensor:
    if filter_type not in FILTERS:
        raise AssertionError(f"Filter type {filter_type} not supported")
    return ramp(num_det, det_size, dtype) if filter_type == "ramp" else sheeplogan(num_det, det_size, dtype)
