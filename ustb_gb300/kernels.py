"""Functional wrappers of the C-ABI on PyTorch CUDA tensors.

Tensors are passed in the ABI memory layout, i.e. MATLAB's column-major arrays
viewed as C-contiguous tensors with the dimensions reversed:

    channel data  [L, N, W, F]   ->  tensor (F, W, N, L)
    tx tables     [P, W]         ->  tensor (W, P)
    rx tables     [P, N]         ->  tensor (N, P)
    output        [P, Nk, Wk, F] ->  tensor (F, Wk, Nk, P)

``to_matlab_order`` / ``from_matlab_order`` convert between this layout and a
tensor with the MATLAB shape (a permuted view, no copy).
Every call runs on the current torch stream of the tensors' device.
"""
from __future__ import annotations

import torch

from . import _lib
from .enums import Dimension


def _stream_ptr(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _ptr(t) -> int:
    return t.data_ptr() if t is not None else 0


def _need(t: torch.Tensor, name: str, dtype, device=None):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch tensor")
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous in the ABI layout")
    if device is not None and t.device != device:
        raise ValueError(f"{name} is on {t.device}, expected {device}")


def to_matlab_order(t: torch.Tensor) -> torch.Tensor:
    """(F, W, N, L)-style ABI tensor -> view with the MATLAB shape [L, N, W, F]."""
    return t.permute(*reversed(range(t.dim())))


def from_matlab_order(t: torch.Tensor) -> torch.Tensor:
    """MATLAB-shaped tensor -> contiguous ABI-layout tensor (reversed dims)."""
    return t.permute(*reversed(range(t.dim()))).contiguous()


def out_shape_abi(P, N, W, F, dimension):
    d = int(dimension)
    nk = N if d in (0, 2) else 1
    wk = W if d in (0, 1) else 1
    return (F, wk, nk, P)


def das_table_f32(ch: torch.Tensor, fs: float, t0: float, apo_tx: torch.Tensor,
                  apo_rx: torch.Tensor, delay_tx: torch.Tensor, delay_rx: torch.Tensor,
                  fd: float, dimension=Dimension.both, out: torch.Tensor = None) -> torch.Tensor:
    """das_c drop-in on device tensors (``ustb_das_table_f32``).

    ``ch``: complex64 (F, W, N, L), or float32 (F, W, N, L) RF with fd = 0.
    Tables: float32 (W, P) for tx, (N, P) for rx.  Returns (F, Wk, Nk, P).
    """
    cplx = ch.is_complex()
    _need(ch, "ch", torch.complex64 if cplx else torch.float32)
    dev = ch.device
    F, W, N, L = ch.shape
    for name, t, rows in (("apo_tx", apo_tx, W), ("delay_tx", delay_tx, W),
                          ("apo_rx", apo_rx, N), ("delay_rx", delay_rx, N)):
        _need(t, name, torch.float32, dev)
        if t.dim() != 2 or t.shape[0] != rows:
            raise ValueError(f"{name} must be ({rows}, P), got {tuple(t.shape)}")
    P = apo_tx.shape[1]
    if not (apo_rx.shape[1] == delay_tx.shape[1] == delay_rx.shape[1] == P):
        raise ValueError("tables disagree on the number of pixels")
    shp = out_shape_abi(P, N, W, F, dimension)
    if out is None:
        out = torch.empty(shp, dtype=ch.dtype, device=dev)
    else:
        _need(out, "out", ch.dtype, dev)
        if tuple(out.shape) != shp:
            raise ValueError(f"out must be {shp}")
    with torch.cuda.device(dev):
        _lib.call("ustb_das_table_f32", _ptr(ch), int(cplx), L, N, W, F, float(fs), float(t0),
                  _ptr(apo_tx), _ptr(apo_rx), _ptr(delay_tx), _ptr(delay_rx), P, float(fd),
                  int(dimension), _ptr(out), _stream_ptr(dev))
    return out


def apply_pixel_phase(data: torch.Tensor, phase: torch.Tensor) -> torch.Tensor:
    """In place: data(..., p) *= phase(p) for an ABI-layout complex64 tensor."""
    _need(data, "data", torch.complex64)
    _need(phase, "phase", torch.complex64, data.device)
    P = phase.numel()
    if data.shape[-1] != P:
        raise ValueError("phase length must match the pixel dimension")
    with torch.cuda.device(data.device):
        _lib.call("ustb_apply_pixel_phase", _ptr(data), P, data.numel() // max(P, 1), _ptr(phase),
                  _stream_ptr(data.device))
    return data
