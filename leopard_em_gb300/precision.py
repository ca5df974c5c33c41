"""Precision form of the search: the inverse DFT stages as split-precision
tensor-core contractions (tcgen05, BF16 or FP16 hi + lo operands, FP32
accumulation).

This module holds the host side: the blocked core-matrix operand layout the
tensor-core kernels read (``to_blocked``), and the driver of the precision
search.
"""

from __future__ import annotations

import ctypes

import torch

from ._native import check, lib

KCHUNK = 64


def split16(x: torch.Tensor, f16: bool = False) -> tuple[torch.Tensor, torch.Tensor]:
    """x (FP32) -> (hi, lo) 16-bit parts, x ~= hi + lo."""
    dt = torch.float16 if f16 else torch.bfloat16
    hi = x.to(dt)
    lo = (x - hi.to(torch.float32)).to(dt)
    return hi, lo


def to_blocked(x: torch.Tensor, tile_rows: int) -> torch.Tensor:
    """[R, K] matrix -> 1-D blocked core-matrix layout (rows padded to a
    multiple of tile_rows, K to a multiple of 64, with zeros): element (r, k)
    at (((r/TR)*KC + k/64)*(TR/8) + (r%TR)/8)*512 + ((k%64)/8)*64 + (r%8)*8 + k%8."""
    R, K = x.shape
    Rp = -(-R // tile_rows) * tile_rows
    Kp = -(-K // KCHUNK) * KCHUNK
    xp = torch.zeros((Rp, Kp), dtype=x.dtype, device=x.device)
    xp[:R, :K] = x
    t = xp.reshape(Rp // tile_rows, tile_rows // 8, 8, Kp // KCHUNK, KCHUNK // 8, 8)
    return t.permute(0, 3, 1, 4, 2, 5).contiguous().reshape(-1)


def blocked_split(x: torch.Tensor, tile_rows: int, f16: bool = False) -> tuple[torch.Tensor, torch.Tensor]:
    """FP32 [R, K] -> blocked (hi, lo) 16-bit operands."""
    hi, lo = split16(x.to(torch.float32), f16)
    return to_blocked(hi, tile_rows), to_blocked(lo, tile_rows)


def tc_gemm(a: torch.Tensor, b: torch.Tensor, bn: int = 256, f16: bool = False, terms: int = 3) -> torch.Tensor:
    """D = A @ B^T on the tensor cores from FP32 device matrices A [M, K],
    B [N, K] (split, blocked and multiplied by ``lgb_tc_gemm``)."""
    if a.dim() != 2 or b.dim() != 2 or a.shape[1] != b.shape[1]:
        raise ValueError("a must be [M, K] and b [N, K]")
    M, K = a.shape
    N = b.shape[0]
    dev = a.device
    a_hi, a_lo = blocked_split(a, 128, f16)
    b_hi, b_lo = blocked_split(b, bn, f16)
    d = torch.empty((M, N), dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    with torch.cuda.device(dev):
        s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        check(lib().lgb_tc_gemm(-(-M // 128), -(-N // bn), -(-K // KCHUNK), bn, int(f16), terms, a_hi.data_ptr(),
                                a_lo.data_ptr(), b_hi.data_ptr(), b_lo.data_ptr(), d.data_ptr(), N, M, N,
                                err.data_ptr(), s), "lgb_tc_gemm")
    e = int(err.item())
    if e:
        raise RuntimeError(f"lgb_tc_gemm: device status {e}")
    return d
