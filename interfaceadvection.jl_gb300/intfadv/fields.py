"""Device fields in the reference's Julia memory layout.

A scalar field of ghost-inclusive shape ``Ng = (n0, n1[, n2])`` is a torch
tensor whose memory is column-major (x fastest); a vector field has shape
``Ng + (D,)`` with the component index last (SoA).  The tensors returned here
are views with Fortran strides over contiguous storage, so ``data_ptr()`` is
the address the C-ABI expects and ``.cpu().numpy()`` gives an array that
indexes like the Julia array (0-based).
"""
from __future__ import annotations

import torch


def fempty(shape, dtype=torch.float64, device="cuda"):
    t = torch.empty(tuple(reversed(tuple(shape))), dtype=dtype, device=device)
    return t.permute(*reversed(range(len(shape))))


def fzeros(shape, dtype=torch.float64, device="cuda"):
    return fempty(shape, dtype, device).zero_()


def fones(shape, dtype=torch.float64, device="cuda"):
    return fempty(shape, dtype, device).fill_(1)


def ffrom(array, device="cuda", dtype=None):
    """Copy a numpy / torch array (any order) into a Fortran-layout device tensor."""
    src = torch.as_tensor(array)
    out = fempty(tuple(src.shape), dtype or src.dtype, device)
    out.copy_(src)
    return out


def is_fortran(t: torch.Tensor) -> bool:
    """True when ``t`` is column-major and dense (the layout the C-ABI reads)."""
    exp = 1
    for size, stride in zip(t.shape, t.stride()):
        if size != 1 and stride != exp:
            return False
        exp *= size
    return True


def ptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("field must live on the CUDA device")
    if not is_fortran(t):
        raise ValueError("field must be column-major (Julia layout); build it with intfadv.fields.fzeros")
    return t.data_ptr()


def cell_coords(ng, device="cuda", dtype=torch.float64):
    """Cell-centre coordinates, WaterLily loc(0,I) = I - 1.5 (1-based I), as broadcastable tensors.

    Returns ``D`` tensors that broadcast to the reversed shape ``(n2, n1, n0)`` (C order),
    i.e. to a buffer whose memory is x-fastest.
    """
    D = len(ng)
    out = []
    for d in range(D):
        v = torch.arange(ng[d], device=device, dtype=dtype) - 0.5
        shape = [1] * D
        shape[D - 1 - d] = ng[d]
        out.append(v.view(*shape))
    return out


def face_coords(ng, i, device="cuda", dtype=torch.float64):
    """Coordinates of the lower i-faces, WaterLily loc(i,I) = I - 1.5 - 0.5 e_i."""
    x = cell_coords(ng, device, dtype)
    x[i] = x[i] - 0.5
    return x


def evaluate(fn, coords, ng, device="cuda", dtype=torch.float64):
    """Evaluate a vectorised function of coordinate tensors into a Fortran-layout field."""
    val = fn(coords)
    val = torch.as_tensor(val, device=device, dtype=dtype)
    full = val.expand(*reversed(tuple(ng))).contiguous()
    return full.permute(*reversed(range(len(ng))))
