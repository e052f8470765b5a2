"""Synthetic workloads with the shapes and value distributions of the benchmark configs.

All quantities are in WaterLily grid units (Δx = 1): a domain of physical
length 1 resolved by N cells has h = 1/N, cell centres at loc(0,I) = I - 1.5
(1-based I) and velocities in cells per unit time.

* deformation_field — the 3D LeVeque deformation u = 2sin²(πx)sin(2πy)sin(2πz),
  v = -sin(2πx)sin²(πy)sin(2πz), w = -sin(2πx)sin(2πy)sin²(πz) (times
  cos(πt/3)), built as the discrete curl of an edge-sampled vector potential
  A = (0, -sin²(πx)sin(2πy)sin²(πz)/π, sin²(πx)sin²(πy)sin(2πz)/π) so the
  face velocities are discretely divergence-free to round-off.
* sphere_sdf — signed distance (grid units) to a sphere, negative inside.
* bubble_params / swarm_layout — the rising-bubble and bubble-swarm configurations in grid units.
"""
from __future__ import annotations

import math

import torch

from .fields import fzeros


def _sin2pi_half(x):
    # sin²(πx) with exact zeros on the walls x = 0 and x = 1
    s = torch.sin(math.pi * x) ** 2
    return torch.where((x == 0) | (x == 1), torch.zeros_like(s), s)


def deformation_field(N: int, device="cuda", dtype=torch.float64):
    """Spatial part U of the LeVeque field on the faces of an N³ grid (grid units, Ng+(3,))."""
    h = 1.0 / N
    ng = N + 2
    # edge/node coordinates along one axis: index c -> face position (c-1) h, centre (c-0.5) h
    c = torch.arange(ng + 1, device=device, dtype=dtype)
    xf = (c - 1) * h          # face-aligned coordinate
    xc = (c - 0.5) * h        # centre-aligned coordinate
    S_f = _sin2pi_half(xf)
    T_c = torch.sin(2 * math.pi * xc)
    # A2 on y-edges: (x face, y centre, z face);  A3 on z-edges: (x face, y face, z centre)
    # arrays indexed [cz, cy, cx] (C order, so memory is x fastest)
    A2 = -(S_f[None, None, :] * T_c[None, :, None] * S_f[:, None, None]) / math.pi
    A3 = (S_f[None, None, :] * S_f[None, :, None] * T_c[:, None, None]) / math.pi
    sl = slice(0, ng)
    sp = slice(1, ng + 1)
    ux = (A3[sl, sp, sl] - A3[sl, sl, sl]) - (A2[sp, sl, sl] - A2[sl, sl, sl])
    uy = -(A3[sl, sl, sp] - A3[sl, sl, sl])            # ∂z A1 = 0
    uz = (A2[sl, sl, sp] - A2[sl, sl, sl])             # ∂y A1 = 0
    U = fzeros((ng, ng, ng, 3), dtype, device)
    inv = 1.0 / (h * h)                                # curl_h A / h: cells per unit time
    for d, comp in enumerate((ux, uy, uz)):
        U[..., d].copy_((comp * inv).permute(2, 1, 0))
    return U


def deformation_time_factor(t: float, period: float = 3.0) -> float:
    return math.cos(math.pi * t / period)


def sphere_sdf(center, radius, N):
    """Vectorised SDF (grid units) of a sphere given in unit-domain coordinates; dark inside."""
    cN = [c * N for c in center]
    rN = radius * N

    def sdf(x):
        r2 = 0
        for xi, ci in zip(x, cN):
            r2 = r2 + (xi - ci) ** 2
        return torch.sqrt(r2) - rN

    return sdf


def discrete_divergence(u: torch.Tensor) -> torch.Tensor:
    """Σ_d u[I+δd,d] - u[I,d] over interior cells (WaterLily div)."""
    D = u.shape[-1]
    inner = tuple(slice(1, n - 1) for n in u.shape[:-1])
    out = 0
    for d in range(D):
        hi = tuple(slice(2, n) if e == d else slice(1, n - 1) for e, n in enumerate(u.shape[:-1]))
        out = out + (u[hi + (d,)] - u[inner + (d,)])
    return out


def bubble_params(N: int, Eo: float = 10.0, Mo: float = 1e-3, G: float = 1e-3, D=None):
    """Rising bubble in grid units at N cells per unit length: Eo = ρ g D²/σ, Mo = g μ⁴/(ρ σ³) with
    ρ_liquid = 1, gravity G (which sets the time scale), bubble diameter D (default 0.25 N)."""
    D = 0.25 * N if D is None else D
    sigma = G * D * D / Eo
    mu = (Mo * sigma ** 3 / G) ** 0.25
    return dict(dims=(N, 2 * N, N), centre=(N / 2, N / 2, N / 2), radius=0.125 * N, G=G, sigma=sigma, mu=mu,
                lrho=1e-3, lmu=1e-2, perdir=(0, 2))


def swarm_layout(seed=5, n=64, rmin=0.02, rmax=0.05, N=512, max_tries=200000):
    """n non-overlapping bubbles with radii uniform in [rmin, rmax] in the unit cube (PCG64 seed), as
    (centre, radius) in grid units of an N³ grid; rejection-sampled with a 0.01 gap."""
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(max_tries):
        if len(out) == n:
            break
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(r + 0.01, 1 - r - 0.01, size=3)
        if all(np.linalg.norm(c - c2) > r + r2 + 0.01 for c2, r2 in out):
            out.append((c, r))
    if len(out) != n:
        raise RuntimeError("could not place the bubbles")
    return [(tuple(float(v) * N for v in c), float(r) * N) for c, r in out]
