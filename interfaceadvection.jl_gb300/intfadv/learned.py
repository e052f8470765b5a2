"""Learned Poisson preconditioner, host side (no counterpart in the reference).

The network (csrc/nn.cuh: 3-level 3D conv encoder-decoder, 3x3x3 kernels,
channels 4-16-32-32-32-16-1) maps (r / max|r|, λρ·L_x, λρ·L_y, λρ·L_z) to a
correction proportional to A⁻¹ r and preconditions the inner flexible CG of
``poisson="learned"`` (csrc/poisson.cu), with the plain V-cycle as fallback.

This module holds
  * the parameter layout, initialisation and the weights file format,
  * ``Net``: the library's own FP32 forward / backward / Adam kernels and its
    BF16 tensor-core forward, on device tensors,
  * ``PairGenerator``: training pairs from the solver's own runs — rising-bubble
    runs with 1-8 random bubbles; after each step the pressure system (face
    coefficients μ₀ and right-hand side σ) is cut into non-overlapping patches
    and each patch system (walls on the patch boundary) is solved by the FP64
    multigrid, giving (input, correction) pairs,
  * ``train``: the training loop, and a command line
    ``python -m intfadv.learned --pairs 20000 --out weights.npz``.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import time

import numpy as np
import torch

from . import _lib
from .core import Handle, make_config
from .fields import fzeros, ptr

CIN = (4, 16, 32, 32, 32, 16)
COUT = (16, 32, 32, 32, 16, 1)
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "precond.npz")


def layer_offsets():
    """[(w_offset, b_offset)] of W_l[27][Cout][Cin] and b_l[Cout] in the parameter vector."""
    out, o = [], 0
    for ci, co in zip(CIN, COUT):
        out.append((o, o + 27 * co * ci))
        o += 27 * co * ci + co
    return out


def param_count() -> int:
    return sum(27 * co * ci + co for ci, co in zip(CIN, COUT))


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights (std sqrt(2 / (27 Cin))), zero biases; the linear output layer at half that."""
    rng = np.random.Generator(np.random.PCG64(seed))
    w = np.zeros(param_count(), dtype=np.float32)
    for l, ((wo, bo), ci, co) in enumerate(zip(layer_offsets(), CIN, COUT)):
        std = math.sqrt(2.0 / (27 * ci)) * (0.5 if l == len(CIN) - 1 else 1.0)
        w[wo:bo] = rng.normal(0.0, std, size=bo - wo).astype(np.float32)
    return w


def save_params(path: str, w: np.ndarray, **meta) -> None:
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez(path, w=np.asarray(w, dtype=np.float32), meta=json.dumps(meta))


def load_params(path: str = WEIGHTS):
    z = np.load(path, allow_pickle=False)
    return z["w"].astype(np.float32), json.loads(str(z["meta"]))


def _dev_ptr(t: torch.Tensor):
    assert t.is_cuda and t.is_contiguous()
    return C.c_void_p(t.data_ptr())


class Net:
    """The network state of one library handle (any grid; a small 3D one by default)."""

    def __init__(self, handle: Handle | None = None, device="cuda"):
        if handle is None:
            handle = Handle(make_config((8, 8, 8)))
        self.handle = handle
        self.device = device
        self.n = int(_lib.load().ia_nn_param_count())
        assert self.n == param_count()

    def set_params(self, w: np.ndarray) -> None:
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == self.n
        _lib.check(self.handle.call("ia_nn_set_params", C.c_void_p(w.ctypes.data)), "ia_nn_set_params")

    def set_loss(self, kind: str) -> None:
        """"mse" or "energy" (energy norm of the error with the input coefficient channels)."""
        _lib.check(self.handle.call("ia_nn_set_loss", {"mse": 0, "energy": 1}[kind]), "ia_nn_set_loss")

    def get_params(self) -> np.ndarray:
        w = np.zeros(self.n, dtype=np.float32)
        _lib.check(self.handle.call("ia_nn_get_params", C.c_void_p(w.ctypes.data)), "ia_nn_get_params")
        return w

    @staticmethod
    def _dims(x0: torch.Tensor):
        B, nzp, nyp, nxp, c = x0.shape
        assert c == 4 and x0.dtype == torch.float32
        return B, nxp - 2, nyp - 2, nzp - 2

    def forward(self, x0: torch.Tensor, tensor_cores: bool = False) -> torch.Tensor:
        """FP32 training kernels, or the BF16 tcgen05 inference kernels (the solver's path)."""
        B, nx, ny, nz = self._dims(x0)
        out = torch.zeros(x0.shape[:-1], dtype=torch.float32, device=x0.device)
        mode = 1 if tensor_cores else 0
        _lib.check(self.handle.call("ia_nn_forward", _dev_ptr(x0), _dev_ptr(out), B, nx, ny, nz, mode),
                   "ia_nn_forward")
        return out

    def loss_grad(self, x0: torch.Tensor, tgt: torch.Tensor):
        B, nx, ny, nz = self._dims(x0)
        g = torch.zeros(self.n, dtype=torch.float32, device=x0.device)
        loss = C.c_double()
        _lib.check(self.handle.call("ia_nn_loss_grad", _dev_ptr(x0), _dev_ptr(tgt), B, nx, ny, nz, _dev_ptr(g),
                                    C.byref(loss)), "ia_nn_loss_grad")
        return loss.value, g

    def train_step(self, x0: torch.Tensor, tgt: torch.Tensor, lr: float) -> float:
        B, nx, ny, nz = self._dims(x0)
        loss = C.c_double()
        _lib.check(self.handle.call("ia_nn_train_step", _dev_ptr(x0), _dev_ptr(tgt), B, nx, ny, nz, C.c_float(lr),
                                    C.byref(loss)), "ia_nn_train_step")
        return loss.value


# ---------------------------------------------------------------------------------- tensors
def _cl(a: torch.Tensor) -> torch.Tensor:
    """Fortran-layout grid view (x fastest) -> [z][y][x] view of the same memory."""
    return a.permute(2, 1, 0)


def net_input(r: torch.Tensor, L: torch.Tensor, lrho: float) -> torch.Tensor:
    """Training-layout input [1, nz+2, ny+2, nx+2, 4] (FP32) from a grid residual r (Ng) and
    face coefficients L (Ng + (3,)), both Fortran-layout; channels as the solver's own input."""
    nxp, nyp, nzp = r.shape
    x0 = torch.zeros((1, nzp, nyp, nxp, 4), dtype=torch.float32, device=r.device)
    ri = _cl(r)[1:-1, 1:-1, 1:-1]
    s = float(ri.abs().max())
    x0[0, 1:-1, 1:-1, 1:-1, 0] = (ri / (s if s > 0 else 1.0)).float()
    for d in range(3):
        x0[0, 1:-1, 1:-1, 1:-1, 1 + d] = (lrho * _cl(L[..., d])[1:-1, 1:-1, 1:-1]).float()
    return x0


def interior(a: torch.Tensor) -> torch.Tensor:
    return a[1:-1, 1:-1, 1:-1]


# ---------------------------------------------------------------------------------- pairs
def bubble_layout(seed: int, N: int, nmin=1, nmax=8, rmin=0.05, rmax=0.15, max_tries=10000):
    """1-8 non-overlapping bubbles in a unit box scaled to N cells (PCG64 seeded)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nb = int(rng.integers(nmin, nmax + 1))
    out = []
    for _ in range(max_tries):
        if len(out) == nb:
            break
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(r + 0.02, 1.0 - r - 0.02, size=3)
        if all(np.linalg.norm(c - c2) > r + r2 + 0.02 for c2, r2 in out):
            out.append((c, r))
    return [(tuple(float(v) * N for v in c), float(r) * N) for c, r in out]


def bubbles_sdf(bubbles):
    """Vectorised SDF, positive inside any bubble (light fluid), negative in the liquid."""
    def sdf(x):
        best = None
        for c, r in bubbles:
            v = r - torch.sqrt((x[0] - c[0]) ** 2 + (x[1] - c[1]) ** 2 + (x[2] - c[2]) ** 2)
            best = v if best is None else torch.maximum(best, v)
        return best
    return sdf


class PatchSolver:
    """FP64 multigrid-preconditioned CG on a P³ patch system with walls on the patch boundary."""

    def __init__(self, P: int, device="cuda", tol_rel=1e-6, itmx=200):
        self.P = P
        self.handle = Handle(make_config((P, P, P), poisson="fp64"))
        ng = (P + 2,) * 3
        self.x = fzeros(ng, device=device)
        self.z = fzeros(ng, device=device)
        self.r = fzeros(ng, device=device)
        self.L = fzeros(ng + (3,), device=device)
        self.tol_rel, self.itmx = tol_rel, itmx
        self.tol = 0.0

    def set_system(self, r: torch.Tensor, L: torch.Tensor) -> float:
        """r: P³ right-hand side (made mean-free); L: (P, P, P, 3) lower-face coefficients of the
        patch cells (the patch's own boundary faces become walls).  Returns max|r|."""
        self.z.zero_()
        self.L.zero_()
        rm = r - r.mean()
        self.z[1:-1, 1:-1, 1:-1] = rm
        self.L[1:-1, 1:-1, 1:-1, :] = L
        self.L[1, :, :, 0] = 0.0
        self.L[:, 1, :, 1] = 0.0
        self.L[:, :, 1, 2] = 0.0
        s = float(rm.abs().max())
        self.tol = self.tol_rel * s
        return s

    def run(self, itmx=None):
        """CG from zero for at most itmx iterations (default: to tol_rel); returns the iterations."""
        self.x.zero_()
        it, res = C.c_int32(), C.c_double()
        rc = self.handle.call("ia_poisson_solve", ptr(self.x), ptr(self.z), ptr(self.L), self.tol,
                              int(itmx or self.itmx), C.byref(it), C.byref(res))
        _lib.check(rc, "ia_poisson_solve", allow=(_lib.IA_OK, _lib.IA_WARN_NOT_CONVERGED))
        return it.value

    def residual(self) -> torch.Tensor:
        """z - A x of the current iterate (interior, P³)."""
        linf = C.c_double()
        _lib.check(self.handle.call("ia_poisson_residual", ptr(self.r), ptr(self.x), ptr(self.z), ptr(self.L),
                                    C.byref(linf)), "ia_poisson_residual")
        return self.r[1:-1, 1:-1, 1:-1].clone()


class PairGenerator:
    """(input, target) patch pairs from rising-bubble runs on an N³ box (periodic x/z, walls y).

    Run k uses ``bubble_layout(seed_base + k, N)``; after ``warm`` steps every step's pressure
    system is cut into the (N/P)³ non-overlapping P³ patches.  Each patch system is solved by
    the multigrid-preconditioned CG (correction e*), and for every k in ``ks`` the iterate x_k
    after k multigrid-preconditioned iterations gives one pair: input the residual
    t = r - A x_k (as t / max|t|, with the face coefficients), target the remaining correction
    e* - x_k (mean-free, as a fraction of its maximum) — the residuals the net meets behind the
    V-cycle in the hybrid preconditioner.  Flexible CG and the hybrid's least-squares ω are
    blind to the amplitude of each preconditioner output, so only its shape is learned."""

    def __init__(self, N=128, P=64, seed_base=1000, steps_per_run=6, warm=2, poisson="mixed", device="cuda",
                 lrho=1e-3, lmu=1e-2, ks=(1, 2)):
        assert N % P == 0 and P % 4 == 0
        self.N, self.P, self.seed_base = N, P, seed_base
        self.steps_per_run, self.warm = steps_per_run, warm
        self.poisson, self.device = poisson, device
        self.lrho, self.lmu, self.ks = lrho, lmu, tuple(ks)
        self.solver = PatchSolver(P, device=device)
        self.gains = []   # max|e| / max|t| per pair (information only)
        self.iters = []

    def _sim(self, k):
        from .simulation import TwoPhaseSimulation
        N = self.N
        G, D = 1e-3, 0.25 * N
        sigma = G * D * D / 10.0
        mu = (1e-3 * sigma ** 3 / G) ** 0.25
        return TwoPhaseSimulation((N, N, N), (0.0, 0.0, 0.0), float(N), perdir=(0, 2), λρ=self.lrho, λμ=self.lmu,
                                  ν=mu, η=sigma, g=(0.0, -G, 0.0),
                                  InterfaceSDF=bubbles_sdf(bubble_layout(self.seed_base + k, N)),
                                  poisson=self.poisson, poisson_tol=1e-8, poisson_itmx=400, device=self.device)

    def snapshots(self):
        from .simulation import sim_step
        k = 0
        while True:
            sim = self._sim(k)
            for s in range(self.warm + self.steps_per_run):
                sim_step(sim)
                if s >= self.warm:
                    yield interior(sim.flow.sigma).clone(), sim.flow.mu0[1:-1, 1:-1, 1:-1, :].clone()
            k += 1

    def _pair(self, t, e):
        P = self.P
        s, em = float(t.abs().max()), float(e.abs().max())
        if not (s > 0 and em > 0):
            return None
        self.gains.append(em / s)
        tg = torch.zeros((P + 2,) * 3, dtype=torch.float64, device=t.device)
        tg[1:-1, 1:-1, 1:-1] = t
        x0 = net_input(tg, self.solver.L, self.lrho)
        tgt = torch.zeros(x0.shape[:-1], dtype=torch.float32, device=t.device)
        tgt[0, 1:-1, 1:-1, 1:-1] = _cl(e / em).float()
        return x0, tgt

    def pairs(self):
        """Yields (x0 [1,P+2,P+2,P+2,4], target [1,P+2,P+2,P+2]) FP32 device tensors."""
        P, n, sv = self.P, self.N // self.P, self.solver
        for z, L in self.snapshots():
            for ox in range(n):
                for oy in range(n):
                    for oz in range(n):
                        sl = (slice(ox * P, ox * P + P), slice(oy * P, oy * P + P), slice(oz * P, oz * P + P))
                        if not (sv.set_system(z[sl], L[sl]) > 0):
                            continue
                        self.iters.append(sv.run())
                        e_star = interior(sv.x).clone()
                        for k in self.ks:
                            if k == 0:
                                t, e = interior(sv.z).clone(), e_star
                            else:
                                sv.run(k)
                                t = sv.residual()
                                e = e_star - interior(sv.x)
                            pr = self._pair(t, e - e.mean())
                            if pr is not None:
                                yield pr


def batches(pairs, B):
    xs, ts = [], []
    for x0, t in pairs:
        xs.append(x0)
        ts.append(t)
        if len(xs) == B:
            yield torch.cat(xs), torch.cat(ts)
            xs, ts = [], []


def augment(x0: torch.Tensor, tgt: torch.Tensor, gen: torch.Generator, amin=0.05):
    """Random sign and amplitude c ∈ [amin, 1] (log-uniform) per sample on the residual channel and the
    target: the pair relation is linear in the residual, and the solver meets residuals whose local
    amplitude is far below the normalising maximum."""
    B = x0.shape[0]
    u = torch.rand(B, generator=gen, device="cpu", dtype=torch.float64)
    sg = torch.where(torch.rand(B, generator=gen, device="cpu", dtype=torch.float64) < 0.5, -1.0, 1.0)
    c = (sg * torch.exp(u * math.log(amin))).to(x0.device, torch.float32)
    x0[..., 0] *= c.view(B, 1, 1, 1)
    tgt *= c.view(B, 1, 1, 1)
    return x0, tgt


def train(net: Net, pairs, n_pairs: int, batch=4, lr=1e-3, lr_final=1e-4, log_every=50, log=print, seed=0,
          aug=True):
    """One pass of Adam over n_pairs streamed pairs; cosine learning-rate decay; sign/amplitude
    augmentation (``augment``)."""
    steps = max(1, n_pairs // batch)
    losses = []
    t0 = time.time()
    g = torch.Generator().manual_seed(seed)
    for k, (x0, tgt) in enumerate(batches(pairs, batch)):
        if k >= steps:
            break
        if aug:
            x0, tgt = augment(x0, tgt, g)
        a = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * k / steps))
        losses.append(net.train_step(x0, tgt, a))
        if log and (k % log_every == 0 or k == steps - 1):
            log(f"step {k}/{steps} loss {losses[-1]:.4e} lr {a:.2e} {time.time() - t0:.1f}s")
    return losses


def eval_system(N=64, seed=999, steps=2, device="cuda"):
    """A held-out pressure system: μ₀ and σ after ``steps`` steps of a bubbly N³ run."""
    from .simulation import TwoPhaseSimulation, sim_step
    G, D = 1e-3, 0.25 * N
    sigma = G * D * D / 10.0
    mu = (1e-3 * sigma ** 3 / G) ** 0.25
    sim = TwoPhaseSimulation((N, N, N), (0.0, 0.0, 0.0), float(N), perdir=(0, 2), λρ=1e-3, λμ=1e-2, ν=mu, η=sigma,
                             g=(0.0, -G, 0.0), InterfaceSDF=bubbles_sdf(bubble_layout(seed, N)), poisson="mixed",
                             poisson_tol=1e-9, poisson_itmx=400, device=device)
    for _ in range(steps):
        sim_step(sim)
    return sim.flow.mu0.clone(), sim.flow.sigma.clone()


def evaluate(weights, L, z, tol=1e-8, preconds=("none", "net", "vcycle", "hybrid"), inner_max=30, reps=3):
    """FCG iterations, solve time (median of ``reps``) and FP64 residual of the learned mode per
    inner preconditioner, against the plain FP64 multigrid, on the system (L, z)."""
    from .simulation import poisson_stats, set_learned
    N = tuple(n - 2 for n in z.shape)
    out = {}

    def run(mode, precond=None):
        h = Handle(make_config(N, perdir=(0, 2), poisson=mode, lrho=1e-3))
        if mode == "learned":
            set_learned(h, precond=precond, weights=weights,
                        inner_max=(2000 if precond in ("none", "net") else inner_max))
        times, it, res = [], C.c_int32(), C.c_double()
        for _ in range(reps):
            x = fzeros(z.shape)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rc = h.call("ia_poisson_solve", ptr(x), ptr(z), ptr(L), tol, 4000, C.byref(it), C.byref(res))
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
            _lib.check(rc, "ia_poisson_solve", allow=(_lib.IA_OK, _lib.IA_WARN_NOT_CONVERGED))
        r = dict(iters=it.value, resid=res.value, ms=1e3 * float(np.median(times)))
        if mode == "learned":
            st = poisson_stats(h)
            r.update(fallbacks=st["fallbacks"] // reps, net_per_solve=st["net"] // reps,
                     vcycles_per_solve=st["vcycles"] // reps)
        return r

    out["fp64_mg"] = run("fp64")
    out["mixed_mg"] = run("mixed")
    for p in preconds:
        out[p] = run("learned", p)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description="train the learned Poisson preconditioner")
    ap.add_argument("--pairs", type=int, default=20000)
    ap.add_argument("--N", type=int, default=128)
    ap.add_argument("--P", type=int, default=64)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--steps-per-run", type=int, default=6)
    ap.add_argument("--loss", default="mse", choices=("mse", "energy"))
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--eval-N", type=int, default=64, help="held-out system size for the ablation (0 = skip)")
    a = ap.parse_args(argv)
    torch.cuda.set_device(0)
    net = Net()
    net.set_params(init_params(a.seed))
    net.set_loss(a.loss)
    gen = PairGenerator(N=a.N, P=a.P, steps_per_run=a.steps_per_run)
    t0 = time.time()
    losses = train(net, gen.pairs(), a.pairs, batch=a.batch, lr=a.lr, seed=a.seed)
    meta = dict(pairs=a.pairs, N=a.N, P=a.P, batch=a.batch, lr=a.lr, seed=a.seed, seed_base=gen.seed_base, loss=a.loss,
                steps_per_run=gen.steps_per_run, gain_median=float(np.median(gen.gains)), first_loss=losses[0],
                final_loss=float(np.mean(losses[-20:])), seconds=time.time() - t0,
                patch_mg_iters_mean=float(np.mean(gen.iters)) if gen.iters else None)
    save_params(a.out, net.get_params(), **meta)
    print(json.dumps(meta))
    if a.eval_N:
        L, z = eval_system(a.eval_N)
        print(json.dumps({"eval_N": a.eval_N, **evaluate(a.out, L, z)}))


if __name__ == "__main__":
    main()
