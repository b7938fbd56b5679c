"""Surrogate-assisted powder FID: exact FIDs on a coarse grid train a small
network that predicts FIDs at the orientations of a dense grid.

Steps (all on one GPU; torch holds device buffers and runs the SVD):
  1. exact FP32 FIDs at the coarse grid (the engine's propagation kernel,
     per-orientation output as in kernel/contexts/powder.m:291-297),
  2. time basis: the ``rank`` leading right singular vectors of those FIDs
     (randomised range finder on the device),
  3. the MLP of spx_surrogate_* (spherical-harmonic features of (beta, gamma),
     BF16 weights, FP32 accumulation) is trained on the GPU to map an
     orientation to the 2*rank real coefficients (centred, one global scale),
  4. prediction at every dense orientation; only the weighted sum of the
     coefficients is needed for the powder FID,
  5. control variate: P = sum_dense w s + sum_coarse w (f - s), so the coarse
     exact FIDs correct the network's bias and the truncation of the basis,
  6. judge: exact FIDs at held-out dense orientations.  The powder error is
     estimated as |sum_held w (s - f) - sum_coarse w (s - f)| / |P|; above the
     tolerance the exact path runs on the dense grid (fallback).
Before any training a cheaper test can reject the network outright: the
powders of the coarse grid's two interleaved halves (even and odd points)
differ by the angular structure the coarse grid does not resolve.  When they
differ by more than ``prejudge_factor`` times the tolerance, the FIDs vary on
angular scales finer than the coarse grid, which a network over a few
spherical-harmonic degrees fitted to it cannot recover, so training is
skipped and the exact dense run follows at once.
Weights of each grid are normalised to sum 1 before mixing grids (the
powder weights of kernel/contexts/powder.m:280-287 sum to 1 already).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import engine as E


@dataclass
class SurrogateResult:
    fid: np.ndarray                 # powder FID returned (surrogate-assisted, or exact after fallback)
    surrogate_fid: np.ndarray       # control-variate estimate, whatever the judge decided
    coarse_fid: np.ndarray          # exact coarse-grid powder (the method without the network)
    accepted: bool
    judge_estimate: float           # estimated relative powder error of surrogate_fid
    holdout_rel_err: float          # median per-orientation relative error at held-out orientations
    nearest_rel_err: float          # same for the nearest coarse orientation's exact FID
    loss: np.ndarray
    seconds: dict = field(default_factory=dict)
    half_grid_rel_diff: float = 0.0     # |P_even - P_odd| / |P| of the coarse grid's halves
    trained: bool = True                # False when the half-grid test rejected the network


def _xyz(beta, gamma):
    b = np.asarray(beta, float)
    g = np.asarray(gamma, float)
    return np.stack([np.sin(b) * np.cos(g), np.sin(b) * np.sin(g), np.cos(b)], 1)


def _time_basis(F, rank: int, seed: int, oversample: int = 16, power: int = 3):
    """Leading right singular vectors of F (n x T) by a randomised range finder
    with power iterations (Halko, Martinsson and Tropp, SIAM Rev. 53 (2011) 217,
    algorithms 4.4 and 5.1), on the device: a few products with F instead of a full SVD."""
    import torch
    n, T = F.shape
    k = min(rank + oversample, n, T)
    g = torch.Generator(device=F.device).manual_seed(seed)
    Om = torch.randn(n, k, generator=g, device=F.device, dtype=torch.float32).to(F.dtype)
    Y = F.conj().T @ Om                                  # (T, k): range of F^H
    Q, _ = torch.linalg.qr(Y)
    for _ in range(power):
        Q, _ = torch.linalg.qr(F @ Q)
        Q, _ = torch.linalg.qr(F.conj().T @ Q)
    Bs = F @ Q                                           # (n, k) = F restricted to span(Q)
    _, _, Wh = torch.linalg.svd(Bs, full_matrices=False)
    V = Q @ Wh.conj().T                                  # (T, k) right singular vectors
    r = min(rank, k)
    return V[:, :r].conj().T.contiguous()


class SurrogatePowder:
    """Surrogate-assisted powder FID on an uploaded engine."""

    def __init__(self, engine: E.Engine, device: int = 0, lmax: int = 12, hidden: int = 256,
                 layers: int = 4, rank: int = 64, seed: int = 0):
        import torch
        self.torch = torch
        self.engine = engine
        self.dev = torch.device('cuda', device)
        self.rank = rank
        self.net = E.Surrogate(device, lmax, hidden, layers, 2 * rank, seed)
        self.seed = seed

    def run(self, coarse_grid, dense_grid, holdout_idx, dt: float, nsteps: int, epochs: int = 1500,
            lr: float = 1e-3, tol: float = 1e-5, precision: int = E.FP32,
            prejudge_factor: float = 100.0) -> SurrogateResult:
        torch = self.torch
        sec = {}
        ca, cb, cg, cw = (np.asarray(a, float) for a in coarse_grid)
        da, db, dg, dw = (np.asarray(a, float) for a in dense_grid)
        cw = cw / cw.sum()
        dw = dw / dw.sum()
        ho = np.asarray(holdout_idx, np.int64)

        t0 = time.perf_counter()
        coarse = self.engine.run(ca, cb, cg, cw, dt, nsteps, precision=precision, per_orientation=True)
        sec['coarse_exact'] = time.perf_counter() - t0

        # half-grid test: the powders of the even and odd coarse points
        even, odd = coarse.fids[0::2], coarse.fids[1::2]
        pe = (cw[0::2] / cw[0::2].sum()) @ even
        po = (cw[1::2] / cw[1::2].sum()) @ odd
        half = float(np.linalg.norm(pe - po) / max(np.linalg.norm(coarse.fid), 1e-300))
        if prejudge_factor > 0 and half > prejudge_factor * tol:
            t0 = time.perf_counter()
            fid = self.engine.run(da, db, dg, dw, dt, nsteps, precision=precision).fid
            sec['fallback'] = time.perf_counter() - t0
            return SurrogateResult(fid=fid, surrogate_fid=coarse.fid, coarse_fid=coarse.fid, accepted=False,
                                   judge_estimate=float('nan'), holdout_rel_err=float('nan'),
                                   nearest_rel_err=float('nan'), loss=np.zeros(0), seconds=sec,
                                   half_grid_rel_diff=half, trained=False)

        t0 = time.perf_counter()
        F = torch.from_numpy(coarse.fids).to(self.dev, torch.complex64)
        B = _time_basis(F, self.rank, self.seed)                    # (r, nsteps+1)
        r = B.shape[0]
        coef = F @ B.conj().T                                       # (n_coarse, r)
        T = torch.cat([coef.real, coef.imag], 1)
        if r < self.rank:
            T = torch.cat([T, torch.zeros(T.shape[0], 2 * (self.rank - r), device=self.dev)], 1)
        mu = T.mean(0)
        sig = float(torch.sqrt(((T - mu) ** 2).mean()).clamp_min(1e-30))
        Tn = ((T - mu) / sig).float().contiguous()
        d_cb = torch.from_numpy(cb).to(self.dev)
        d_cg = torch.from_numpy(cg).to(self.dev)
        torch.cuda.synchronize(self.dev)
        sec['basis'] = time.perf_counter() - t0

        t0 = time.perf_counter()
        loss = self.net.train(cb.size, d_cb.data_ptr(), d_cg.data_ptr(), Tn.data_ptr(), epochs, lr)
        sec['train'] = time.perf_counter() - t0

        def predict(beta, gamma):
            n = beta.size
            out = torch.empty(n, 2 * self.rank, device=self.dev, dtype=torch.float32)
            d_b = torch.from_numpy(np.ascontiguousarray(beta)).to(self.dev)
            d_g = torch.from_numpy(np.ascontiguousarray(gamma)).to(self.dev)
            self.net.predict(n, d_b.data_ptr(), d_g.data_ptr(), out.data_ptr())
            c = out.double() * sig + mu.double()
            return torch.complex(c[:, :r], c[:, self.rank:self.rank + r])   # (n, r) complex128

        t0 = time.perf_counter()
        Bd = B.to(torch.complex128)
        cd = predict(db, dg)
        wd = torch.from_numpy(dw).to(self.dev, torch.complex128)
        s_dense = (wd @ cd) @ Bd
        cc = predict(cb, cg)
        wc = torch.from_numpy(cw).to(self.dev, torch.complex128)
        Fc = F.to(torch.complex128)
        sc = cc @ Bd
        est = s_dense + wc @ (Fc - sc)
        P = est.cpu().numpy()
        sec['predict'] = time.perf_counter() - t0

        t0 = time.perf_counter()
        hold = self.engine.run(da[ho], db[ho], dg[ho], np.full(ho.size, 1.0 / ho.size), dt, nsteps,
                               precision=precision, per_orientation=True)
        Hf = torch.from_numpy(hold.fids).to(self.dev)
        sh = predict(db[ho], dg[ho]) @ Bd
        rh = sh - Hf
        wh = torch.full((ho.size,), 1.0 / ho.size, device=self.dev, dtype=torch.complex128)
        err = wh @ rh - wc @ (sc - Fc)
        judge = float(torch.linalg.norm(err) / torch.linalg.norm(est).clamp_min(1e-300))
        per = torch.linalg.norm(rh, dim=1) / torch.linalg.norm(Hf, dim=1).clamp_min(1e-300)
        holdout_rel = float(per.median())
        nn = np.argmax(_xyz(db[ho], dg[ho]) @ _xyz(cb, cg).T, axis=1)
        rn = Fc[torch.from_numpy(nn).to(self.dev)] - Hf
        nearest_rel = float((torch.linalg.norm(rn, dim=1) / torch.linalg.norm(Hf, dim=1).clamp_min(1e-300)).median())
        sec['judge'] = time.perf_counter() - t0

        accepted = judge <= tol
        fid = P
        if not accepted:
            t0 = time.perf_counter()
            fid = self.engine.run(da, db, dg, dw, dt, nsteps, precision=precision).fid
            sec['fallback'] = time.perf_counter() - t0
        return SurrogateResult(fid=fid, surrogate_fid=P, coarse_fid=coarse.fid, accepted=accepted,
                               judge_estimate=judge, holdout_rel_err=holdout_rel,
                               nearest_rel_err=nearest_rel, loss=loss, seconds=sec, half_grid_rel_diff=half)
