"""Gradients of a probe-misfit loss by the discrete adjoint of the time stepping.

No counterpart in the reference (HeatFlow computes no gradients).  The forward model is exactly
the library's step (``simulate``); the loss is

    J = sum_k sum_p (T_k[probe_p] - observed[k, p])^2 ,   k = 1..K,

and its gradient with respect to per-cell log-conductivity and per-cell heater power comes from
the adjoint recurrence (H symmetric, so the same CG solver serves H^T):

    H lambda_k = dJ/dT_k + a * lambda_(k+1) + c * lambda_(k+2),   k = K..1,
    dJ/dtheta  = sum_k lambda_k^T (dS_k/dtheta - dH/dtheta T_k),

with a = -rho c/dt - 2 tau' rho c and c = tau' rho c per cell (c = 0 in Fourier mode).  Forward
states are checkpointed every `ckpt_every` steps and recomputed segment by segment during the
backward sweep.  The device kernels are ``hf_adjoint_rhs`` and ``hf_adjoint_accumulate``; the
solves are ``hf_solve_device``.

`ProbeMisfit` wraps this as a ``torch.autograd.Function`` of (log_kappa, source amplitudes).
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np
import torch

from . import abi
from .problem import Problem
from .solver import HeatFlow


def _ptr(t: torch.Tensor):
    assert t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()
    return C.c_void_p(t.data_ptr())


class AdjointModel:
    """Forward/backward driver for one grid.

    template:  the Problem (kappa and per-cell power are replaced on every evaluation)
    probes:    cell indices whose temperature is observed after every step
    sources:   cell indices of the heaters whose power amplitudes are parameters
    nsteps:    K
    opts:      solver options of HeatFlow (FP64 with a tight true-residual tolerance for
               finite-difference checks; mixed precision for speed)
    """

    def __init__(self, template: Problem, probes, sources, nsteps: int, ckpt_every: int = 25,
                 **opts):
        if any(template.cg_face) or (template.em is not None and np.any(template.em != 0)):
            raise ValueError("the adjoint covers Dirichlet/periodic boundaries without emissivity")
        self.template = template
        self.probes = torch.as_tensor(np.asarray(probes, np.int64), device="cuda")
        self.sources = torch.as_tensor(np.asarray(sources, np.int64), device="cuda")
        self.sources_np = np.asarray(sources, np.int64)
        self.nsteps = int(nsteps)
        self.ckpt_every = int(ckpt_every)
        self.opts = opts or dict(precision="fp64", criterion="true", tol=1e-14)
        self.lib = abi.load_library()
        self.n = template.ncells

    def _context(self, log_kappa: np.ndarray, amps: np.ndarray) -> HeatFlow:
        power = np.zeros(self.n) if self.template.power is None else self.template.power.copy()
        power[self.sources_np] = amps
        iheater = np.zeros(self.n, np.int64) if self.template.iheater is None else self.template.iheater.copy()
        iheater[self.sources_np] = np.where(iheater[self.sources_np] > 0, iheater[self.sources_np], 1)
        prob = dataclasses.replace(self.template, kappa=np.exp(log_kappa), power=power,
                                   iheater=iheater, _keep=[])
        hf = HeatFlow(prob, **self.opts)
        hf.set_stream(torch.cuda.current_stream().cuda_stream)
        return hf

    def _initial(self):
        t = torch.full((self.n,), float(self.template.t_system), dtype=torch.float64, device="cuda")
        return t, t.clone()

    def _set(self, hf, tp, tpp):
        abi.check(self.lib.hf_set_state_device(hf.h, _ptr(tp), _ptr(tpp)), "hf_set_state_device")

    def _get(self, hf, tp, tpp):
        abi.check(self.lib.hf_get_state_device(hf.h, _ptr(tp), _ptr(tpp)), "hf_get_state_device")

    def forward(self, log_kappa: np.ndarray, amps: np.ndarray):
        """Run K steps; returns (probe series [K, P], checkpoints, context)."""
        hf = self._context(log_kappa, amps)
        tp, tpp = self._initial()
        self._set(hf, tp, tpp)
        ckpts = {0: (tp.clone(), tpp.clone())}
        series = torch.empty(self.nsteps, self.probes.numel(), dtype=torch.float64, device="cuda")
        self.forward_stats = {"iterations": 0, "inner_iterations": 0, "refinements": 0,
                              "unconverged": 0}
        for k in range(1, self.nsteps + 1):
            st = hf.simulate(k)
            for key in self.forward_stats:
                self.forward_stats[key] += st[key]
            self._get(hf, tp, tpp)
            series[k - 1] = tp[self.probes]
            if k % self.ckpt_every == 0 and k < self.nsteps:
                ckpts[k] = (tp.clone(), tpp.clone())
        return series, ckpts, hf

    def backward(self, hf: HeatFlow, ckpts: dict, dJ: torch.Tensor):
        """dJ: [K, P] derivative of the loss w.r.t. the probe series.  Returns
        (dJ/dlog_kappa [N], dJ/dpower [N]) as device tensors."""
        n = self.n
        z = lambda: torch.zeros(n, dtype=torch.float64, device="cuda")
        lam1, lam2, g, rhs = z(), z(), z(), z()
        grad_lk, grad_src = z(), z()
        tp, tpp = z(), z()
        starts = sorted(ckpts)
        for si in range(len(starts) - 1, -1, -1):
            s0 = starts[si]
            s1 = starts[si + 1] if si + 1 < len(starts) else self.nsteps
            self._set(hf, *ckpts[s0])                       # recompute the segment
            xs = {}
            for k in range(s0 + 1, s1 + 1):
                hf.simulate(k)
                self._get(hf, tp, tpp)
                xs[k] = tp.clone()
            for k in range(s1, s0, -1):                     # adjoint steps of the segment
                g.zero_()
                g.index_put_((self.probes,), dJ[k - 1], accumulate=True)
                abi.check(self.lib.hf_adjoint_rhs(hf.h, _ptr(g), _ptr(lam1), _ptr(lam2), _ptr(rhs)),
                          "hf_adjoint_rhs")
                lam = lam1.clone()
                st = abi.HfStats()
                abi.check(self.lib.hf_solve_device(hf.h, _ptr(rhs), _ptr(lam), C.byref(st)),
                          "hf_solve_device")
                abi.check(self.lib.hf_adjoint_accumulate(hf.h, _ptr(lam), _ptr(xs[k]), int(k),
                                                         _ptr(grad_lk), _ptr(grad_src)),
                          "hf_adjoint_accumulate")
                lam2, lam1 = lam1, lam
        return grad_lk, grad_src

    def loss(self, log_kappa: np.ndarray, amps: np.ndarray, observed: torch.Tensor) -> float:
        series, _, hf = self.forward(log_kappa, amps)
        hf.close()
        return float(((series - observed) ** 2).sum())


class ProbeMisfit(torch.autograd.Function):
    """J(log_kappa, amplitudes) = sum (T_k[probes] - observed)^2 with the adjoint gradient."""

    @staticmethod
    def forward(ctx, log_kappa: torch.Tensor, amps: torch.Tensor, model: AdjointModel,
                observed: torch.Tensor):
        series, ckpts, hf = model.forward(log_kappa.detach().double().cpu().numpy(),
                                          amps.detach().double().cpu().numpy())
        ctx.model, ctx.hf, ctx.ckpts = model, hf, ckpts
        ctx.save_for_backward(series, observed)
        return ((series - observed) ** 2).sum()

    @staticmethod
    def backward(ctx, gout):
        series, observed = ctx.saved_tensors
        dJ = 2.0 * (series - observed) * gout
        glk, gsrc = ctx.model.backward(ctx.hf, ctx.ckpts, dJ.contiguous())
        ctx.hf.close()
        return glk, gsrc[ctx.model.sources], None, None


def smooth_log_kappa(shape, length: float = 8.0, std: float = 0.5, mean: float = float(np.log(50.0)),
                     seed: int = 0) -> np.ndarray:
    """Gaussian-smoothed N(0,1) noise (length scale in cells) renormalised to `std` about `mean`,
    flattened in cell order (x fastest)."""
    nz, ny, nx = shape[2], shape[1], shape[0]
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((nz, ny, nx))
    f = np.fft.rfftn(w)
    kz = np.fft.fftfreq(nz)[:, None, None]
    ky = np.fft.fftfreq(ny)[None, :, None]
    kx = np.fft.rfftfreq(nx)[None, None, :]
    f *= np.exp(-2.0 * (np.pi * length) ** 2 * (kx ** 2 + ky ** 2 + kz ** 2))
    s = np.fft.irfftn(f, s=(nz, ny, nx), axes=(0, 1, 2))
    s = (s - s.mean()) / (s.std() + 1e-300) * std + mean
    return s.reshape(-1)


def inverse_problem(n: int = 64, nsteps: int = 300, nprobes: int = 64, nsources: int = 8,
                    seed: int = 0, dx: float = 1e-9, dt: float = 1e-13):
    """The adjoint workload: hidden smoothed log-kappa field, random probes and point sources on
    an n^3 Cattaneo grid (rho c = 2e6, tau 1e-12, Dirichlet 300 K).  Returns
    (template Problem, probes, sources, hidden log-kappa, true amplitudes)."""
    rng = np.random.default_rng(seed)
    N = n ** 3
    hidden = smooth_log_kappa((n, n, n), length=8.0 * n / 64.0 if n < 64 else 8.0, seed=seed)
    cells = rng.choice(N, size=nprobes + nsources, replace=False)
    probes, sources = cells[:nprobes], cells[nprobes:]
    amps = rng.uniform(1e-7, 1e-5, size=nsources)
    ih = np.zeros(N, np.int64)
    ih[sources] = 1
    power = np.zeros(N)
    power[sources] = amps
    template = Problem(nx=n, ny=n, nz=n, lx=n * dx, ly=n * dx, lz=n * dx, kappa=np.exp(hidden),
                       rho=2000.0, heat_capacity=1000.0, tau=1e-12, em=0.0, iheater=ih, power=power,
                       time_step=dt, icattaneo=1, qdens_mode=abi.HF_QDENS_CELL_VOLUME,
                       kappa_bound=(50.0,) * 6, t_bath_face=(300.0,) * 6, t_bath=300.0)
    return template, probes, sources, hidden, amps


def _main(argv=None):
    """Time one loss + gradient evaluation of the inverse problem (forward steps with
    checkpoints, backward adjoint solves), FP64 and mixed, and print one JSON line per path."""
    import argparse
    import json
    import time
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--probes", type=int, default=64)
    ap.add_argument("--sources", type=int, default=8)
    ap.add_argument("--ckpt", type=int, default=25)
    # per-step conditional graphs: at 64^3 (256 tasks) faster than the persistent solve, whose
    # grid-wide rounds then wait on a few busy SMs
    ap.add_argument("--use-graph", type=int, default=2)
    a = ap.parse_args(argv)
    # untimed warm-up on a small copy: the first use of each torch operation on the device may
    # compile its kernel (PTX JIT), which is not part of the workload
    wt, wp, ws, wh, wa = inverse_problem(8, 4, 4, 2)
    for prec in ("fp64", "mixed"):
        wm = AdjointModel(wt, wp, ws, 4, 2, precision=prec, criterion="true", tol=1e-10,
                          use_graph=a.use_graph)
        wobs, _, whf = wm.forward(wh, wa)
        whf.close()
        lw = torch.tensor(wh, dtype=torch.float64, device="cuda", requires_grad=True)
        aw = torch.tensor(wa, dtype=torch.float64, device="cuda", requires_grad=True)
        ProbeMisfit.apply(lw, aw, wm, wobs).backward()
        float(lw.grad.norm())
    template, probes, sources, hidden, amps = inverse_problem(a.n, a.steps, a.probes, a.sources)
    obs_model = AdjointModel(template, probes, sources, a.steps, a.ckpt, precision="fp64",
                             criterion="true", tol=1e-12, use_graph=a.use_graph)
    obs, _, hf = obs_model.forward(hidden, amps)
    hf.close()
    lk0 = smooth_log_kappa((a.n, a.n, a.n), seed=1)
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-10)):
        model = AdjointModel(template, probes, sources, a.steps, a.ckpt, precision=prec,
                             criterion="true", tol=tol, use_graph=a.use_graph)
        lk = torch.tensor(lk0, dtype=torch.float64, device="cuda", requires_grad=True)
        am = torch.tensor(amps * 0.7, dtype=torch.float64, device="cuda", requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J = ProbeMisfit.apply(lk, am, model, obs)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        J.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        print(json.dumps({"workload": f"adjoint inverse problem {a.n}^3, {a.steps} Cattaneo steps, "
                                      f"{a.probes} probes, {a.sources} sources, checkpoints every {a.ckpt}",
                          "precision": prec, "loss": float(J.detach()),
                          "forward_s": t1 - t0, "backward_s": t2 - t1,
                          "forward_solver": model.forward_stats,
                          "gradient_norm": float(lk.grad.norm())}), flush=True)


if __name__ == "__main__":
    _main()
