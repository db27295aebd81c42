"""The discrete adjoint (hf_adjoint_rhs / hf_adjoint_accumulate / hf_solve_device behind
torch.autograd.Function) against central finite differences and against the FP64 gradient.

Workload: a 12^3 copy of the inverse problem (hidden smoothed log-kappa field, probes, 8 point
sources, Cattaneo), 60 steps with checkpoints every 25 steps (segments 25, 25, 10)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FP64 = dict(precision="fp64", criterion="recursive", tol=1e-32)


@pytest.fixture(scope="module")
def setup(cuda_lib):
    from heatflow_gb300.adjoint import AdjointModel, inverse_problem
    template, probes, sources, hidden, amps = inverse_problem(n=12, nsteps=60, nprobes=16,
                                                              nsources=8, seed=3)
    model = AdjointModel(template, probes, sources, 60, ckpt_every=25, **FP64)
    obs, _, hf = model.forward(hidden, amps)
    hf.close()
    N = template.ncells
    lk0 = hidden + 0.3 * np.sin(np.arange(N) * 0.37)      # a guess away from the hidden field
    a0 = amps * 0.7
    return model, obs, lk0, a0


def _adjoint_grad(model, obs, lk0, a0):
    from heatflow_gb300.adjoint import ProbeMisfit
    lk = torch.tensor(lk0, dtype=torch.float64, device="cuda", requires_grad=True)
    a = torch.tensor(a0, dtype=torch.float64, device="cuda", requires_grad=True)
    J = ProbeMisfit.apply(lk, a, model, obs)
    J.backward()
    return float(J), lk.grad.cpu().numpy(), a.grad.cpu().numpy()


def test_adjoint_matches_central_fd(setup):
    model, obs, lk0, a0 = setup
    J, glk, ga = _adjoint_grad(model, obs, lk0, a0)
    assert J > 0 and np.isfinite(glk).all() and np.isfinite(ga).all()
    eps = 1e-6
    cells = list(np.argsort(-np.abs(glk))[:6])
    for i in cells:
        lp, lm = lk0.copy(), lk0.copy()
        lp[i] += eps
        lm[i] -= eps
        fd = (model.loss(lp, a0, obs) - model.loss(lm, a0, obs)) / (2 * eps)
        assert abs(fd - glk[i]) <= 1e-6 * abs(glk[i]) + 1e-9 * np.abs(glk).max(), (i, fd, glk[i])
    for s in range(len(a0)):
        h = eps * a0[s]
        ap, am = a0.copy(), a0.copy()
        ap[s] += h
        am[s] -= h
        fd = (model.loss(lk0, ap, obs) - model.loss(lk0, am, obs)) / (2 * h)
        assert abs(fd - ga[s]) <= 1e-6 * abs(ga[s]) + 1e-9 * np.abs(ga).max(), (s, fd, ga[s])


def test_mixed_gradient_close_to_fp64(setup):
    from heatflow_gb300.adjoint import AdjointModel
    model, obs, lk0, a0 = setup
    _, glk, ga = _adjoint_grad(model, obs, lk0, a0)
    mixed = AdjointModel(model.template, model.probes.cpu().numpy(), model.sources_np, model.nsteps,
                         ckpt_every=25, precision="mixed", criterion="true", tol=1e-12)
    _, glk_m, ga_m = _adjoint_grad(mixed, obs, lk0, a0)
    assert np.linalg.norm(glk_m - glk) <= 1e-6 * np.linalg.norm(glk)
    assert np.linalg.norm(ga_m - ga) <= 1e-6 * np.linalg.norm(ga)


def test_persistent_solves_give_the_same_gradient(setup):
    """The forward steps and the adjoint solves through the persistent solve kernel
    (use_graph=1) give the host-polled path's gradient bit for bit."""
    from heatflow_gb300.adjoint import AdjointModel
    model, obs, lk0, a0 = setup
    kw = dict(precision="mixed", criterion="true", tol=1e-12)
    grads = []
    for g in (0, 1):
        m = AdjointModel(model.template, model.probes.cpu().numpy(), model.sources_np,
                         model.nsteps, ckpt_every=25, use_graph=g, **kw)
        grads.append(_adjoint_grad(m, obs, lk0, a0))
    (J0, l0, s0), (J1, l1, s1) = grads
    assert J0 == J1
    assert np.array_equal(l0, l1) and np.array_equal(s0, s1)


def test_config4_inverse_problem_at_size(cuda_lib):
    """The inverse problem at its stated size: 64^3, 300 Cattaneo steps, 64 probes, 8 sources,
    checkpoints every 25 steps (the forward differentiated is simulate, mod_evolve.f90:45-177).
    Gradients with respect to per-cell log-kappa and the source amplitudes are finite, the mixed
    gradient agrees with the FP64 one to 1e-6 relative, and the timings are printed."""
    import time
    from heatflow_gb300.adjoint import AdjointModel, ProbeMisfit, inverse_problem, smooth_log_kappa
    n, K = 64, 300
    template, probes, sources, hidden, amps = inverse_problem(n, K, 64, 8)
    obs_model = AdjointModel(template, probes, sources, K, 25, precision="fp64", criterion="true",
                             tol=1e-12, use_graph=1)
    obs, _, hf = obs_model.forward(hidden, amps)
    hf.close()
    lk0 = smooth_log_kappa((n, n, n), seed=1)
    out = {}
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-10)):
        model = AdjointModel(template, probes, sources, K, 25, precision=prec, criterion="true",
                             tol=tol, use_graph=1)
        lk = torch.tensor(lk0, dtype=torch.float64, device="cuda", requires_grad=True)
        a = torch.tensor(amps * 0.7, dtype=torch.float64, device="cuda", requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J = ProbeMisfit.apply(lk, a, model, obs)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        J.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        out[prec] = (float(J.detach()), lk.grad.cpu().numpy(), a.grad.cpu().numpy())
        print(f"\nconfig 4 ({n}^3, {K} steps, {prec}): loss {out[prec][0]:.6e}, forward "
              f"{t1 - t0:.3f} s, backward {t2 - t1:.3f} s")
    (J64, g64, s64), (J32, g32, s32) = out["fp64"], out["mixed"]
    assert J64 > 0 and np.isfinite(g64).all() and np.isfinite(s64).all()
    assert np.isfinite(g32).all() and np.isfinite(s32).all()
    assert np.linalg.norm(g64) > 0 and np.linalg.norm(s64) > 0
    eg = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
    es = np.linalg.norm(s32 - s64) / np.linalg.norm(s64)
    print(f"config 4: mixed vs FP64 gradient rel L2: log-kappa {eg:.3e}, sources {es:.3e}; "
          f"loss {abs(J32 - J64) / J64:.3e}")
    assert eg <= 1e-6 and es <= 1e-6
