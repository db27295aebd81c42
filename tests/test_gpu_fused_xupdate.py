"""The x update folded into the inner CG update predicted to end the inner solve (true-residual
criterion).  The prediction (the iteration cap, or the criterion shrinking once more by the last
iteration's factor) only decides which round forms x_new = x + sigma S^-1 y; the bits must be those
of the separate x update.  Two contexts run the same step with the same CG iterates: one with a
large iteration cap, where the last iteration is often not predicted and the separate update runs,
and one whose cap equals the iteration count, which makes that iteration form x itself.  Their
states must agree bit for bit, and the round logs show which form each took."""
import numpy as np
import pytest

from heatflow_gb300.problem import Problem, layered_slab, point_source_cube
from heatflow_gb300.solver import HeatFlow

pytestmark = pytest.mark.gpu


def _mixed_materials(nx, ny, nz, seed):
    """Cells of three materials at random (kappa 149 / 0.2 / 50): irregular CG convergence, where
    the prediction misses some last iterations."""
    rng = np.random.default_rng(seed)
    N = nx * ny * nz
    ih = np.zeros(N, np.int64)
    ih[rng.integers(0, N, 3)] = 1
    return Problem(nx=nx, ny=ny, nz=nz, lx=nx * 1e-9, ly=ny * 1e-9, lz=nz * 1e-9,
                   kappa=rng.choice([149.0, 0.2, 50.0], size=N), rho=rng.uniform(1000, 3000, N),
                   heat_capacity=rng.uniform(500, 1500, N), tau=1e-12, em=0.0, iheater=ih,
                   power_in=1e-5, time_step=1e-13, icattaneo=1, kappa_bound=(149.0,) * 6,
                   t_bath_face=(300.0,) * 6, t_bath=300.0)


CASES = [("slab24", lambda: layered_slab(24, layer=4, peak=1e-5)),
         ("slab32", lambda: layered_slab(32, layer=8, peak=1e-5)),
         ("cube16", lambda: point_source_cube(16, power_in=1e-5)),
         ("cube24", lambda: point_source_cube(24, power_in=1e-6))] + \
        [(f"mixed{nx}x{ny}x{nz}s{seed}", lambda nx=nx, ny=ny, nz=nz, seed=seed:
          _mixed_materials(nx, ny, nz, seed))
         for (nx, ny, nz) in ((8, 8, 8), (12, 8, 12), (16, 16, 8), (20, 12, 16), (32, 24, 20))
         for seed in (1, 2, 3)]
OPTS = {"mixed": dict(precision="mixed", criterion="true", tol=1e-10),
        "fp64": dict(precision="fp64", criterion="true", tol=1e-12)}
# Loose inner targets give inner solves of one iteration, which the prediction never foresees
# (it has no rate yet): there the separate update runs unless the cap is 1.
VARIANTS = {"mixed": [{}, {"inner_tol": 3e-2}, {"inner_tol": 1e-1}],
            "fp64": [{}, {"tol": 1e-5}, {"tol": 1e-4}, {"tol": 1e-3}]}


def _solves(phases):
    """Per inner solve of a step, from its round log: (CG iterations, the round that formed the x
    the following residual sweep reads: 'cg_bx' or 'xupd')."""
    out, it, last = [], 0, None
    for p in phases:
        if p in ("res_init", "res_init_hx", "res"):
            if p == "res":
                out.append((it, last))
            it, last = 0, None
        elif p in ("cg_b", "cg_bx"):
            it += 1
            last = p
        elif p == "xupd":
            last = p
    return out


def _step(prob, state, itime, **kw):
    with HeatFlow(prob, use_graph=1, **kw) as hf:
        hf.set_state(*state) if state is not None else hf.initial_evolve()
        st = hf.run(itime, 1)
        rounds, total = hf.solve_profile()
        return hf.get_state(), st, [p for p, _ in rounds], total <= len(rounds)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_fused_x_update_equals_separate_update(prec):
    forms = []
    for (name, make), var in [(c, v) for v in VARIANTS[prec] for c in CASES]:
        prob = make()
        opts = {**OPTS[prec], **var}
        state = None
        for itime in (1, 2):
            (T, Tp), st, ph, whole = _step(prob, state, itime, **opts)
            assert whole, (name, itime, "round log truncated")
            assert st["unconverged"] == 0, (name, itime, st)
            solves = _solves(ph)
            state0, state = state, (T, Tp)
            if not solves:                      # accepted at its first residual
                continue
            cap_k = max(it for it, _ in solves)
            cap = {"inner_itmax": cap_k} if prec == "mixed" else {"itmax": cap_k}
            (T2, Tp2), st2, ph2, _ = _step(prob, state0, itime, **opts, **cap)
            solves2 = _solves(ph2)
            assert [it for it, _ in solves2] == [it for it, _ in solves], (name, itime)
            for it, form in solves2:            # the capped iteration forms x itself
                if it == cap_k:
                    assert form == "cg_bx", (name, itime, ph2)
            assert np.array_equal(T, T2) and np.array_equal(Tp, Tp2), (name, itime, solves, solves2)
            keys = ("iterations", "inner_iterations", "refinements", "unconverged")
            assert {k: st[k] for k in keys} == {k: st2[k] for k in keys}, (name, itime)
            forms += [(f, f2) for (_, f), (_, f2) in zip(solves, solves2)]
    print(prec, {f: forms.count(f) for f in set(forms)})
    # the comparison met the separate update against the fused one at least once
    assert ("xupd", "cg_bx") in forms, forms


def test_fused_x_update_on_every_step_path():
    """The captured loop, the per-step conditional graph and the host-polled kernels honour the
    same prediction (the finalize kernels run the same epilogues): equal bits over 6 steps."""
    prob = layered_slab(32, layer=8, peak=1e-5)
    out = {}
    for g in (0, 1, 2):
        with HeatFlow(prob, use_graph=g, **OPTS["mixed"]) as hf:
            hf.initial_evolve()
            st = hf.run(1, 6)
            out[g] = (hf.get_state(), st)
    for g in (1, 2):
        assert out[g][1]["inner_iterations"] == out[0][1]["inner_iterations"]
        for a, b in zip(out[g][0], out[0][0]):
            assert np.array_equal(a, b), g


def test_padded_rows_keep_separate_update():
    """FP32 vectors on rows that are not 4k cells wide use their own layout: the CG update cannot
    form x there, so the separate update runs (and the prediction never asks otherwise)."""
    prob = layered_slab(22, layer=4, peak=1e-5)
    _, _, phases, _ = _step(prob, None, 1, **OPTS["mixed"])
    assert "cg_bx" not in phases and "xupd" in phases, phases
