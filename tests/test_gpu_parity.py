"""Parity of the CUDA path (through the C ABI) with the oracle, on the GPU.

Bit-exact: the assembled operator and COO (sparse_Hmatrix), the SpMV in SRSax order, the
boundary vector, S_cat, S and x0 (no transcendental functions involved).  Within tolerance:
heater terms that call sin/cos/pow (rtol 1e-14), and temperature fields after the solve
(FP64 path: 1e-10 relative L2, the bar the reference's own output is held to; mixed path:
1e-9 relative L2 at a true relative residual of 1e-10 per step).
"""
import numpy as np
import pytest

from heatflow_gb300 import abi, inputs
from heatflow_gb300.problem import Problem, layered_slab, point_source_cube, random_instance
from heatflow_gb300.solver import HeatFlow, geometric_to_dense
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _rng_problem(nx, ny, nz, seed=1, **kw):
    rng = np.random.default_rng(seed)
    N = nx * ny * nz
    base = dict(nx=nx, ny=ny, nz=nz, lx=nx * 1e-9, ly=ny * 1.3e-9, lz=nz * 0.8e-9,
                kappa=rng.choice([149.0, 0.2, 50.0], size=N), rho=rng.uniform(1000, 3000, N),
                heat_capacity=rng.uniform(500, 1500, N), tau=1e-12, em=0.0,
                time_step=1e-13, icattaneo=1, kappa_bound=(149.0, 20.0, 149.0, 0.2, 60.0, 149.0),
                t_bath_face=(300.0, 310.0, 295.0, 300.0, 305.0, 290.0), t_bath=300.0, br=0.7)
    base.update(kw)
    return Problem(**base)


def _cases():
    c = {}
    c["cube6"] = point_source_cube(6)
    c["layered"] = layered_slab(8, nz=10, layer=3)
    c["br_mixed"] = _rng_problem(5, 4, 6)
    c["periodic_xy"] = _rng_problem(5, 4, 3, periodic=(1, 1, 0))
    c["periodic_all_n2"] = _rng_problem(2, 2, 2, periodic=(1, 1, 1))
    c["periodic_z2"] = _rng_problem(3, 3, 2, periodic=(0, 0, 1))
    c["flat"] = _rng_problem(7, 5, 1)
    c["line"] = _rng_problem(6, 1, 1)
    c["single"] = _rng_problem(1, 1, 1)
    c["neumann"] = _rng_problem(4, 5, 3, cg_face=(1, 0, 0, 0, 0, 1), t_bath_cg=2.0)
    c["steady"] = _rng_problem(3, 3, 3, isteady=1, iheater=np.r_[np.zeros(13), 1, np.zeros(13)].astype(np.int64),
                               power_in=1e-6)
    c["fourier"] = _rng_problem(4, 3, 5, icattaneo=0)
    return c


CASES = _cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_operator_bit_exact(cuda_lib, name):
    prob = CASES[name]
    ref = Oracle(prob).dense()
    with HeatFlow(prob) as hf:
        H = geometric_to_dense(prob, hf.operator())
    assert np.array_equal(H, ref), np.abs(H - ref).max()


@pytest.mark.parametrize("name", sorted(CASES))
def test_coo_assembly_bit_exact(cuda_lib, name):
    prob = CASES[name]
    ri, rj, rv, rc = Oracle(prob).coo()
    with HeatFlow(prob) as hf:
        gi, gj, gv, gc = hf.sparse_hmatrix()
    assert gc == rc
    assert np.array_equal(gi, ri) and np.array_equal(gj, rj) and np.array_equal(gv, rv)


@pytest.mark.parametrize("name", sorted(CASES))
def test_atimes_srsax_order(cuda_lib, name):
    prob = CASES[name]
    x = np.random.default_rng(3).uniform(250, 350, prob.ncells)
    ref = Oracle(prob).atimes(x)
    with HeatFlow(prob) as hf:
        y = hf.atimes(x)
    assert np.array_equal(y, ref), np.abs(y - ref).max()


def _heater_problem(em=0.3):
    n = 4
    N = n ** 3
    ih = np.arange(N, dtype=np.int64) % 9 - 1          # cases -1..7
    return _rng_problem(n, n, n, iheater=ih, power_in=2e-6, freq=3.0e11, heated_steps=2,
                        em=em, t_bath=280.0)


@pytest.mark.parametrize("itime", [1, 2, 3, 7])
@pytest.mark.parametrize("em", [0.0, 0.3])
def test_rhs_pieces(cuda_lib, itime, em):
    prob = _heater_problem(em)
    rng = np.random.default_rng(itime)
    tp = rng.uniform(290, 320, prob.ncells)
    tpp = tp + rng.uniform(-1, 1, prob.ncells)
    o = Oracle(prob)
    o.set_state(tp, tpp)
    rc, ref = o.rhs(itime)
    assert rc == 0
    with HeatFlow(prob) as hf:
        hf.set_state(tp, tpp)
        got = hf.rhs(itime)
    assert np.array_equal(got["B"], ref["B"])
    assert np.array_equal(got["S_cat"], ref["S_cat"])
    assert np.array_equal(got["x0"], ref["x0"])
    ih = prob.iheater
    exact = np.isin(ih, [-1, 0, 1, 2, 6, 7]) if em == 0.0 else np.zeros(prob.ncells, bool)
    for key in ("Q", "Qdens", "S"):
        assert np.array_equal(got[key][exact], ref[key][exact]), key
        np.testing.assert_allclose(got[key], ref[key], rtol=1e-14, atol=0, err_msg=key)


def test_golden_tempdis_gpu(cuda_lib, golden):
    """The reference's test deck, 10 steps, FP64 path with the reference's stopping rule."""
    param, prob = inputs.read_all_files(golden["param_in"], golden["mat_in"], golden["system_in"])
    with HeatFlow(prob, precision="fp64", criterion="recursive", tol=1e-32) as hf:
        hf.initial_evolve()
        st = hf.run(1, param["ntime"])
        T, _ = hf.get_state()
    gold = np.asarray(golden["tempdis"])
    assert np.linalg.norm(T - gold) / np.linalg.norm(gold) < 1.1e-9
    o = Oracle(prob)
    o.set_state(*prob.initial_state())
    o.run(param["ntime"])
    Tref, _ = o.get_state()
    assert np.linalg.norm(T - Tref) / np.linalg.norm(Tref) < 1e-12
    assert st["steps"] == 10 and st["unconverged"] == 0


def _oracle_run(prob, nsteps, mode=0, tol=1e-32):
    o = Oracle(prob)
    o.set_state(*prob.initial_state())
    rc, iters = o.run(nsteps, mode=mode, tol=tol)
    assert rc == 0
    return o.get_state()[0], iters


def test_config1_fp64_reference_rule(cuda_lib):
    """20^3 Cattaneo point source, 100 steps: FP64 path with the reference's BiCG rule (tol
    1e-32 on the recursive residual) against the oracle's BiCG, 1e-10 relative L2."""
    prob = point_source_cube(20)
    Tref, iters = _oracle_run(prob, 100)
    with HeatFlow(prob, precision="fp64", criterion="recursive", tol=1e-32) as hf:
        hf.initial_evolve()
        st = hf.run(1, 100)
        T, _ = hf.get_state()
    assert np.linalg.norm(T - Tref) / np.linalg.norm(Tref) < 1e-10
    assert st["unconverged"] == 0


@pytest.mark.parametrize("precision,tol_err", [("fp64", 1e-10), ("mixed", 1e-9)])
def test_config1_true_residual(cuda_lib, precision, tol_err):
    prob = point_source_cube(20)
    Tref, _ = _oracle_run(prob, 30)
    with HeatFlow(prob, precision=precision, criterion="true", tol=1e-10) as hf:
        hf.initial_evolve()
        for k in range(1, 31):
            st = hf.simulate(k)
            assert st["last_true_relres"] <= 1e-10
            assert st["unconverged"] == 0
        T, _ = hf.get_state()
    assert np.linalg.norm(T - Tref) / np.linalg.norm(Tref) < tol_err


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_layered_slab_vs_oracle(cuda_lib, precision):
    prob = layered_slab(24, layer=4, sigma=3.0)
    Tref, _ = _oracle_run(prob, 20, mode=1, tol=1e-13)
    with HeatFlow(prob, precision=precision, criterion="true", tol=1e-10 if precision == "mixed" else 1e-13) as hf:
        hf.initial_evolve()
        st = hf.run(1, 20)
        T, _ = hf.get_state()
    err = np.linalg.norm(T - Tref) / np.linalg.norm(Tref)
    assert err < (1e-9 if precision == "mixed" else 1e-12), err
    assert st["last_true_relres"] <= (1e-10 if precision == "mixed" else 1e-13)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("g", [0, 1])
def test_batch_equals_single(cuda_lib, precision, g):
    """A batch of uneven grids (host loop or one persistent launch per step) gives each grid's
    own single-grid result bit for bit."""
    rng = np.random.default_rng(5)
    probs = [random_instance(rng, lo=5, hi=12) for _ in range(4)]
    kw = dict(precision=precision, criterion="true", tol=1e-10)
    with HeatFlow(probs, use_graph=g, **kw) as hf:
        hf.initial_evolve()
        hf.run(1, 6)
        Tb, _ = hf.get_state()
    parts = []
    for p in probs:
        with HeatFlow(p, **kw) as hf:
            hf.initial_evolve()
            hf.run(1, 6)
            parts.append(hf.get_state()[0])
    assert np.array_equal(Tb, np.concatenate(parts))


def test_nan_in_boundary_vector(cuda_lib):
    prob = point_source_cube(4)
    prob.kappa = prob.kappa.copy()
    prob.kappa[0] = np.nan            # a corner cell: its boundary faces become NaN
    with HeatFlow(prob) as hf:
        hf.initial_evolve()
        with pytest.raises(abi.HeatFlowError) as e:
            hf.simulate(1)
        assert e.value.code == abi.HF_ENAN_B
        assert "NAN in B vector" in str(e.value)


@pytest.mark.parametrize("icattaneo,code", [(1, abi.HF_ENAN_SCAT), (0, abi.HF_ENAN_S)])
def test_nan_in_state(cuda_lib, icattaneo, code):
    prob = point_source_cube(4, icattaneo=icattaneo)
    tp, tpp = prob.initial_state()
    tp[5] = np.nan
    with HeatFlow(prob) as hf:
        hf.set_state(tp, tpp)
        with pytest.raises(abi.HeatFlowError) as e:
            hf.simulate(1)
        assert e.value.code == code
        after, _ = hf.get_state()
    assert np.isnan(after[5])          # the state was not rotated (the reference stops)


def test_reject_nx1_grid(cuda_lib):
    with pytest.raises(abi.HeatFlowError) as e:
        HeatFlow(_rng_problem(1, 3, 3))
    assert e.value.code == abi.HF_EARG


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_full_size_residual_property(cuda_lib, precision):
    """256^3 layered slab (the measured workload), one step: the solution satisfies
    ||S - H T|| / ||S|| <= 1e-10, checked with the independent SRSax-order SpMV."""
    prob = layered_slab(256)
    with HeatFlow(prob, precision=precision, criterion="true", tol=1e-10) as hf:
        hf.initial_evolve()
        S = hf.rhs(1)["S"]
        st = hf.simulate(1)
        T, Tpp = hf.get_state()
        HT = hf.atimes(T)
    assert np.all(Tpp == 300.0)
    rel = np.linalg.norm(S - HT) / np.linalg.norm(S)
    assert rel <= 1e-10, rel
    assert st["last_true_relres"] <= 1e-10
    assert np.isfinite(T).all() and T.max() > 300.0


@pytest.mark.parametrize("opts", [
    dict(precision="fp64", criterion="recursive", tol=1e-32),
    dict(precision="fp64", criterion="true", tol=1e-10),
    dict(precision="mixed", criterion="true", tol=1e-10),
])
def test_graph_equals_host_loop(cuda_lib, opts):
    """Both captured steps -- the persistent cooperative solve kernel (use_graph=1) and the
    conditional WHILE/SWITCH graph (use_graph=2) -- run the same task bodies and reductions as the
    host-driven loop: identical fields and iteration counts on a batch of uneven grids."""
    rng = np.random.default_rng(11)
    probs = [point_source_cube(10)] + [random_instance(rng, lo=6, hi=14) for _ in range(3)]
    out = []
    for g in (0, 1, 2):
        with HeatFlow(probs, use_graph=g, **opts) as hf:
            hf.initial_evolve()
            st = hf.run(1, 8)
            out.append((hf.get_state(), st))
    a, sa = out[0]
    for b, sb in out[1:]:
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        for k in ("iterations", "inner_iterations", "refinements", "unconverged"):
            assert sa[k] == sb[k], k
        assert sb["kernel_launches"] > 0
    assert out[1][1]["kernel_launches"] == 5 * 8          # persistent: 5 kernels per step


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_persistent_full_size_equals_host_loop(cuda_lib, precision):
    """256^3 layered slab, 3 steps: the persistent solve (one cooperative launch per step over
    4096 tasks) gives the host loop's fields bit for bit."""
    prob = layered_slab(256)
    out = []
    for g in (0, 1):
        with HeatFlow(prob, precision=precision, criterion="true", tol=1e-10, use_graph=g) as hf:
            hf.initial_evolve()
            st = hf.run(1, 3)
            out.append((hf.get_state()[0], st))
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1]["inner_iterations"] == out[1][1]["inner_iterations"]
    assert out[1][1]["last_true_relres"] <= 1e-10


@pytest.mark.parametrize("g", [1, 2])
def test_graph_nan_stops(cuda_lib, g):
    prob = point_source_cube(4, icattaneo=0)
    tp, tpp = prob.initial_state()
    tp[3] = np.nan
    with HeatFlow(prob, use_graph=g) as hf:
        hf.set_state(tp, tpp)
        with pytest.raises(abi.HeatFlowError) as e:
            hf.run(1, 3)
        assert e.value.code == abi.HF_ENAN_S


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotune_leaves_state_and_picks_a_candidate(cuda_lib, precision):
    """The autotuner times every candidate from the same state and restores it: the state and the
    step statistics are unchanged, and stepping afterwards equals a context with the same step
    history switched to the chosen options (the stored products H T^n, H T^(n-1) are restored
    with the state)."""
    rng = np.random.default_rng(3)
    probs = [point_source_cube(12), random_instance(rng, lo=8, hi=20)]
    kw = dict(precision=precision, criterion="true", tol=1e-10, use_graph=1)
    with HeatFlow(probs, **kw) as hf:
        hf.initial_evolve()
        hf.run(1, 2)
        before = hf.get_state()
        res = hf.autotune(itime0=3, steps=2)
        assert len(res) == (12 if precision == "mixed" else 4)
        assert sum(r["chosen"] for r in res) == 1 and all(r["ms_per_step"] > 0 for r in res)
        best = next(r for r in res if r["chosen"])
        after = hf.get_state()
        assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
        st = hf.run(3, 3)
        T = hf.get_state()[0]
    with HeatFlow(probs, **kw) as h2:
        h2.initial_evolve()
        h2.run(1, 2)
        h2.set_opts(task_depth=best["task_depth"], inner_tol=best["inner_tol"], **kw)
        st2 = h2.run(3, 3)
        T2 = h2.get_state()[0]
    assert np.array_equal(T, T2)
    assert st["inner_iterations"] == st2["inner_iterations"]


def _vector_cases():
    """Grids whose rows hold a multiple of 4 cells, so every step pass takes its 16-byte vector
    form (RHS, direction update, SpMV, CG update, x update)."""
    c = {}
    c["heaters_em_4"] = _heater_problem(0.3)
    c["heaters_4"] = _heater_problem(0.0)
    c["periodic_xyz_8"] = _rng_problem(8, 4, 6, periodic=(1, 1, 1))
    c["periodic_x_40"] = _rng_problem(40, 3, 4, periodic=(1, 0, 0))
    c["neumann_12"] = _rng_problem(12, 5, 4, cg_face=(1, 0, 0, 1, 0, 1), t_bath_cg=2.0)
    c["steady_8"] = _rng_problem(8, 3, 3, isteady=1,
                                 iheater=np.r_[np.zeros(37), 1, np.zeros(34)].astype(np.int64),
                                 power_in=1e-6)
    c["fourier_16"] = _rng_problem(16, 8, 5, icattaneo=0)
    c["wide_36"] = _rng_problem(36, 9, 17)
    return c


VECTOR_CASES = _vector_cases()


@pytest.mark.parametrize("g", [0, 1])
@pytest.mark.parametrize("name", sorted(VECTOR_CASES))
def test_vector_paths_match_oracle(cuda_lib, name, g):
    """Three FP64 steps (true residual <= 1e-14) on the vector paths against the oracle's
    reference-rule BiCG: the fields agree to 1e-11 relative L2."""
    prob = VECTOR_CASES[name]
    assert prob.nx % 4 == 0
    o = Oracle(prob)
    o.set_state(*prob.initial_state())
    rc, _ = o.run(3, itime0=1, mode=0, tol=1e-32, itmax=50000)
    assert rc == 0
    Tref, Tpref = o.get_state()
    with HeatFlow(prob, precision="fp64", criterion="true", tol=1e-14, use_graph=g) as hf:
        hf.initial_evolve()
        st = hf.run(1, 3)
        T, Tp = hf.get_state()
    err = np.linalg.norm(T - Tref) / np.linalg.norm(Tref)
    assert err <= 1e-11, (name, err, st)
    assert np.linalg.norm(Tp - Tpref) / np.linalg.norm(Tpref) <= 1e-11


def _padded_cases():
    """Grids whose rows are not a multiple of 4 cells: the mixed path's FP32 vectors then carry
    padding cells (rows rounded up to 4), and a row's last quad holds 1, 2 or 3 grid cells, with
    the periodic x wrap taken from a load; several grids are more than one tile wide."""
    c = {}
    c["px_5"] = _rng_problem(5, 4, 3, periodic=(1, 1, 0))         # 4k+1, x and y periodic
    c["px_6"] = _rng_problem(6, 3, 4, periodic=(1, 0, 1))         # 4k+2
    c["px_7"] = _rng_problem(7, 5, 3, periodic=(1, 0, 0))         # 4k+3
    c["px_2"] = _rng_problem(2, 3, 4, periodic=(1, 1, 1))         # both x faces join the same pair
    c["wide_37"] = _rng_problem(37, 9, 6)                         # a second tile of 5 cells
    c["px_wide_35"] = _rng_problem(35, 4, 5, periodic=(1, 0, 0))  # wrap across two tiles
    c["neumann_9"] = _rng_problem(9, 5, 4, cg_face=(1, 0, 0, 1, 0, 1), t_bath_cg=2.0)
    c["heaters_5"] = _rng_problem(5, 5, 5, iheater=np.arange(125, dtype=np.int64) % 9 - 1,
                                  power_in=2e-6, freq=3.0e11, heated_steps=2, em=0.3, t_bath=280.0)
    c["single"] = _rng_problem(1, 1, 1)
    c["px_50"] = _rng_problem(50, 20, 6, periodic=(1, 1, 0))       # wrap across two tiles
    c["rows_20"] = _rng_problem(20, 30, 5)                         # rows of 4k cells, no padding
    return c


PADDED_CASES = _padded_cases()


@pytest.mark.parametrize("name", sorted(PADDED_CASES))
def test_padded_rows_mixed_match_oracle(cuda_lib, name):
    """Five mixed-precision steps to true rel-res <= 1e-10 on grids with padded FP32 rows, host
    loop and persistent solve, against the oracle's FP64 PCG to 1e-13: fields within 1e-9
    relative L2 (the mixed path's tolerance); the two paths give the same bits."""
    prob = PADDED_CASES[name]
    Tref, _ = _oracle_run(prob, 5, mode=1, tol=1e-13)
    fields = []
    for g in (0, 1):
        with HeatFlow(prob, precision="mixed", criterion="true", tol=1e-10, use_graph=g) as hf:
            hf.initial_evolve()
            for k in range(1, 6):
                st = hf.simulate(k)
                assert st["unconverged"] == 0
                assert st["last_true_relres"] <= 1e-10
            fields.append(hf.get_state()[0])
    assert np.array_equal(fields[0], fields[1])
    err = np.linalg.norm(fields[1] - Tref) / np.linalg.norm(Tref)
    assert err < 1e-9, (name, err)
