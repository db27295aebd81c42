"""Temperature-dependent properties (tabulated kappa, rho, c re-evaluated after every step, the
operator rebuilt): the oracle's restatement and the GPU paths agree."""
import numpy as np
import pytest

from heatflow_gb300.problem import Problem


def table_a():
    # a conductor whose kappa falls and whose heat capacity rises with temperature
    T = np.array([250.0, 290.0, 300.0, 305.0, 320.0, 400.0])
    return np.c_[T, 150.0 - 0.6 * (T - 250.0), 2300.0 - 0.1 * (T - 250.0), 700.0 + 0.8 * (T - 250.0)]


def table_b():
    return np.array([[290.0, 0.3, 1200.0, 1100.0], [330.0, 0.2, 1150.0, 1300.0]])


def tempdep_problem():
    nx, ny, nz = 12, 10, 8
    N = nx * ny * nz
    rng = np.random.default_rng(2)
    ih = np.zeros(N, np.int64)
    ih[rng.choice(N, 4, replace=False)] = 1
    power = np.where(ih > 0, 3e-6, 0.0)
    prob = Problem(nx=nx, ny=ny, nz=nz, lx=nx * 1e-9, ly=ny * 1e-9, lz=nz * 1e-9, kappa=149.0,
                   rho=2329.0, heat_capacity=710.0, tau=1e-12, em=0.0, iheater=ih, power=power,
                   time_step=1e-13, icattaneo=1, qdens_mode=1, kappa_bound=(149.0,) * 6,
                   t_bath_face=(300.0,) * 6, t_bath=300.0)
    iz = np.repeat(np.arange(nz), nx * ny)
    cell_table = np.where(iz < 3, 1, 0).astype(np.int32)
    cell_table[iz == nz - 1] = -1                           # a layer with fixed properties
    return prob, [table_a(), table_b()], cell_table


def test_oracle_tables_change_the_run():
    from oracle.oracle import Oracle
    prob, tables, ct = tempdep_problem()
    out = []
    for with_tables in (False, True):
        o = Oracle(prob)
        if with_tables:
            o.set_property_tables(tables, ct)
        o.set_state(*prob.initial_state())
        rc, _ = o.run(5, itime0=1, mode=0, tol=1e-32, itmax=50000)
        assert rc == 0
        out.append(o.get_state()[0])
    assert np.isfinite(out[1]).all()
    assert np.linalg.norm(out[1] - out[0]) / np.linalg.norm(out[0] - 300.0) > 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [0, 1, 2])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tables_match_oracle(cuda_lib, precision, use_graph):
    """8 steps with the properties re-evaluated after each: the operator after the run equals the
    oracle's bit for bit, and the fields agree to 1e-10 (FP64) / 1e-9 (mixed) relative L2."""
    from oracle.oracle import Oracle
    from heatflow_gb300.solver import HeatFlow, geometric_to_dense
    prob, tables, ct = tempdep_problem()
    o = Oracle(prob)
    o.set_property_tables(tables, ct)
    o.set_state(*prob.initial_state())
    rc, _ = o.run(8, itime0=1, mode=0, tol=1e-32, itmax=50000)
    assert rc == 0
    Tref, _ = o.get_state()
    tol = 1e-13 if precision == "fp64" else 1e-10
    with HeatFlow(prob, precision=precision, criterion="true", tol=tol, use_graph=use_graph) as hf:
        hf.set_property_tables(tables, ct)
        hf.initial_evolve()
        st = hf.run(1, 8)
        T, _ = hf.get_state()
        H = geometric_to_dense(prob, hf.operator())
    err = np.linalg.norm(T - Tref) / np.linalg.norm(Tref)
    assert err <= (1e-10 if precision == "fp64" else 1e-9), err
    assert st["unconverged"] == 0
    # the rebuilt operator is exactly the one of the properties at the GPU's final field
    kappa, rho, hc = prob.kappa.copy(), prob.rho.copy(), prob.heat_capacity.copy()
    for i in np.nonzero(ct >= 0)[0]:
        rows = tables[ct[i]]
        kappa[i], rho[i], hc[i] = (table_value(rows, c, T[i]) for c in (1, 2, 3))
    import dataclasses
    ref_prob = dataclasses.replace(prob, kappa=kappa, rho=rho, heat_capacity=hc, _keep=[])
    assert np.array_equal(H, Oracle(ref_prob).dense())


def table_value(rows, col, T):
    """The tables' rule (held constant outside, linear inside), in the kernels' operation order."""
    m = len(rows)
    if T <= rows[0, 0]:
        return rows[0, col]
    if T >= rows[m - 1, 0]:
        return rows[m - 1, col]
    k = 0
    while k + 1 < m - 1 and not (T < rows[k + 1, 0]):
        k += 1
    f = (T - rows[k, 0]) / (rows[k + 1, 0] - rows[k, 0])
    return rows[k, col] + f * (rows[k + 1, col] - rows[k, col])


def periodic_problem(nx, ny, nz, periodic):
    N = nx * ny * nz
    rng = np.random.default_rng(nx * 100 + ny * 10 + nz)
    ih = np.zeros(N, np.int64)
    ih[rng.choice(N, max(1, N // 20), replace=False)] = 1
    power = np.where(ih > 0, 3e-6, 0.0)
    prob = Problem(nx=nx, ny=ny, nz=nz, lx=nx * 1e-9, ly=ny * 1e-9, lz=nz * 1e-9, kappa=149.0,
                   rho=2329.0, heat_capacity=710.0, tau=1e-12, em=0.0, iheater=ih, power=power,
                   time_step=1e-13, icattaneo=1, qdens_mode=1, kappa_bound=(149.0,) * 6,
                   t_bath_face=(300.0,) * 6, t_bath=300.0, periodic=periodic)
    cell_table = (rng.random(N) < 0.5).astype(np.int32)
    cell_table[rng.random(N) < 0.1] = -1
    return prob, [table_a(), table_b()], cell_table


@pytest.mark.gpu
@pytest.mark.parametrize("dims,periodic", [
    ((12, 10, 8), (0, 0, 0)),
    ((8, 6, 4), (1, 1, 1)),
    ((2, 5, 3), (1, 0, 0)),      # nx = 2: both x faces of a cell join the same neighbour
    ((6, 2, 4), (0, 1, 0)),      # ny = 2 periodic
    ((4, 3, 2), (0, 0, 1)),      # nz = 2 periodic
    ((5, 4, 1), (1, 1, 0)),      # one layer, odd nx (scalar passes)
])
def test_step_rebuild_equals_setup_assembly(cuda_lib, dims, periodic):
    """The operator rebuilt inside the step (one conductivity evaluation per face orientation)
    equals, bit for bit, the set-up assembly's (hmatrixfunc per stored slot) and the oracle's
    dense H for the same properties, on periodic axes, two-cell axes and one-cell axes."""
    from oracle.oracle import Oracle
    from heatflow_gb300.solver import HeatFlow, geometric_to_dense
    import dataclasses
    prob, tables, ct = periodic_problem(*dims, periodic)
    with HeatFlow(prob, precision="fp64", criterion="true", tol=1e-13, use_graph=1) as hf:
        hf.set_property_tables(tables, ct)
        hf.initial_evolve()
        hf.run(1, 3)
        T, _ = hf.get_state()
        op = hf.operator()
    kappa, rho, hc = prob.kappa.copy(), prob.rho.copy(), prob.heat_capacity.copy()
    for i in np.nonzero(ct >= 0)[0]:
        rows = tables[ct[i]]
        kappa[i], rho[i], hc[i] = (table_value(rows, c, T[i]) for c in (1, 2, 3))
    assert len(np.unique(kappa)) > 2                     # the properties really vary cell to cell
    ref_prob = dataclasses.replace(prob, kappa=kappa, rho=rho, heat_capacity=hc, _keep=[])
    with HeatFlow(ref_prob, precision="fp64", criterion="true", tol=1e-13, use_graph=0) as hf0:
        op0 = hf0.operator()
    for key in ("diag", "cx", "cy", "cz"):
        assert np.array_equal(op[key], op0[key]), key
    assert np.array_equal(geometric_to_dense(prob, op), Oracle(ref_prob).dense())


def test_oracle_one_cell_periodic_axis_has_zero_diagonal():
    """A periodic axis one cell long: hmatrixfunc's wrap rule for that axis (offset (n-1)*stride = 0)
    overwrites the diagonal with the self-face term, 0, so the set-up's check that H_II < 0 rejects
    such a grid; the oracle shows the zero diagonal the check is guarding against."""
    from oracle.oracle import Oracle
    prob, _, _ = periodic_problem(6, 1, 4, (0, 1, 0))
    assert np.all(np.diag(Oracle(prob).dense()) == 0.0)


# ---- the reference's table format and per-material lookup (mod_tempdep.f90:44-55) ---------------
def _reference_table_text():
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "tempdep_table.json")) as f:
        return json.load(f)["text"]


def _tempdep_deck(golden, d, with_table=True):
    """The reference's test deck with TempDepProp = 1 and, for its material 1, the reference's
    table test/data/tempdep.in as ./inputs/MatTable1."""
    d.mkdir(parents=True, exist_ok=True)
    param = golden["param_in"].replace("TempDepProp = 0", "TempDepProp = 1")
    assert "TempDepProp = 1" in param
    (d / "param.in").write_text(param)
    (d / "mat.in").write_text(golden["mat_in"])
    (d / "system.in").write_text(golden["system_in"])
    if with_table:
        (d / "MatTable1").write_text(_reference_table_text())
    return param


def test_reference_table_parses():
    from heatflow_gb300.inputs import parse_property_table
    text = _reference_table_text()
    rows = parse_property_table(text)
    assert rows.shape == (24, 4)
    assert np.all(np.diff(rows[:, 0]) > 0)
    want = np.array([[float(v) for v in line.split()] for line in text.splitlines() if line.split()])
    assert np.array_equal(rows, want)


@pytest.mark.parametrize("bad", ["300 1 2\n", "300 1 2 3\n290 1 2 3\n", "300 1 2 3\n"])
def test_bad_tables_refused(bad):
    from heatflow_gb300.inputs import InputError, parse_property_table
    with pytest.raises(InputError):
        parse_property_table(bad)


def test_host_program_reads_material_tables(golden, tmp_path):
    """The C++ host program and the Python readers find the same MatTable<imaterial> files and
    read the same rows (--dump-problem stops before any GPU call)."""
    import json
    import subprocess
    from heatflow_gb300 import inputs
    from heatflow_gb300.build import build_driver, build_library
    build_library()
    drv = build_driver()
    d = tmp_path / "inputs"
    _tempdep_deck(golden, d)
    r = subprocess.run([drv, "--inputs", str(d), "--dump-problem"], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    js = json.loads(next(l for l in r.stdout.splitlines() if l.startswith("{")))
    assert js["temp_dep_prop"] == 1
    sysd = inputs.read_system(golden["system_in"])
    tables, ct = inputs.material_tables(str(d), sysd.imaterial)
    pt = js["property_tables"]
    assert pt["materials"] == [1] and pt["offsets"] == [0, 24]
    assert np.array_equal(np.asarray(pt["rows"]).reshape(-1, 4), tables[0])
    assert np.array_equal(np.asarray(pt["cell_table"]), ct) and np.all(ct == 0)
    # without a MatTable file the material keeps fixed properties (the reference's `continue`)
    (d / "MatTable1").unlink()
    r = subprocess.run([drv, "--inputs", str(d), "--dump-problem"], capture_output=True, text=True,
                       timeout=60)
    js = json.loads(next(l for l in r.stdout.splitlines() if l.startswith("{")))
    assert "property_tables" not in js
    assert inputs.material_tables(str(d), sysd.imaterial)[0] == []
    # a malformed table stops the program with a message, as input errors do
    (d / "MatTable1").write_text("300 1 2\n")
    r = subprocess.run([drv, "--inputs", str(d), "--dump-problem"], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 1 and "MatTable1" in r.stdout


@pytest.mark.gpu
def test_reference_table_deck_on_gpu(cuda_lib, golden, tmp_path):
    """The reference's test deck with TempDepProp = 1 and its table file: the C++ host program
    runs it end to end; its TempDis.dat equals the Python path's (same library) byte for byte,
    and that field is within 1e-10 of the oracle run with the same tables."""
    import subprocess
    from oracle.oracle import Oracle
    from heatflow_gb300 import inputs
    from heatflow_gb300.build import build_driver, build_library
    from heatflow_gb300.solver import HeatFlow
    build_library()
    drv = build_driver()
    work = tmp_path / "run"
    param_text = _tempdep_deck(golden, work / "inputs")
    r = subprocess.run([drv], cwd=work, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    param, prob = inputs.read_all_files(param_text, golden["mat_in"], golden["system_in"])
    sysd = inputs.read_system(golden["system_in"])
    tables, ct = inputs.material_tables(str(work / "inputs"), sysd.imaterial)
    nt = param["ntime"]
    o = Oracle(prob)
    o.set_property_tables(tables, ct)
    o.set_state(*prob.initial_state())
    rc, _ = o.run(nt, itime0=1, mode=0, tol=1e-32, itmax=50000)
    assert rc == 0
    Tref, _ = o.get_state()
    o0 = Oracle(prob)                                    # the same deck without the table
    o0.set_state(*prob.initial_state())
    o0.run(nt, itime0=1, mode=0, tol=1e-32, itmax=50000)
    assert np.linalg.norm(o0.get_state()[0] - Tref) / np.linalg.norm(Tref) > 1e-6
    with HeatFlow(prob, precision="fp64", criterion="recursive", tol=1e-32) as hf:
        hf.set_property_tables(tables, ct)
        hf.initial_evolve()
        for k in range(1, nt + 1):
            hf.run(k, 1)
        Tp, Tpp = hf.get_state()
    assert np.linalg.norm(Tp - Tref) / np.linalg.norm(Tref) <= 1e-10
    assert (work / "outputs" / "TempDis.dat").read_text() == inputs.format_temp_file(Tp)
    assert (work / "outputs" / "TempDisTPD.dat").read_text() == inputs.format_temp_file(Tpp)
