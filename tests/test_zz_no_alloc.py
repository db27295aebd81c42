"""hf_residual_noalloc: the residual r = b - H x and its norms for callers that cannot allocate
device memory (hosts that give the library only pre-allocated buffers, loops that may not stall
on the allocator).  The entry point keeps its
reduction scratch in a static device array; this test checks it against the library's
allocating SpMV (hf_apply_operator, the reference's SRSax order) and against the oracle's COO
product (SRSax, mod_Sparse.f90:293-315) on two calls in a row, on grids with periodic axes of
length 2, and that grids above the static limit - also those whose cell count would overflow -
are refused.  Collected last so that a failure here does not hide the other tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(periodic, dims=(37, 20, 11)):
    from heatflow_gb300.problem import Problem
    rng = np.random.default_rng(7)
    nx, ny, nz = dims
    N = nx * ny * nz
    return Problem(nx=nx, ny=ny, nz=nz, lx=nx * 1e-9, ly=ny * 1e-9, lz=nz * 1e-9,
                   kappa=rng.choice([149.0, 0.2, 50.0], size=N), rho=rng.uniform(1000, 3000, N),
                   heat_capacity=1000.0, tau=1e-12, time_step=1e-13, icattaneo=1,
                   periodic=periodic, kappa_bound=(149.0,) * 6, t_bath_face=(300.0,) * 6,
                   t_bath=300.0)


@pytest.mark.parametrize("periodic,dims", [((0, 0, 0), (37, 20, 11)), ((1, 1, 0), (37, 20, 11)),
                                          ((1, 1, 1), (2, 9, 2)), ((0, 1, 1), (5, 2, 3))])
def test_residual_noalloc_matches_allocating_path(cuda_lib, periodic, dims):
    import torch
    from heatflow_gb300 import abi
    from heatflow_gb300.solver import HeatFlow
    from oracle.oracle import Oracle

    prob = _problem(periodic, dims)
    rng = np.random.default_rng(11)
    x = rng.uniform(290.0, 310.0, prob.ncells)
    b = rng.uniform(-6e21, -4e21, prob.ncells)
    with HeatFlow(prob) as hf:
        op = hf.operator()
        ref = b - hf.atimes(x)
    # the oracle's COO product in the reference's order: the same bits as the library's
    ref_oracle = b - Oracle(prob).atimes(x)
    assert np.array_equal(ref, ref_oracle)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
    ops = [dev(op[k]) for k in ("diag", "cx", "cy", "cz")]
    xd, bd = dev(x), dev(b)
    r = torch.empty_like(xd)
    norms = torch.empty(2, dtype=torch.float64, device="cuda")
    per = (C.c_int32 * 3)(*periodic)
    lib = abi.load_library()
    for _ in range(2):                       # the static scratch keeps the previous call's data
        r.fill_(float("nan"))
        norms.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = lib.hf_residual_noalloc(prob.nx, prob.ny, prob.nz, per,
                                     *[C.c_void_p(t.data_ptr()) for t in ops],
                                     C.c_void_p(bd.data_ptr()), C.c_void_p(xd.data_ptr()),
                                     C.c_void_p(r.data_ptr()), C.c_void_p(norms.data_ptr()), None)
        assert rc == abi.HF_OK, lib.hf_last_error()
        torch.cuda.synchronize()
        got = r.cpu().numpy()
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
        nr = norms.cpu().numpy()
        np.testing.assert_allclose(nr, [np.dot(ref, ref), np.dot(b, b)], rtol=1e-12)


def test_residual_noalloc_refuses_grids_above_limit(cuda_lib):
    from heatflow_gb300 import abi
    lib = abi.load_library()
    per = (C.c_int32 * 3)(0, 0, 0)
    fake = C.c_void_p(16)                    # never dereferenced: the size check comes first
    for dims in ((257, 256, 256), (3, 2 ** 62, 3), (2 ** 40, 2 ** 40, 1), (1, 1, 2 ** 25),
                 (16777217, 1, 1)):
        rc = lib.hf_residual_noalloc(*dims, per, fake, fake, fake, fake, fake, fake, fake, fake,
                                     None)
        assert rc == abi.HF_EARG, dims
        assert b"HF_NOALLOC_MAX_CELLS" in lib.hf_last_error()
