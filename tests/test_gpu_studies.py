"""The study-level entry points under the reference's names, on the device: the PQ/PV
power-flow object of the reference's plugin interface, the batched time series and the N-1
sweep (p3s_gb300.studies)."""

import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

from oracle import cpu
from oracle.build import build_oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def setup_module(_):
    build_oracle()


def test_pqpv_object_jacobian_and_mismatch_match_the_reference():
    """create_J at the golden point equals the reference's own Jacobian (nr_klu debug_J, the
    same matrix as PQPVPowerflow.create_J: unknowns [dVa(pv, pq); dVm(pq)]) to 1e-10 of its
    largest entry; evaluate_Fx equals the reference's mismatch formula; the reference's Newton
    loop (NewtonPowerflow.py:500-547) driven by the object reaches the oracle's solution."""
    from p3s_gb300.studies import PowerflowObject, PQPVPowerflowGPU

    d = np.load(os.path.join(GOLDEN, "golden_118.npz"))
    n = len(d["Yp"]) - 1
    Y = sp.csr_matrix((d["Yx"], d["Yj"], d["Yp"]), shape=(n, n))
    obj = PQPVPowerflowGPU(Y, d["pq"], d["pv"], np.setdiff1d(np.arange(n), np.r_[d["pv"], d["pq"]]))
    assert isinstance(obj, PowerflowObject) and obj.offset == 0
    Jx, Jp, Jj = obj.create_J(d["V0"])
    m = len(Jp) - 1
    J = sp.csr_matrix((Jx, Jj, Jp), shape=(m, m))
    Jref = sp.csc_matrix((d["Jx"], d["Ji"], d["Jp"]), shape=(m, m))
    assert abs(J - Jref).max() <= 1e-10 * abs(Jref).max()
    assert (np.diff(Jp) > 0).all() and all((np.diff(Jj[Jp[r]:Jp[r + 1]]) > 0).all() for r in range(m))
    V = d["V0"]
    mis = V * np.conj(Y @ V) - d["Sbus"]
    Fref = np.r_[mis[d["pv"]].real, mis[d["pq"]].real, mis[d["pq"]].imag]
    F = obj.evaluate_Fx(d["Sbus"], V)
    assert np.abs(F - Fref).max() <= 1e-12 * max(1.0, np.abs(Fref).max())
    # the reference's own loop over power-flow objects, with this object in it
    voltage = V.copy()
    mismatch = obj.evaluate_Fx(d["Sbus"], voltage)
    for it in range(30):
        if np.linalg.norm(mismatch, np.inf) < 1e-8:
            break
        Jx, Jp, Jj = obj.create_J(voltage)
        dx = -1 * spl.spsolve(sp.csr_matrix((Jx, Jj, Jp)), mismatch)
        voltage = obj.evaluate_Results(dx, voltage)
        mismatch = obj.evaluate_Fx(d["Sbus"], voltage)
    ref = cpu.Solver(d["Yp"], d["Yj"], d["Yx"], d["pv"], d["pq"]).solve_batch(d["Sbus"][:, None], V, tol=1e-12)
    assert np.linalg.norm(mismatch, np.inf) < 1e-8
    assert np.abs(voltage - ref["V"][:, 0]).max() < 1e-8


def test_calculate_timeseries_cpp_from_the_dc_start(grid118):
    from p3s_gb300.cuda.nr_polar_solver import PolarNewtonSolverCUDA
    from p3s_gb300.solver import GpuSolver
    from p3s_gb300.studies import LoadflowNotConverged, calculate_timeseries_cpp
    from p3s_gb300.synthetic import timeseries_injections

    g = grid118
    S = timeseries_injections(g, 24)
    V = calculate_timeseries_cpp(g, S)
    v_dc, used = GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).dc_start(g.Sbus.real, g.V0)
    assert used
    ref = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, v_dc)
    assert ref["converged"].all() and np.abs(V - ref["V"]).max() < 1e-11
    flat = calculate_timeseries_cpp(g, S, init="flat", precision="mixed")
    assert np.abs(flat - ref["V"]).max() < 1e-8
    bad = S.copy()
    bad[3, 5] = np.nan
    with pytest.raises(ValueError, match="NaN or inf"):
        calculate_timeseries_cpp(g, bad)
    with pytest.raises(ValueError, match="zero time steps"):
        calculate_timeseries_cpp(g, S[:, :0])
    with pytest.raises(LoadflowNotConverged, match="did not converge for 24 of 24"):
        calculate_timeseries_cpp(g, S, max_iterations=1, solver=PolarNewtonSolverCUDA(g.Yp, g.Yj, g.Yx, g.pv, g.pq))


def test_solve_contingencies_cuda_matches_the_driver_and_reference(grid118):
    from p3s_gb300 import contingency
    from p3s_gb300.studies import solve_contingencies_cpp, solve_contingencies_cuda

    d = np.load(os.path.join(GOLDEN, "golden_n1_118.npz"))
    g = grid118
    flat = solve_contingencies_cuda(g, reslack_islands=True, init="flat")
    direct = contingency.solve_contingencies(g, reslack_islands=True)
    assert np.array_equal(flat.served, d["served"]) and np.array_equal(flat.converged, d["cv_strict"])
    assert np.array_equal(np.isnan(flat.V), np.isnan(direct.V)) and np.array_equal(flat.iterations, direct.iterations)
    assert np.nanmax(np.abs(flat.V - direct.V)) == 0.0
    dc = solve_contingencies_cpp(g, reslack_islands=True, n_threads=4)
    assert np.array_equal(dc.served, d["served"]) and dc.converged[d["cv_strict"]].all()
    with pytest.raises(ValueError, match="init must be"):
        solve_contingencies_cuda(g, init="warm")
    with pytest.raises(ValueError, match="backend must be 'lean'"):
        solve_contingencies_cuda(g, backend="cudss")
