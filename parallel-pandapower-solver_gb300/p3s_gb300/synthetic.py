"""Seeded synthetic power-flow grids and injection series.

The reference benchmarks on pandapower/IEEE grids, which are not available here; these
generators produce grids with the same shape of data the reference's solver entry points
consume (``nr_klu.Solver(Yp, Yj, Yx, pv, pq)``, ``solve_batch(Sbus (n,T), V0)``):

* buses uniform in the unit square, a Euclidean minimum spanning tree plus the shortest
  non-tree chords;
* pi-model branches: ``x = 0.02 + 0.3 * length``, ``r = x * U(0.1, 0.4)``, total
  charging ``b ~ U(0, 0.05)``; a share of the branches are transformers with an
  off-nominal tap ``t ~ U(0.95, 1.05)``;
* one slack (Vm 1.04), PV buses (Vm ``U(0.98, 1.05)``, P ``U(0.2, 2.0)``), PQ loads
  (P ``U(0, 0.6)``, Q = P * ``U(0.1, 0.5)``); generation scaled to 1.03 x load.

Branch stamp (standard pi model, the same convention as the reference's
``p3s/models/TwoPort.py:133-167`` and ``TransmissionLineModel.py:32-49`` for tap 1)::

    Y_ff = (y + j b/2) / t^2,  Y_ft = Y_tf = -y / t,  Y_tt = y + j b/2

stamped at rows ``[f, f, t, t]`` / cols ``[f, t, f, t]`` and summed by scipy's COO->CSR
conversion with sorted column indices (``TwoPort.py:148-151``).
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
from scipy.sparse.csgraph import minimum_spanning_tree
from scipy.spatial import cKDTree


@dataclass
class Grid:
    """One synthetic grid in the array form the reference's solvers take."""

    n: int
    Yp: np.ndarray  # (n+1,) int32 CSR indptr
    Yj: np.ndarray  # (nnz,) int32 CSR indices, sorted per row
    Yx: np.ndarray  # (nnz,) complex128
    pv: np.ndarray  # (npv,) int32
    pq: np.ndarray  # (npq,) int32
    ref: np.ndarray  # (1,) int32 slack bus
    Sbus: np.ndarray  # (n,) complex128 base-case injections (gen - load)
    V0: np.ndarray  # (n,) complex128 flat start carrying the voltage set-points
    # branch table
    f: np.ndarray  # (nbr,) int32 from bus
    t: np.ndarray  # (nbr,) int32 to bus
    stamp: np.ndarray  # (nbr, 4) complex128  Y_ff, Y_ft, Y_tf, Y_tt
    stamp_pos: np.ndarray  # (nbr, 4) int32 CSR data positions of (f,f), (f,t), (t,f), (t,t)
    # injections split for time series
    p_load: np.ndarray = field(default=None)  # (n,) load P at PQ buses
    q_load: np.ndarray = field(default=None)  # (n,) load Q at PQ buses
    p_gen: np.ndarray = field(default=None)  # (n,) scheduled generation at PV buses
    vm_set: np.ndarray = field(default=None)  # (n,) voltage set-point (slack/PV), 1 elsewhere
    loading: float = 1.0  # factor applied to the nominal per-unit injections (see make_grid)

    @property
    def nnz(self) -> int:
        return int(self.Yj.shape[0])

    @property
    def n_branch(self) -> int:
        return int(self.f.shape[0])


def _candidate_edges(xy: np.ndarray, k: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Undirected k-nearest-neighbour edges (u < v) with their Euclidean lengths."""
    n = xy.shape[0]
    kk = min(k + 1, n)
    tree = cKDTree(xy)
    dist, idx = tree.query(xy, k=kk)
    u = np.repeat(np.arange(n), kk - 1)
    v = idx[:, 1:].ravel()
    a = np.minimum(u, v)
    b = np.maximum(u, v)
    key = np.unique(a.astype(np.int64) * n + b)
    a = (key // n).astype(np.int64)
    b = (key % n).astype(np.int64)
    length = np.linalg.norm(xy[a] - xy[b], axis=1)
    return a, b, length


def _mst_and_chords(xy: np.ndarray, n_branches: int, rng) -> tuple[np.ndarray, np.ndarray]:
    """Euclidean MST plus the ``n_branches - (n-1)`` shortest non-tree chords.

    The MST is computed on the k-nearest-neighbour graph (grown until it is connected
    and holds enough chords); the Euclidean MST and the shortest chords of a random
    point set are short edges, which that graph contains.
    """
    n = xy.shape[0]
    n_chords = n_branches - (n - 1)
    if n_chords < 0:
        raise ValueError("n_branches must be >= n - 1")
    k = 10
    while True:
        a, b, length = _candidate_edges(xy, k)
        G = sp.coo_matrix((length, (a, b)), shape=(n, n)).tocsr()
        ncomp, _ = sp.csgraph.connected_components(G, directed=False)
        if ncomp == 1 and len(a) - (n - 1) >= n_chords:
            break
        if k >= n - 1:
            raise ValueError("cannot build a connected grid")
        k = min(2 * k, n - 1)
    T = minimum_spanning_tree(G).tocoo()
    ta = np.minimum(T.row, T.col).astype(np.int64)
    tb = np.maximum(T.row, T.col).astype(np.int64)
    in_tree = np.zeros(len(a), dtype=bool)
    key = a * n + b
    tkey = np.sort(ta * n + tb)
    in_tree[np.isin(key, tkey)] = True
    cand = np.nonzero(~in_tree)[0]
    order = np.lexsort((key[cand], length[cand]))
    chords = cand[order[:n_chords]]
    f = np.concatenate([ta, a[chords]])
    t = np.concatenate([tb, b[chords]])
    return f.astype(np.int32), t.astype(np.int32)


def build_ybus(n: int, f: np.ndarray, t: np.ndarray, stamp: np.ndarray):
    """CSR Ybus (sorted indices, duplicates summed) and each branch's 4 CSR positions."""
    rows = np.stack([f, f, t, t], axis=1).ravel()
    cols = np.stack([f, t, f, t], axis=1).ravel()
    vals = stamp.ravel()
    # every bus gets a structural diagonal (also isolated ones)
    rows = np.concatenate([rows, np.arange(n)])
    cols = np.concatenate([cols, np.arange(n)])
    vals = np.concatenate([vals, np.zeros(n, dtype=np.complex128)])
    Y = sp.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()
    Y.sum_duplicates()
    Y.sort_indices()
    Yp = Y.indptr.astype(np.int32)
    Yj = Y.indices.astype(np.int32)
    Yx = Y.data.astype(np.complex128)
    # CSR position of (r, c): binary search in row r
    def pos(r, c):
        out = np.empty(len(r), dtype=np.int64)
        for i in range(len(r)):
            lo, hi = Yp[r[i]], Yp[r[i] + 1]
            out[i] = lo + np.searchsorted(Yj[lo:hi], c[i])
        return out

    rr = np.stack([f, f, t, t], axis=1).ravel()
    cc = np.stack([f, t, f, t], axis=1).ravel()
    # vectorised search: global key r*n+c is sorted in CSR order
    keys = np.repeat(np.arange(n, dtype=np.int64), np.diff(Yp)) * n + Yj
    stamp_pos = np.searchsorted(keys, rr.astype(np.int64) * n + cc).reshape(-1, 4).astype(np.int32)
    del pos
    return Yp, Yj, Yx, stamp_pos


def _loading_scale(n, Yp, Yj, Yx, slack, P, max_angle_deg) -> float:
    """Largest factor <= 1 keeping the DC power-flow angles of injections ``P`` within
    ``max_angle_deg`` of the slack. B is the susceptance Laplacian of the branches
    (off-diagonal -Im Ybus, diagonal the negated row sum: no shunts), slack removed."""
    import scipy.sparse.linalg as spl

    Y = sp.csr_matrix((Yx, Yj, Yp), shape=(n, n)).tocoo()
    off = Y.row != Y.col
    B = sp.coo_matrix((-Y.data.imag[off], (Y.row[off], Y.col[off])), shape=(n, n)).tocsr()
    B = B - sp.diags(np.asarray(B.sum(axis=1)).ravel())
    keep = np.setdiff1d(np.arange(n), [slack])
    if len(keep) == 0:
        return 1.0
    th = spl.spsolve(B[keep][:, keep].tocsc(), P[keep])
    worst = float(np.degrees(np.abs(th)).max()) if len(th) else 0.0
    if not np.isfinite(worst) or worst <= max_angle_deg:
        return 1.0
    return max_angle_deg / worst


def _voltage_scale(n, Yp, Yj, Yx, fixed, Q, max_drop_pu) -> float:
    """Largest factor <= 1 keeping the decoupled (Q-V) estimate of the voltage drops of
    reactive loads ``Q`` within ``max_drop_pu``: dV = B_pq^-1 Q with the branch susceptance
    Laplacian and the voltage-controlled buses (``fixed``) held."""
    import scipy.sparse.linalg as spl

    Y = sp.csr_matrix((Yx, Yj, Yp), shape=(n, n)).tocoo()
    off = Y.row != Y.col
    B = sp.coo_matrix((-Y.data.imag[off], (Y.row[off], Y.col[off])), shape=(n, n)).tocsr()
    B = B - sp.diags(np.asarray(B.sum(axis=1)).ravel())
    keep = np.setdiff1d(np.arange(n), fixed)
    if len(keep) == 0:
        return 1.0
    dv = spl.spsolve(B[keep][:, keep].tocsc(), Q[keep])
    worst = float(np.abs(dv).max()) if len(dv) else 0.0
    if not np.isfinite(worst) or worst <= max_drop_pu:
        return 1.0
    return max_drop_pu / worst


def make_grid(
    n: int,
    n_branches: int | None = None,
    n_pv: int | None = None,
    n_trafo: int | None = None,
    seed: int = 0,
    gen_scale: float = 1.03,
    max_angle_deg: float = 20.0,
    charging_scale: float | None = None,
    max_drop_pu: float | None = None,
) -> Grid:
    """A synthetic meshed grid (see the module docstring for the recipe)."""
    rng = np.random.default_rng(seed)
    if n_branches is None:
        n_branches = int(round(1.5 * n))
    if n_pv is None:
        n_pv = max(1, int(round(0.1 * n)))
    if n_trafo is None:
        n_trafo = int(round(0.05 * n_branches))
    xy = rng.random((n, 2))
    f, t = _mst_and_chords(xy, n_branches, rng)
    nbr = len(f)
    length = np.linalg.norm(xy[f] - xy[t], axis=1)
    x = 0.02 + 0.3 * length
    r = x * rng.uniform(0.1, 0.4, nbr)
    b = rng.uniform(0.0, 0.05, nbr)
    if charging_scale is None:
        # charging is drawn per branch whatever its length; on grids of more than 2,000
        # buses (branches ever shorter, injections scaled down with the DC angle spread)
        # it is scaled so the total stays that of a 2,000-bus grid -- otherwise the lines'
        # reactive generation swamps the loads and the grid has no AC solution
        charging_scale = min(1.0, 2000.0 / n)
    if charging_scale != 1.0:
        b = b * charging_scale
    tap = np.ones(nbr)
    tr = rng.choice(nbr, size=n_trafo, replace=False) if n_trafo else np.zeros(0, dtype=int)
    tap[tr] = rng.uniform(0.95, 1.05, len(tr))
    if n > 2000:
        # lines get shorter as the unit square fills up, but a transformer's leakage
        # reactance does not: on grids of more than 2,000 buses transformers get at least
        # 0.1 pu, else off-nominal taps on near-zero impedances drive circulating reactive
        # flows of several pu around every mesh and the grid has no AC solution; their
        # off-nominal ratios spread less for the same reason
        x[tr] = np.maximum(x[tr], 0.1)
        tap[tr] = 1.0 + (tap[tr] - 1.0) * (2000.0 / n)
    y = 1.0 / (r + 1j * x)
    ysh = 0.5j * b
    stamp = np.empty((nbr, 4), dtype=np.complex128)
    stamp[:, 0] = (y + ysh) / tap**2
    stamp[:, 1] = -y / tap
    stamp[:, 2] = -y / tap
    stamp[:, 3] = y + ysh
    Yp, Yj, Yx, stamp_pos = build_ybus(n, f, t, stamp)

    # bus types: slack nearest the centre, PV drawn among the rest
    slack = int(np.argmin(np.linalg.norm(xy - 0.5, axis=1)))
    rest = np.setdiff1d(np.arange(n), [slack])
    pv = np.sort(rng.choice(rest, size=n_pv, replace=False)).astype(np.int32)
    is_pv = np.zeros(n, dtype=bool)
    is_pv[pv] = True
    pq = np.nonzero(~is_pv & (np.arange(n) != slack))[0].astype(np.int32)

    vm_set = np.ones(n)
    vm_set[slack] = 1.04
    vm_set[pv] = rng.uniform(0.98, 1.05, n_pv)
    if n > 2000:
        # generator and slack set points lie closer to 1 pu on denser grids: two PV buses a
        # short line apart holding set points 0.07 pu apart exchange reactive power
        # ~ 0.07 / x, which grows without bound as the lines shorten
        vm_set[pv] = 1.0 + (vm_set[pv] - 1.015) * (2000.0 / n)
        vm_set[slack] = 1.0 + (vm_set[slack] - 1.0) * (2000.0 / n)
    p_load = np.zeros(n)
    q_load = np.zeros(n)
    p_load[pq] = rng.uniform(0.0, 0.6, len(pq))
    q_load[pq] = p_load[pq] * rng.uniform(0.1, 0.5, len(pq))
    p_gen = np.zeros(n)
    p_gen[pv] = rng.uniform(0.2, 2.0, n_pv)
    if p_gen.sum() > 0:
        p_gen *= gen_scale * p_load.sum() / p_gen.sum()
    # Loading level. A Euclidean MST plus the SHORTEST chords is meshed only locally: at
    # large scale it stays tree-like, so regional generation/load imbalance has to cross
    # single bridges towards the one slack. At the nominal per-unit levels above that
    # needs DC angle spreads of hundreds of degrees on 2,000-bus grids (no AC solution).
    # All injections are therefore scaled by the largest factor <= 1 whose DC power flow
    # keeps every bus angle within `max_angle_deg` of the slack.
    lam = _loading_scale(n, Yp, Yj, Yx, slack, p_gen - p_load, max_angle_deg)
    if max_drop_pu is not None:
        # optionally also bound the decoupled estimate of the reactive voltage drops (small
        # grids have long lines: the angle bound alone leaves some near voltage collapse)
        lam = min(lam, _voltage_scale(n, Yp, Yj, Yx, np.r_[slack, pv], q_load, max_drop_pu))
    p_load *= lam
    q_load *= lam
    p_gen *= lam
    Sbus = (p_gen - p_load) - 1j * q_load
    V0 = vm_set.astype(np.complex128)
    return Grid(
        n=n,
        Yp=Yp,
        Yj=Yj,
        Yx=Yx,
        pv=pv,
        pq=pq,
        ref=np.array([slack], dtype=np.int32),
        Sbus=Sbus.astype(np.complex128),
        V0=V0,
        f=f,
        t=t,
        stamp=stamp,
        stamp_pos=stamp_pos,
        p_load=p_load,
        q_load=q_load,
        p_gen=p_gen,
        vm_set=vm_set,
        loading=lam,
    )


# ----------------------------------------------------------------------------- configs
def grid_118(seed: int = 0) -> Grid:
    """Meshed 118-bus grid: MST + chords = 186 branches, 9 transformers, 19 PV, 98 PQ."""
    return make_grid(118, n_branches=186, n_pv=19, n_trafo=9, seed=seed)


def grid_2000(seed: int = 0) -> Grid:
    """2,000-bus grid: 3,000 branches (5% transformers), 1 slack, 300 PV, 1,699 PQ."""
    return make_grid(2000, n_branches=3000, n_pv=300, n_trafo=150, seed=seed)


def timeseries_injections(g: Grid, T: int = 8760, seed: int = 1, balanced: bool = True) -> np.ndarray:
    """(n, T) complex injections for an hourly series.

    Load at hour h: ``base * (1 + 0.3 sin(2 pi h / 24)) * LogNormal(0, 0.1)`` (P and Q of a
    bus scaled alike); PV generation: ``base * U(0.5, 1.2)``, then dispatched so that the
    hour's total generation is the grid's generation/load ratio times the hour's total
    load (``balanced=True``): with one slack bus, an unbalanced hour would have to import
    or export tens of per cent of the system load through the slack's few branches, which
    has no AC solution. C order, so a column is one hour (the layout
    ``nr_klu.Solver.solve_batch`` takes).
    """
    rng = np.random.default_rng(seed)
    h = np.arange(T)
    daily = 1.0 + 0.3 * np.sin(2.0 * np.pi * h / 24.0)
    pq = g.pq
    pv = g.pv
    lf = daily[None, :] * rng.lognormal(0.0, 0.1, (len(pq), T))
    gf = rng.uniform(0.5, 1.2, (len(pv), T))
    S = np.zeros((g.n, T), dtype=np.complex128)
    pl = g.p_load[pq, None] * lf
    S[pq, :] = -(pl + 1j * g.q_load[pq, None] * lf)
    pg = g.p_gen[pv, None] * gf
    if balanced and g.p_load.sum() > 0 and len(pv):
        ratio = g.p_gen.sum() / g.p_load.sum()
        pg *= (ratio * pl.sum(axis=0) / pg.sum(axis=0))[None, :]
    S[pv, :] = pg
    return np.ascontiguousarray(S)


def scenario_injections(g: Grid, n_scen: int, seed: int = 2, spread: float = 0.2) -> np.ndarray:
    """(n, n_scen) load scenarios: every load scaled by ``U(1-spread, 1+spread)``."""
    rng = np.random.default_rng(seed)
    S = np.repeat(g.Sbus[:, None], n_scen, axis=1)
    fac = rng.uniform(1.0 - spread, 1.0 + spread, (len(g.pq), n_scen))
    S[g.pq, :] = S[g.pq, :] * fac
    return np.ascontiguousarray(S)


def lanes(T: int, K: int) -> np.ndarray:
    """Split hours ``0..T-1`` into K contiguous warm-start lanes; returns (K+1,) offsets."""
    K = max(1, min(K, T))
    base, extra = divmod(T, K)
    sizes = np.full(K, base, dtype=np.int64)
    sizes[:extra] += 1
    off = np.zeros(K + 1, dtype=np.int64)
    off[1:] = np.cumsum(sizes)
    return off


def multigrid_batch(n_grids: int = 256, n_scen: int = 16, lo: int = 30, hi: int = 20000, seed: int = 7):
    """Uneven multi-grid batch: bus counts log-uniform in [lo, hi], 1.5 n branches, 10% PV."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), n_grids)).astype(int)
    grids = [make_grid(int(s), seed=int(seed * 1000 + i), max_drop_pu=0.05) for i, s in enumerate(sizes)]
    scen = [scenario_injections(g, n_scen, seed=int(seed * 1000 + i + 17)) for i, g in enumerate(grids)]
    return grids, scen
